// Conversion of the caller's SoA field (x fastest) into the GB300 stores:
// interleaved float4 nodes, fp16 bricks with per-brick scales and fp16 cell
// records with per-cell power-of-two scales.
#include "qsl_internal.h"

namespace qsl {

__global__ void k_pack_f4(const float* __restrict__ bx, const float* __restrict__ by, const float* __restrict__ bz,
                          long long n, float4* __restrict__ out) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = make_float4(__ldg(bx + i), __ldg(by + i), __ldg(bz + i), 0.f);
}

cudaError_t launch_pack_f4(const float* bx, const float* by, const float* bz, Dims d, float4* out, cudaStream_t st) {
    const long long n = (long long)d.nx * d.ny * d.nz;
    long long g = (n + 255) / 256;
    if (g > 65535LL * 64) g = 65535LL * 64;
    k_pack_f4<<<(unsigned)g, 256, 0, st>>>(bx, by, bz, n, out);
    return cudaGetLastError();
}

// x-pair records of the packed stretched stores: record o = {node o, node
// o + 1} as two float4 (Bx, By, Bz, 0), o = ix + nx (iy + ny iz); the last node
// of a row pairs with itself (no cell reads that half).  One 32-byte record
// per x corner pair of a trilinear stencil.
__global__ void k_pack_f4x2(const float* __restrict__ bx, const float* __restrict__ by,
                            const float* __restrict__ bz, int nx, long long n, float4* __restrict__ out) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long j = (i % nx == nx - 1) ? i : i + 1;
        out[2 * i] = make_float4(__ldg(bx + i), __ldg(by + i), __ldg(bz + i), 0.f);
        out[2 * i + 1] = make_float4(__ldg(bx + j), __ldg(by + j), __ldg(bz + j), 0.f);
    }
}

cudaError_t launch_pack_f4x2(const float* bx, const float* by, const float* bz, Dims d, float4* out,
                             cudaStream_t st) {
    const long long n = (long long)d.nx * d.ny * d.nz;
    long long g = (n + 255) / 256;
    if (g > 65535LL * 64) g = 65535LL * 64;
    k_pack_f4x2<<<(unsigned)g, 256, 0, st>>>(bx, by, bz, d.nx, n, out);
    return cudaGetLastError();
}

// Search tables of a stretched grid (FieldStretchP::srec / sbin), all three
// axes in one launch: one thread per cell and per bin.
//  * cell j: the reference's search at c = a[j+1] (its comparisons c > a[m]
//    come out the same for every c in (a[j], a[j+1]], and it never compares
//    with a[0], so a coordinate pinned at a[0] gets cell 0's answer too);
//  * bin b: the cells of its edges moved out by 1 % of a bin plus the float
//    rounding of the kernel's bin index ((c - a0) * binv, a few ulp of a
//    value up to nb: 4e-7 nb bins covers it), in double, each the largest
//    j <= n-2 with a[j] below the edge (0 if none).  A coordinate the
//    kernel puts in bin b lies within those edges, so its interval is in the
//    range [lo, hi], on axes of any length.  A range of one or two intervals
//    (every bin unless cells are under ~1/4 of the mean width) is stored as
//    both intervals' records and the node between them, 32 bytes:
//      {a[lo+1] (+inf for one interval), rec(lo).x, .y, .z}
//      {rec(hi).x, .y, .z, 0}
//    so the lookup is two independent loads and a select; a wider range as
//      {0, lo, hi (int bits), 0} {0, 0, 0, 1 (int bits)}
//    for a bisection over [lo, hi] and the cell record.  (The earlier form,
//    an int2 range per bin and always the dependent record load: 8.05-8.11
//    against 7.63-7.66 ms on the search workload; bins holding one record
//    only, with a branch for the others: 10.0 ms, the lanes of a warp
//    diverging between the two cases.)
__device__ __forceinline__ int stretch_cell_below(double c, int n, const float* __restrict__ a) {
    int lo = 0, hi = n - 2;  // largest j in [0, n-2] with a[j] < c, else 0
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if ((double)__ldg(a + mid) < c) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__global__ void k_stretch_tables(const float* __restrict__ ax, const float* __restrict__ ay,
                                 const float* __restrict__ az, Dims d, float4* __restrict__ srec,
                                 float4* __restrict__ sbin) {
    const int cells = (d.nx - 1) + (d.ny - 1) + (d.nz - 1);
    const int bins = STRETCH_BINS_PER_CELL * cells;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < cells + bins; t += gridDim.x * blockDim.x) {
        const bool is_bin = t >= cells;
        const int u = is_bin ? (t - cells) / STRETCH_BINS_PER_CELL : t;  // cell index over the three axes
        const int k = u < d.nx - 1 ? 0 : (u < d.nx + d.ny - 2 ? 1 : 2);
        const float* a = k == 0 ? ax : (k == 1 ? ay : az);
        const int n = d.n(k);
        const int c0 = stretch_cell_offset(d, k);
        if (!is_bin) {
            const int j = u - c0;
            const int i = stretch_bisect(__ldg(a + j + 1), n, a);
            const float ai = __ldg(a + i);
            srec[t] = make_float4(ai, __ldg(a + i + 1) - ai, __int_as_float(i), 0.f);
        } else {
            const int b = t - cells - STRETCH_BINS_PER_CELL * c0;
            const int nb = STRETCH_BINS_PER_CELL * (n - 1);
            const double a0 = __ldg(a), w = ((double)__ldg(a + n - 1) - a0) / nb;
            const double wid = 0.01 + 4e-7 * (double)nb;
            const int lo = stretch_cell_below(a0 + (b - wid) * w, n, a);
            const int hi = stretch_cell_below(a0 + (b + 1 + wid) * w, n, a);
            const int h = hi < lo ? lo : hi;
            float4* out = sbin + 2 * (t - cells);
            if (h <= lo + 1) {
                auto rec_of = [&](int j) {
                    const int i = stretch_bisect(__ldg(a + j + 1), n, a);
                    const float ai = __ldg(a + i);
                    return make_float4(ai, __ldg(a + i + 1) - ai, __int_as_float(i), 0.f);
                };
                const float4 r0 = rec_of(lo), r1 = rec_of(h);
                const float s = h > lo ? __ldg(a + lo + 1) : __int_as_float(0x7f800000);
                out[0] = make_float4(s, r0.x, r0.y, r0.z);
                out[1] = make_float4(r1.x, r1.y, r1.z, 0.f);
            } else {
                out[0] = make_float4(0.f, __int_as_float(lo), __int_as_float(h), 0.f);
                out[1] = make_float4(0.f, 0.f, 0.f, __int_as_float(1));
            }
        }
    }
}

cudaError_t launch_stretch_tables(const float* ax, const float* ay, const float* az, Dims d, float4* srec,
                                  float4* sbin, cudaStream_t st) {
    const long long total = (long long)(1 + STRETCH_BINS_PER_CELL) * ((d.nx - 1) + (d.ny - 1) + (d.nz - 1));
    long long g = (total + 255) / 256;
    if (g > 4096) g = 4096;
    k_stretch_tables<<<(unsigned)g, 256, 0, st>>>(ax, ay, az, d, srec, sbin);
    return cudaGetLastError();
}

// One block per brick: the brick's 9^3 nodes (clamped to the grid at the far
// faces) are scaled by the largest |component| in the brick and rounded to
// fp16, and written as x-pair records.  The scale is the brick's multiplier
// back to field units.
__global__ void __launch_bounds__(256) k_pack_h4b(const float* __restrict__ bx, const float* __restrict__ by,
                                                  const float* __restrict__ bz, Dims d, int nbx, int nby,
                                                  uint4* __restrict__ bricks, float* __restrict__ scale) {
    const int brick = blockIdx.x;
    const int bi = brick % nbx, bj = (brick / nbx) % nby, bk = brick / (nbx * nby);
    const int64_t sy = d.nx, sz = (int64_t)d.nx * d.ny;
    constexpr int NN = BRICK_NODES * BRICK_NODES * BRICK_NODES;
    __shared__ float red[256];
    float m = 0.f;
    for (int t = threadIdx.x; t < NN; t += blockDim.x) {
        const int a = t % BRICK_NODES, b = (t / BRICK_NODES) % BRICK_NODES, c = t / (BRICK_NODES * BRICK_NODES);
        const int x = min(bi * BRICK_CELLS + a, d.nx - 1), y = min(bj * BRICK_CELLS + b, d.ny - 1),
                  z = min(bk * BRICK_CELLS + c, d.nz - 1);
        const int64_t o = x + sy * y + sz * z;
        m = fmaxf(m, fmaxf(fabsf(__ldg(bx + o)), fmaxf(fabsf(__ldg(by + o)), fabsf(__ldg(bz + o)))));
    }
    red[threadIdx.x] = m;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] = fmaxf(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    const float smax = red[0];
    const float sc = (smax > 0.f && isfinite(smax)) ? smax : 1.f;
    const float inv = 1.f / sc;
    uint4* bp = bricks + (int64_t)brick * BRICK_U4;
    for (int t = threadIdx.x; t < BRICK_U4; t += blockDim.x) {
        const int a = t & 7, row = t >> 3, b = row % BRICK_NODES, c = row / BRICK_NODES;
        const int y = min(bj * BRICK_CELLS + b, d.ny - 1), z = min(bk * BRICK_CELLS + c, d.nz - 1);
        unsigned w[4];
#pragma unroll
        for (int dx = 0; dx < 2; ++dx) {
            const int x = min(bi * BRICK_CELLS + a + dx, d.nx - 1);
            const int64_t o = x + sy * y + sz * z;
            const __half2 xy = __floats2half2_rn(__ldg(bx + o) * inv, __ldg(by + o) * inv);
            const __half hz = __float2half_rn(__ldg(bz + o) * inv);
            w[2 * dx] = *reinterpret_cast<const unsigned*>(&xy);
            w[2 * dx + 1] = (unsigned)__half_as_ushort(hz);
        }
        bp[t] = make_uint4(w[0], w[1], w[2], w[3]);
    }
    if (threadIdx.x == 0) scale[brick] = sc;
}

cudaError_t launch_pack_h4b(const float* bx, const float* by, const float* bz, Dims d, int nbx, int nby, int nbz,
                            uint4* bricks, float* scale, cudaStream_t st) {
    const long long nb = (long long)nbx * nby * nbz;
    if (nb <= 0 || nb > 0x7fffffffLL) return cudaErrorInvalidValue;
    k_pack_h4b<<<(unsigned)nb, 256, 0, st>>>(bx, by, bz, d, nbx, nby, bricks, scale);
    return cudaGetLastError();
}

// One thread per cell record.  The cell's 8 corner nodes are scaled by the
// power of two 2^e with max |component| = m 2^e, m in [0.5, 1) (e clamped to
// [-100, 127]), and rounded to fp16.  Scaling by a power of two commutes with
// the rounding, so a node has the same value in every cell that holds it and
// the interpolated field stays continuous across cell faces.  Records of
// cells outside the grid (brick padding) are zero.
__global__ void __launch_bounds__(256) k_pack_h8c(const float* __restrict__ bx, const float* __restrict__ by,
                                                  const float* __restrict__ bz, Dims d, int nbx, int nby,
                                                  long long nrec, uint4* __restrict__ cells) {
    const int64_t sy = d.nx, sz = (int64_t)d.nx * d.ny;
    for (long long rec = (long long)blockIdx.x * blockDim.x + threadIdx.x; rec < nrec;
         rec += (long long)gridDim.x * blockDim.x) {
        const long long brick = rec >> 9;
        const int local = (int)(rec & 511);
        const int bi = (int)(brick % nbx), bj = (int)((brick / nbx) % nby), bk = (int)(brick / ((long long)nbx * nby));
        const int ix = bi * 8 + (local & 7), iy = bj * 8 + ((local >> 3) & 7), iz = bk * 8 + (local >> 6);
        uint4* out = cells + rec * CELL_RECORD_U4;
        if (ix > d.nx - 2 || iy > d.ny - 2 || iz > d.nz - 2) {
            const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
            out[0] = zero; out[1] = zero; out[2] = zero; out[3] = zero;
            continue;
        }
        // v[m][q]: component m of corner q = (dx << 2) | (dy << 1) | dz
        float v[3][8];
        float mx = 0.f;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int64_t o = (ix + ((q >> 2) & 1)) + sy * (iy + ((q >> 1) & 1)) + sz * (iz + (q & 1));
            v[0][q] = __ldg(bx + o);
            v[1][q] = __ldg(by + o);
            v[2][q] = __ldg(bz + o);
            mx = fmaxf(mx, fmaxf(fabsf(v[0][q]), fmaxf(fabsf(v[1][q]), fabsf(v[2][q]))));
        }
        int e = 0;
        if (mx > 0.f && isfinite(mx)) {
            frexpf(mx, &e);
            e = max(-100, min(127, e));
        }
        const float inv = ldexpf(1.f, -e);
        unsigned w[16];
#pragma unroll
        for (int m = 0; m < 3; ++m) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const __half2 h = __floats2half2_rn(v[m][k] * inv, v[m][4 + k] * inv);
                w[4 * m + k] = *reinterpret_cast<const unsigned*>(&h);
            }
        }
        w[12] = __float_as_uint(ldexpf(1.f, e));
        w[13] = 0u; w[14] = 0u; w[15] = 0u;
        out[0] = make_uint4(w[0], w[1], w[2], w[3]);
        out[1] = make_uint4(w[4], w[5], w[6], w[7]);
        out[2] = make_uint4(w[8], w[9], w[10], w[11]);
        out[3] = make_uint4(w[12], w[13], w[14], w[15]);
    }
}

cudaError_t launch_pack_h8c(const float* bx, const float* by, const float* bz, Dims d, int nbx, int nby, int nbz,
                            uint4* cells, cudaStream_t st) {
    const long long nrec = (long long)nbx * nby * nbz * 512;
    if (nrec <= 0) return cudaErrorInvalidValue;
    long long g = (nrec + 255) / 256;
    if (g > 65535LL * 64) g = 65535LL * 64;
    k_pack_h8c<<<(unsigned)g, 256, 0, st>>>(bx, by, bz, d, nbx, nby, nrec, cells);
    return cudaGetLastError();
}

}  // namespace qsl
