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
