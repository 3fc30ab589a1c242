// Conversion of the caller's SoA field (x fastest) into the GB300 stores:
// interleaved float4 nodes and fp16 bricks with per-brick scales.
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
// fp16.  The scale is the brick's multiplier back to field units.
__global__ void __launch_bounds__(256) k_pack_h4b(const float* __restrict__ bx, const float* __restrict__ by,
                                                  const float* __restrict__ bz, Dims d, int nbx, int nby,
                                                  uint2* __restrict__ bricks, float* __restrict__ scale) {
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
    uint2* bp = bricks + (int64_t)brick * BRICK_U2;
    for (int t = threadIdx.x; t < BRICK_U2; t += blockDim.x) {
        if (t >= NN) {
            bp[t] = make_uint2(0u, 0u);
            continue;
        }
        const int a = t % BRICK_NODES, b = (t / BRICK_NODES) % BRICK_NODES, c = t / (BRICK_NODES * BRICK_NODES);
        const int x = min(bi * BRICK_CELLS + a, d.nx - 1), y = min(bj * BRICK_CELLS + b, d.ny - 1),
                  z = min(bk * BRICK_CELLS + c, d.nz - 1);
        const int64_t o = x + sy * y + sz * z;
        const __half2 xy = __floats2half2_rn(__ldg(bx + o) * inv, __ldg(by + o) * inv);
        const __half hz = __float2half_rn(__ldg(bz + o) * inv);
        uint2 u;
        u.x = *reinterpret_cast<const unsigned*>(&xy);
        u.y = (unsigned)__half_as_ushort(hz);
        bp[t] = u;
    }
    if (threadIdx.x == 0) scale[brick] = sc;
}

cudaError_t launch_pack_h4b(const float* bx, const float* by, const float* bz, Dims d, int nbx, int nby, int nbz,
                            uint2* bricks, float* scale, cudaStream_t st) {
    const long long nb = (long long)nbx * nby * nbz;
    if (nb <= 0 || nb > 0x7fffffffLL) return cudaErrorInvalidValue;
    k_pack_h4b<<<(unsigned)nb, 256, 0, st>>>(bx, by, bz, d, nbx, nby, bricks, scale);
    return cudaGetLastError();
}

}  // namespace qsl
