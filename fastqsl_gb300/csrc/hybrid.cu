// Hybrid finite-difference + Scott Q (demo/Q_RKF45MixCuPyDiffScott.ipynb
// cell 9): the interior pixels whose finite-difference Q is unusable — B_flag
// set (the field lies within ~0.6 degrees of the seed plane) or Q NaN (a
// boundary-flag jump among the four neighbours) — are re-traced with the
// Scott deviation-vector tracer and take its q_perp.  The notebook gathers
// those seeds on the host (cupy.where, fancy indexing) and scatters q_perp
// back through host memory; here both steps are kernels and the Scott pass
// reads its seed count from the device.
#include "qsl_internal.h"

namespace qsl {

// Interior pixel p of the stacked planes: plane k, row i+1, column j+1 of an
// (n0, n1) plane; Q index p = (k (n0-2) + i) (n1-2) + j; seed (k n0 + i+1) n1 + j+1.
__device__ __forceinline__ long long hybrid_seed(long long p, long long n0, long long n1) {
    const long long w = n1 - 2, h = n0 - 2;
    const long long k = p / (w * h), r = p - k * w * h;
    const long long i = r / w, j = r - i * w;
    return (k * n0 + i + 1) * n1 + j + 1;
}

// One warp-aggregated append per warp: the selected seeds' order in the list
// is not deterministic, the results are (each line is traced on its own).
__global__ void __launch_bounds__(256) k_hybrid_select(const int* __restrict__ bflag, const double* __restrict__ q,
                                                       long long n0, long long n1, long long npix,
                                                       unsigned* __restrict__ seeds,
                                                       unsigned long long* __restrict__ count) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long base = (long long)blockIdx.x * blockDim.x;
    for (long long p0 = base; p0 < npix; p0 += stride) {  // uniform trip count per warp
        const long long p = p0 + threadIdx.x;
        long long s = 0;
        bool bad = false;
        if (p < npix) {
            s = hybrid_seed(p, n0, n1);
            bad = (__ldg(bflag + s) != 0) | isnan(__ldg(q + p));
        }
        const unsigned m = __ballot_sync(0xffffffffu, bad);
        if (!m) continue;
        const int lane = threadIdx.x & 31;
        unsigned long long w0 = 0;
        if (lane == __ffs(m) - 1) w0 = atomicAdd(count, (unsigned long long)__popc(m));
        w0 = __shfl_sync(0xffffffffu, w0, __ffs(m) - 1);
        if (bad) seeds[w0 + __popc(m & ((1u << lane) - 1u))] = (unsigned)s;
    }
}

__global__ void __launch_bounds__(256) k_hybrid_merge(const int* __restrict__ bflag, const float* __restrict__ qperp,
                                                      long long n0, long long n1, long long npix,
                                                      double* __restrict__ q) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += stride) {
        const long long s = hybrid_seed(p, n0, n1);
        const double v = q[p];
        if ((__ldg(bflag + s) != 0) | isnan(v)) q[p] = (double)__ldg(qperp + s);
    }
}

static int grid_of(long long n) {
    long long g = (n + 255) / 256;
    return (int)(g < 1 ? 1 : (g > 65535LL * 16 ? 65535LL * 16 : g));
}

cudaError_t launch_hybrid_select(const int* bflag, const double* q, long long n0, long long n1, long long nplanes,
                                 unsigned* seeds, unsigned long long* count, cudaStream_t st) {
    const long long npix = nplanes * (n0 - 2) * (n1 - 2);
    cudaError_t e = cudaMemsetAsync(count, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess || npix <= 0) return e;
    // whole warps per block: the ballot needs every lane of a warp in the loop
    k_hybrid_select<<<grid_of(npix), 256, 0, st>>>(bflag, q, n0, n1, npix, seeds, count);
    return cudaGetLastError();
}

cudaError_t launch_hybrid_merge(const int* bflag, const float* qperp, long long n0, long long n1, long long nplanes,
                                double* q, cudaStream_t st) {
    const long long npix = nplanes * (n0 - 2) * (n1 - 2);
    if (npix <= 0) return cudaSuccess;
    k_hybrid_merge<<<grid_of(npix), 256, 0, st>>>(bflag, qperp, n0, n1, npix, q);
    return cudaGetLastError();
}

}  // namespace qsl
