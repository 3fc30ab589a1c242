// curl B on a rectilinear (possibly stretched) grid by the three-point
// non-uniform difference of fastqslpy/FastQSL.py:120-163 (curl_of_B_grid,
// diff_3point, copy_boundary), the current density of the twist integral.
// One thread per node, float32 arithmetic in the reference's operation order
// (this translation unit is compiled with -fmad=false), float64 output as
// the reference's cupy.zeros arrays.  The reference's boundary copy (six
// plane copies in a fixed order) leaves every boundary node with the value
// of the interior node nearest to it along each axis, i.e. the value at the
// node index clamped into [1, n-2] per axis; each thread evaluates the curl
// there directly.
#include "qsl_internal.h"

namespace qsl {

struct CurlArgs {
    const float *bx, *by, *bz;
    const float *ax, *ay, *az;
    int nx, ny, nz;
    double *cx, *cy, *cz;
};

// d C / d axis at node o (interior along that axis), stride s, coordinates a,
// index i along the axis (diff_3point, FastQSL.py:143-163)
__device__ __forceinline__ float diff3(const float* __restrict__ C, long long o, long long s,
                                       const float* __restrict__ a, int i) {
    const float dl = __ldg(a + i) - __ldg(a + i - 1);
    const float dr = __ldg(a + i + 1) - __ldg(a + i);
    const float c0 = __ldg(C + o);
    const float t1 = (__ldg(C + o + s) - c0) / dr * dl / (dr + dl);
    const float t2 = (c0 - __ldg(C + o - s)) / dl * dr / (dr + dl);
    return t1 + t2;
}

__global__ void __launch_bounds__(256) k_curl(const CurlArgs A) {
    const long long nxy = (long long)A.nx * A.ny, n = nxy * A.nz;
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n;
         p += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(p / nxy);
        const long long r = p - (long long)k * nxy;
        const int j = (int)(r / A.nx), i = (int)(r - (long long)j * A.nx);
        const int ii = min(max(i, 1), A.nx - 2), jj = min(max(j, 1), A.ny - 2), kk = min(max(k, 1), A.nz - 2);
        const long long o = ii + (long long)A.nx * (jj + (long long)A.ny * kk);
        const float cxv = diff3(A.bz, o, A.nx, A.ay, jj) - diff3(A.by, o, nxy, A.az, kk);
        const float cyv = diff3(A.bx, o, nxy, A.az, kk) - diff3(A.bz, o, 1, A.ax, ii);
        const float czv = diff3(A.by, o, 1, A.ax, ii) - diff3(A.bx, o, A.nx, A.ay, jj);
        A.cx[p] = (double)cxv;
        A.cy[p] = (double)cyv;
        A.cz[p] = (double)czv;
    }
}

cudaError_t launch_curl(const float* bx, const float* by, const float* bz, const float* ax, const float* ay,
                        const float* az, int nx, int ny, int nz, double* cx, double* cy, double* cz, cudaStream_t st) {
    const CurlArgs A{bx, by, bz, ax, ay, az, nx, ny, nz, cx, cy, cz};
    const long long n = (long long)nx * ny * nz;
    long long g = (n + 255) / 256;
    if (g > 65535LL * 64) g = 65535LL * 64;
    k_curl<<<(unsigned)(g < 1 ? 1 : g), 256, 0, st>>>(A);
    return cudaGetLastError();
}

}  // namespace qsl
