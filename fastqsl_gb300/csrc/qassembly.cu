// Squashing-factor assembly on the device.
//
//   k_qcalc_plane   — Q on the interior pixels of stacked 2-D seed planes from
//                     the footpoint maps (fastqslpy/FastQSL.py:65-117,
//                     QCalcPlane).  FP32 form: the reference's rounding
//                     sequence; FP64 form: the same formulas in double.
//   k_flag_count / k_tile_scan / k_cook_write
//                   — order-preserving compaction of the B_flag pixels and
//                     their four pseudo-line seeds (FastQSL.py:4-57,
//                     CookPseudoLine).
//   k_qcut          — Q of each compacted pixel from its four pseudo-lines
//                     (demo/Q_RKF45CuPy.ipynb cell 10).
//   k_qmerge        — writes the pseudo-line Q into the map (cell 11).
//   k_*_jobs        — the same kernels over a table of plane jobs, one
//                     launch each for a whole batch (QPostJob).
//
// Compiled with -fmad=false so the FP32 form rounds exactly as the
// reference's array expressions do.
#include <cuda_runtime.h>
#include <stdint.h>
#include <type_traits>
#include "qassembly.h"

namespace qsl {

// Exit-face coordinates of a footpoint: z-face -> (x, y), y-face -> (z, x),
// x-face -> (y, z); flags outside 1..6 give (0, 0) (FastQSL.py:76-84).
template <class T>
__device__ __forceinline__ void face_xy(float x, float y, float z, int flag, T& X, T& Y) {
    const int d = (flag >= 1 && flag <= 6) ? (flag - 1) / 2 : -1;
    if (d == 2) { X = (T)x; Y = (T)y; }
    else if (d == 1) { X = (T)z; Y = (T)x; }
    else if (d == 0) { X = (T)y; Y = (T)z; }
    else { X = (T)0; Y = (T)0; }
}


// Q of the interior pixels first, first + stride, ... of one job.
template <bool F64>
__device__ __forceinline__ void qcalc_range(const QPlaneArgs& a, long long first, long long stride) {
    typedef typename std::conditional<F64, double, float>::type T;
    const long long m0 = a.n0 - 2, m1 = a.n1 - 2;
    const long long per = m0 * m1;
    const long long total = per * a.nplanes;
    for (long long t = first; t < total; t += stride) {
        const long long pl = t / per;
        const long long r = t - pl * per;
        const int i = (int)(r / m1) + 1, j = (int)(r % m1) + 1;
        const long long base = pl * (long long)a.n0 * a.n1;
        const long long c = base + (long long)i * a.n1 + j;
        const long long up = c + a.n1, dn = c - a.n1, rt = c + 1, lf = c - 1;
        float X1u, Y1u, X1d, Y1d, X1r, Y1r, X1l, Y1l, X2u, Y2u, X2d, Y2d, X2r, Y2r, X2l, Y2l;
        face_xy(a.xs[up], a.ys[up], a.zs[up], a.fs[up], X1u, Y1u);
        face_xy(a.xs[dn], a.ys[dn], a.zs[dn], a.fs[dn], X1d, Y1d);
        face_xy(a.xs[rt], a.ys[rt], a.zs[rt], a.fs[rt], X1r, Y1r);
        face_xy(a.xs[lf], a.ys[lf], a.zs[lf], a.fs[lf], X1l, Y1l);
        face_xy(a.xe[up], a.ye[up], a.ze[up], a.fe[up], X2u, Y2u);
        face_xy(a.xe[dn], a.ye[dn], a.ze[dn], a.fe[dn], X2d, Y2d);
        face_xy(a.xe[rt], a.ye[rt], a.ze[rt], a.fe[rt], X2r, Y2r);
        face_xy(a.xe[lf], a.ye[lf], a.ze[lf], a.fe[lf], X2l, Y2l);
        // central differences along axis 0 ("xc") and axis 1 ("yc"), taken in
        // float as the reference takes them (the FP64 form widens the
        // differences, exact in most cells, before the Jacobian products)
        const T dx2xc = (T)(X2u - X2d), dx2yc = (T)(X2r - X2l);
        const T dy2xc = (T)(Y2u - Y2d), dy2yc = (T)(Y2r - Y2l);
        const T dx1xc = (T)(X1u - X1d), dx1yc = (T)(X1r - X1l);
        const T dy1xc = (T)(Y1u - Y1d), dy1yc = (T)(Y1r - Y1l);
        const T qa = dx2xc * dy1yc - dx2yc * dy1xc;
        const T qb = dx2yc * dx1xc - dx2xc * dx1yc;
        const T qc = dy2xc * dy1yc - dy2yc * dy1xc;
        const T qd = dy2yc * dx1xc - dy2xc * dx1yc;
        T bn, bnr;
        if (F64) {
            bn = (T)a.bx0[c] * (T)a.cx + (T)a.by0[c] * (T)a.cy + (T)a.bz0[c] * (T)a.cz;
            const T abn = fabs((double)bn);
            bnr = (T)fabs((double)a.bz_in[c]) / (abn * abn) * (T)fabs((double)a.bz_out[c]) * (T)a.k64;
        } else {
            bn = (T)(a.bx0[c] * a.cx + a.by0[c] * a.cy + a.bz0[c] * a.cz);
            const T abn = (T)fabsf((float)bn);
            bnr = (T)fabsf(a.bz_in[c]) / (abn * abn) * (T)fabsf(a.bz_out[c]) * (T)a.k32;
        }
        T q = (((qa * qa + qb * qb) + qc * qc) + qd * qd) * bnr;
        if (q < (T)1) q = (T)1;
        const int fc = a.fs[c], ec = a.fe[c];
        const bool jump = (a.fs[up] != fc) | (a.fs[dn] != fc) | (a.fs[rt] != fc) | (a.fs[lf] != fc) |
                          (a.fe[up] != ec) | (a.fe[dn] != ec) | (a.fe[rt] != ec) | (a.fe[lf] != ec);
        if (jump) q = (T)NAN;
        if (F64) a.q64[t] = (double)q;
        else a.q32[t] = (float)q;
    }
}

template <bool F64>
__global__ void k_qcalc_plane(const QPlaneArgs a) {
    qcalc_range<F64>(a, (long long)blockIdx.x * blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
}

// ---- ordered compaction of flagged pixels (tile = 1024 pixels) ----
constexpr int kTile = 1024;

__device__ __forceinline__ bool pixel_selected(const int* bflag, long long p, int n0, int n1, int interior_only) {
    if (bflag[p] != 1) return false;
    if (!interior_only) return true;
    const long long per = (long long)n0 * n1;
    const long long r = p % per;
    const int i = (int)(r / n1), j = (int)(r % n1);
    return i >= 1 && i <= n0 - 2 && j >= 1 && j <= n1 - 2;
}

// Selected pixels of one tile, counted by a block of 256 threads.
__device__ __forceinline__ void flag_count_tile(const int* bflag, long long n, int n0, int n1, int interior_only,
                                                long long tile, int* tile_count) {
    const long long t0 = tile * kTile;
    int cnt = 0;
    for (int k = threadIdx.x; k < kTile; k += blockDim.x) {
        const long long p = t0 + k;
        if (p < n && pixel_selected(bflag, p, n0, n1, interior_only)) cnt++;
    }
    __shared__ int red[256];
    red[threadIdx.x] = cnt;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) tile_count[tile] = red[0];
}

__global__ void __launch_bounds__(256) k_flag_count(const int* bflag, long long n, int n0, int n1, int interior_only,
                                                    int* tile_count) {
    flag_count_tile(bflag, n, n0, n1, interior_only, blockIdx.x, tile_count);
}

// Exclusive scan of the tile counts by one block; writes the grand total
// (total[0]) and the number of pseudo-line seeds (total[1] = 4 * total[0]).
__device__ __forceinline__ void tile_scan_block(const int* tile_count, long long ntiles, long long* tile_off,
                                                unsigned long long* total) {
    __shared__ long long carry;
    __shared__ long long warp_sum[32];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (long long b = 0; b < ntiles; b += blockDim.x) {
        const long long i = b + threadIdx.x;
        long long v = i < ntiles ? tile_count[i] : 0;
        long long x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const long long y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_sum[warp] = x;
        __syncthreads();
        if (warp == 0) {
            long long w = warp_sum[lane];
            for (int o = 1; o < 32; o <<= 1) {
                const long long y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += y;
            }
            warp_sum[lane] = w;
        }
        __syncthreads();
        const long long incl = x + (warp > 0 ? warp_sum[warp - 1] : 0);
        if (i < ntiles) tile_off[i] = carry + incl - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry += incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        total[0] = (unsigned long long)carry;      // selected pixels
        total[1] = 4ull * (unsigned long long)carry;  // their pseudo-line seeds
    }
}

__global__ void __launch_bounds__(1024) k_tile_scan(const int* tile_count, long long ntiles, long long* tile_off,
                                                     unsigned long long* total) {
    tile_scan_block(tile_count, ntiles, tile_off, total);
}


// The selected pixels of one tile and their pseudo-line seeds, written in
// pixel order by a block of kTile threads.
__device__ __forceinline__ void cook_write_tile(const CookArgs& a, long long tile) {
    const long long p = tile * kTile + threadIdx.x;
    const bool sel = p < a.n && pixel_selected(a.bflag, p, a.n0, a.n1, a.interior_only);
    __shared__ int wcount[kTile / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned m = __ballot_sync(0xffffffffu, sel);
    if (lane == 0) wcount[warp] = __popc(m);
    __syncthreads();
    if (!sel) return;
    int before = 0;
    for (int w = 0; w < warp; ++w) before += wcount[w];
    unsigned lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
    const long long k = a.tile_off[tile] + before + __popc(m & lt);
    const float x = a.xs[p], y = a.ys[p], z = a.zs[p];
    const int f = a.fs[p];
    const int d = (f >= 1 && f <= 6) ? (f - 1) / 2 : -1;
    float sx[4] = {x, x, x, x}, sy[4] = {y, y, y, y}, sz[4] = {z, z, z, z};
    const float s = a.stride;
    if (d == 2) { sx[0] = x + s; sx[2] = x - s; sy[1] = y + s; sy[3] = y - s; }
    else if (d == 1) { sx[0] = x + s; sx[2] = x - s; sz[1] = z + s; sz[3] = z - s; }
    else if (d == 0) { sy[0] = y + s; sy[2] = y - s; sz[1] = z + s; sz[3] = z - s; }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        a.cx[4 * k + q] = sx[q];
        a.cy[4 * k + q] = sy[q];
        a.cz[4 * k + q] = sz[q];
    }
    a.bz0s[k] = a.bz_in[p];
    a.bz0e[k] = a.bz_out[p];
    if (a.pix) a.pix[k] = p;
}

__global__ void __launch_bounds__(kTile) k_cook_write(const CookArgs a) { cook_write_tile(a, blockIdx.x); }


template <bool F64>
__device__ __forceinline__ void qcut_range(const QcutArgs& a, long long first, long long stride) {
    typedef typename std::conditional<F64, double, float>::type T;
    const long long cnt = a.count_dev ? (long long)*a.count_dev : a.count;
    for (long long k = first; k < cnt; k += stride) {
        T X1[4], Y1[4], X2[4], Y2[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const long long i = 4 * k + q;
            face_xy(a.xs[i], a.ys[i], a.zs[i], a.fs[i], X1[q], Y1[q]);
            face_xy(a.xe[i], a.ye[i], a.ze[i], a.fe[i], X2[q], Y2[q]);
        }
        const T dx2xc = X2[0] - X2[2], dx2yc = X2[1] - X2[3];
        const T dy2xc = Y2[0] - Y2[2], dy2yc = Y2[1] - Y2[3];
        const T dx1xc = X1[0] - X1[2], dx1yc = X1[1] - X1[3];
        const T dy1xc = Y1[0] - Y1[2], dy1yc = Y1[1] - Y1[3];
        const T qa = dx2xc * dy1yc - dx2yc * dy1xc;
        const T qb = dx2yc * dx1xc - dx2xc * dx1yc;
        const T qc = dy2xc * dy1yc - dy2yc * dy1xc;
        const T qd = dy2yc * dx1xc - dy2xc * dx1yc;
        T bnr;
        if (F64) bnr = fabs((double)a.bz0e[k]) / fabs((double)a.bz0s[k]) * a.k64;
        else bnr = (T)(fabsf(a.bz0e[k]) / fabsf(a.bz0s[k]) * a.k32);
        T q = (((qa * qa + qb * qb) + qc * qc) + qd * qd) * bnr;
        if (q < (T)1) q = (T)1;
        if (F64) a.q64[k] = (double)q;
        else a.q32[k] = (float)q;
    }
}

template <bool F64>
__global__ void k_qcut(const QcutArgs a) {
    qcut_range<F64>(a, (long long)blockIdx.x * blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
}

// Q_final[plane, i-1, j-1] = Qcut[k] for each compacted interior pixel.
template <class TQ, class TC>
__device__ __forceinline__ void qmerge_range(const long long* pix, const TC* qcut, long long cnt, int n0, int n1,
                                             TQ* qfinal, long long first, long long stride) {
    const long long per = (long long)n0 * n1, per2 = (long long)(n0 - 2) * (n1 - 2);
    for (long long k = first; k < cnt; k += stride) {
        const long long p = pix[k];
        const long long pl = p / per, r = p % per;
        const int i = (int)(r / n1), j = (int)(r % n1);
        if (i >= 1 && i <= n0 - 2 && j >= 1 && j <= n1 - 2)
            qfinal[pl * per2 + (long long)(i - 1) * (n1 - 2) + (j - 1)] = (TQ)qcut[k];
    }
}

template <class TQ, class TC>
__global__ void k_qmerge(const long long* pix, const TC* qcut, const unsigned long long* count_dev, long long count,
                         int n0, int n1, TQ* qfinal) {
    const long long cnt = count_dev ? (long long)*count_dev : count;
    qmerge_range(pix, qcut, cnt, n0, n1, qfinal, (long long)blockIdx.x * blockDim.x + threadIdx.x,
                 (long long)gridDim.x * blockDim.x);
}

// ---- batched forms: one launch per kernel for every job of a table ----
// The job of block b of a grid whose begin column is `begin` (njobs + 1
// nondecreasing entries): the last j with begin[j] <= b.
__device__ __forceinline__ int post_job(const long long* begin, int njobs, long long b) {
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (begin[mid] <= b) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__global__ void __launch_bounds__(256) k_qcalc_jobs(const QPostJob* jobs, const long long* begin, int njobs) {
    const long long b = blockIdx.x;
    const int j = post_job(begin, njobs, b);
    const QPlaneArgs a = jobs[j].q;
    qcalc_range<true>(a, (b - begin[j]) * blockDim.x + threadIdx.x, jobs[j].qblocks * blockDim.x);
}

__global__ void __launch_bounds__(256) k_flag_count_jobs(const QPostJob* jobs, const long long* begin, int njobs) {
    const long long* tb = begin + (njobs + 1);
    const long long b = blockIdx.x;
    const int j = post_job(tb, njobs, b);
    const CookArgs& c = jobs[j].c;
    flag_count_tile(c.bflag, c.n, c.n0, c.n1, c.interior_only, b - tb[j], jobs[j].tile_count);
}

// one block per job
__global__ void __launch_bounds__(1024) k_tile_scan_jobs(const QPostJob* jobs, const long long* begin, int njobs) {
    const long long* tb = begin + (njobs + 1);
    const int j = blockIdx.x;
    tile_scan_block(jobs[j].tile_count, tb[j + 1] - tb[j], jobs[j].tile_off, jobs[j].total);
}

__global__ void __launch_bounds__(kTile) k_cook_write_jobs(const QPostJob* jobs, const long long* begin, int njobs) {
    const long long* tb = begin + (njobs + 1);
    const long long b = blockIdx.x;
    const int j = post_job(tb, njobs, b);
    const CookArgs a = jobs[j].c;
    cook_write_tile(a, b - tb[j]);
}

__global__ void __launch_bounds__(256) k_qcut_jobs(const QPostJob* jobs, const long long* begin, int njobs) {
    const long long* cb = begin + 2 * (njobs + 1);
    const long long b = blockIdx.x;
    const int j = post_job(cb, njobs, b);
    const QcutArgs a = jobs[j].k;
    qcut_range<true>(a, (b - cb[j]) * blockDim.x + threadIdx.x, jobs[j].cblocks * blockDim.x);
}

__global__ void __launch_bounds__(256) k_qmerge_jobs(const QPostJob* jobs, const long long* begin, int njobs) {
    const long long* cb = begin + 2 * (njobs + 1);
    const long long b = blockIdx.x;
    const int j = post_job(cb, njobs, b);
    const QPostJob& J = jobs[j];
    const long long cnt = (long long)*J.total;
    qmerge_range(J.c.pix, (const double*)J.k.q64, cnt, J.c.n0, J.c.n1, J.q.q64, (b - cb[j]) * blockDim.x + threadIdx.x,
                 J.cblocks * blockDim.x);
}

// ---- host launchers ----
static unsigned grid_for(long long n, int block) {
    long long g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > 65535LL * 32) g = 65535LL * 32;
    return (unsigned)g;
}

cudaError_t launch_qcalc_plane(const QPlaneArgs& a, bool f64, cudaStream_t st) {
    const long long total = (long long)(a.n0 - 2) * (a.n1 - 2) * a.nplanes;
    if (total <= 0) return cudaSuccess;
    if (f64) k_qcalc_plane<true><<<grid_for(total, 256), 256, 0, st>>>(a);
    else k_qcalc_plane<false><<<grid_for(total, 256), 256, 0, st>>>(a);
    return cudaGetLastError();
}

// tile_count: ceil(n/kTile) ints; tile_off: same number of int64; total: 1 u64
cudaError_t launch_cook(const CookArgs& a, int* tile_count, long long* tile_off, unsigned long long* total,
                        cudaStream_t st) {
    const long long ntiles = (a.n + kTile - 1) / kTile;
    if (ntiles <= 0) {
        return cudaMemsetAsync(total, 0, 2 * sizeof(unsigned long long), st);
    }
    if (ntiles > 0x7fffffffLL) return cudaErrorInvalidValue;
    k_flag_count<<<(unsigned)ntiles, 256, 0, st>>>(a.bflag, a.n, a.n0, a.n1, a.interior_only, tile_count);
    k_tile_scan<<<1, 1024, 0, st>>>(tile_count, ntiles, tile_off, total);
    CookArgs b = a;
    b.tile_off = tile_off;
    k_cook_write<<<(unsigned)ntiles, kTile, 0, st>>>(b);
    return cudaGetLastError();
}

long long cook_tiles(long long n) { return (n + kTile - 1) / kTile; }

cudaError_t launch_qcut(const QcutArgs& a, bool f64, long long max_count, cudaStream_t st) {
    if (max_count <= 0) return cudaSuccess;
    if (f64) k_qcut<true><<<grid_for(max_count, 256), 256, 0, st>>>(a);
    else k_qcut<false><<<grid_for(max_count, 256), 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_qmerge_f32(const long long* pix, const float* qcut, const unsigned long long* count_dev,
                              long long count, long long max_count, int n0, int n1, float* qfinal, cudaStream_t st) {
    if (max_count <= 0) return cudaSuccess;
    k_qmerge<float, float><<<grid_for(max_count, 256), 256, 0, st>>>(pix, qcut, count_dev, count, n0, n1, qfinal);
    return cudaGetLastError();
}

cudaError_t launch_qmerge_f64(const long long* pix, const double* qcut, const unsigned long long* count_dev,
                              long long count, long long max_count, int n0, int n1, double* qfinal, cudaStream_t st) {
    if (max_count <= 0) return cudaSuccess;
    k_qmerge<double, double><<<grid_for(max_count, 256), 256, 0, st>>>(pix, qcut, count_dev, count, n0, n1, qfinal);
    return cudaGetLastError();
}

long long qcalc_blocks(long long pixels) { return pixels > 0 ? (long long)grid_for(pixels, 256) : 0; }

cudaError_t launch_qpost_assemble(const QPostJob* jobs, const long long* begin, int njobs, const long long grid[3],
                                  cudaStream_t st) {
    if (njobs < 1) return cudaSuccess;
    for (int g = 0; g < 3; ++g)
        if (grid[g] < 1 || grid[g] > 0x7fffffffLL) return cudaErrorInvalidValue;
    k_qcalc_jobs<<<(unsigned)grid[0], 256, 0, st>>>(jobs, begin, njobs);
    k_flag_count_jobs<<<(unsigned)grid[1], 256, 0, st>>>(jobs, begin, njobs);
    k_tile_scan_jobs<<<(unsigned)njobs, 1024, 0, st>>>(jobs, begin, njobs);
    k_cook_write_jobs<<<(unsigned)grid[1], kTile, 0, st>>>(jobs, begin, njobs);
    return cudaGetLastError();
}

cudaError_t launch_qpost_pseudo(const QPostJob* jobs, const long long* begin, int njobs, const long long grid[3],
                                cudaStream_t st) {
    if (njobs < 1) return cudaSuccess;
    if (grid[2] < 1 || grid[2] > 0x7fffffffLL) return cudaErrorInvalidValue;
    k_qcut_jobs<<<(unsigned)grid[2], 256, 0, st>>>(jobs, begin, njobs);
    k_qmerge_jobs<<<(unsigned)grid[2], 256, 0, st>>>(jobs, begin, njobs);
    return cudaGetLastError();
}

}  // namespace qsl
