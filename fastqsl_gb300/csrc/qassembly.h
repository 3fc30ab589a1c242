// Argument blocks and launchers of the Q-assembly kernels (qassembly.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace qsl {

struct QPlaneArgs {
    const float *xe, *ye, *ze;
    const int* fe;
    const float *xs, *ys, *zs;
    const int* fs;
    const float *bz_in, *bz_out;    // Bz at the start (in) and end (out) footpoints
    const float *bx0, *by0, *bz0;   // B at the seed
    float cx, cy, cz;               // seed-plane normal
    int n0, n1;                     // plane shape (rows, columns)
    long long nplanes;
    float k32;                      // (1/(2*stride))^4 rounded to float
    double k64;
    float* q32;                     // (nplanes, n0-2, n1-2) outputs; one of the two
    double* q64;
};

struct CookArgs {
    const int* bflag;
    const float *xs, *ys, *zs;  // start footpoints
    const int* fs;
    const float *bz_in, *bz_out;
    long long n;
    int n0, n1, interior_only;
    float stride;
    const long long* tile_off;
    float *cx, *cy, *cz;        // 4 seeds per selected pixel
    float *bz0s, *bz0e;         // Bz at start / end of the selected pixel
    long long* pix;             // pixel index of each selected pixel (optional)
};

struct QcutArgs {
    const float *xs, *ys, *zs;
    const int* fs;
    const float *xe, *ye, *ze;
    const int* fe;
    const float *bz0s, *bz0e;
    const unsigned long long* count_dev;  // number of pixels (when set)
    long long count;
    float k32;
    double k64;
    float* q32;
    double* q64;
};

// One plane job of a batched Q assembly (FP64 Q): the argument blocks of
// its Q, compaction and pseudo-Q kernels, and the first block each batched
// grid gives it.  A table of these sits in device memory; every block of a
// batched launch finds its job by bisecting the begin columns.
struct QPostJob {
    QPlaneArgs q;                  // q64 set
    CookArgs c;                    // c.tile_off = tile_off
    int* tile_count;               // cook_tiles(c.n) ints
    long long* tile_off;           // cook_tiles(c.n) offsets (the scan's output)
    unsigned long long* total;     // [0] selected pixels, [1] their pseudo-line seeds
    QcutArgs k;                    // count_dev = total; q64 = the pseudo Q
    long long qblocks;             // blocks of the job's Q grid (grid-stride loop inside)
    long long cblocks;             // blocks of its pseudo-Q and merge grids
};
// begin[g * (njobs + 1) + j]: first block of job j in batched grid g
// (0: Q, 1: compaction tiles, 2: pseudo Q and merge); entry njobs the total.
constexpr int kPostGrids = 3;

cudaError_t launch_qcalc_plane(const QPlaneArgs& a, bool f64, cudaStream_t st);
long long cook_tiles(long long n);
cudaError_t launch_cook(const CookArgs& a, int* tile_count, long long* tile_off, unsigned long long* total,
                        cudaStream_t st);
cudaError_t launch_qcut(const QcutArgs& a, bool f64, long long max_count, cudaStream_t st);
cudaError_t launch_qmerge_f32(const long long* pix, const float* qcut, const unsigned long long* count_dev,
                              long long count, long long max_count, int n0, int n1, float* qfinal, cudaStream_t st);
cudaError_t launch_qmerge_f64(const long long* pix, const double* qcut, const unsigned long long* count_dev,
                              long long count, long long max_count, int n0, int n1, double* qfinal, cudaStream_t st);
// Blocks of a job's Q grid and of its pseudo-Q / merge grids (the
// per-job launchers' grid sizes).
long long qcalc_blocks(long long pixels);
// The batched pipeline of njobs jobs (device table `jobs`, begin columns
// `begin`, grid totals `grid[3]` = the begin columns' last entries): Q of
// every job, then the compaction of every job's flagged pixels (counts,
// scans, writes); and, after the pseudo-line trace, every job's pseudo Q and
// merge.  The same kernels' arithmetic as the per-job launchers.
cudaError_t launch_qpost_assemble(const QPostJob* jobs, const long long* begin, int njobs, const long long grid[3],
                                  cudaStream_t st);
cudaError_t launch_qpost_pseudo(const QPostJob* jobs, const long long* begin, int njobs, const long long grid[3],
                                cudaStream_t st);

}  // namespace qsl
