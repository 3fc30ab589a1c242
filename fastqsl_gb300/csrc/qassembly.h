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

cudaError_t launch_qcalc_plane(const QPlaneArgs& a, bool f64, cudaStream_t st);
long long cook_tiles(long long n);
cudaError_t launch_cook(const CookArgs& a, int* tile_count, long long* tile_off, unsigned long long* total,
                        cudaStream_t st);
cudaError_t launch_qcut(const QcutArgs& a, bool f64, long long max_count, cudaStream_t st);
cudaError_t launch_qmerge_f32(const long long* pix, const float* qcut, const unsigned long long* count_dev,
                              long long count, long long max_count, int n0, int n1, float* qfinal, cudaStream_t st);
cudaError_t launch_qmerge_f64(const long long* pix, const double* qcut, const unsigned long long* count_dev,
                              long long count, long long max_count, int n0, int n1, double* qfinal, cudaStream_t st);

}  // namespace qsl
