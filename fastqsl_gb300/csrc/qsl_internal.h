// Internal launch interface between the C ABI (capi.cu) and the kernel
// translation units.  Not installed; the public surface is
// include/fastqsl_gb300.h.
#pragma once
#include <cuda_runtime.h>
#include "qsl_batch.cuh"
#include "qsl_scott.cuh"
#include "qsl_trace.cuh"

namespace qsl {

enum Layout { LAYOUT_SOA = 0, LAYOUT_F4 = 1, LAYOUT_H4B = 2, LAYOUT_H8C = 3 };
constexpr int kStoreTypes = 4;
enum Schedule { SCHED_QUEUE = 0, SCHED_STATIC = 1 };

constexpr int kTraceBlock = 128;

// Blocks of `kernel` that fit on one SM at kTraceBlock threads, times the SM
// count: the persistent grid.
int persistent_grid(const void* kernel, int block, size_t smem = 0);

// trace_exact.cu (compiled with -fmad=false)
cudaError_t launch_trace_exact(const TraceJob<FieldSoA>& J, bool twist, Schedule sched, long long n_host,
                               cudaStream_t st);
cudaError_t launch_trace_exact_stretch(const TraceJob<FieldStretch>& J, bool twist, Schedule sched, long long n_host,
                                       cudaStream_t st);
cudaError_t launch_trace_exact_stretch_uni(const TraceJob<FieldStretchU>& J, bool twist, Schedule sched,
                                           long long n_host, cudaStream_t st);
// trace_fast_stretch.cu
cudaError_t launch_trace_fast_stretch(const TraceJob<FieldStretch>& J, bool twist, Schedule sched, long long n_host,
                                      cudaStream_t st);
cudaError_t launch_trace_fast_stretch_uni(const TraceJob<FieldStretchU>& J, bool twist, Schedule sched,
                                          long long n_host, cudaStream_t st);
cudaError_t launch_trace_fast_stretch_packed(const TraceJob<FieldStretchP>& J, bool twist, Schedule sched,
                                             long long n_host, cudaStream_t st);
// trace_fast_stretch_packed_uni.cu
cudaError_t launch_trace_fast_stretch_packed_uni(const TraceJob<FieldStretchPU>& J, bool twist, Schedule sched,
                                                 long long n_host, cudaStream_t st);

// trace_fast_<store>.cu
cudaError_t launch_trace_fast_soa(const TraceJob<FieldSoA>& J, bool twist, Schedule sched, long long n_host,
                                  cudaStream_t st);
cudaError_t launch_trace_fast_f4(const TraceJob<FieldF4>& J, bool twist, Schedule sched, long long n_host,
                                 cudaStream_t st);
cudaError_t launch_trace_fast_h4b(const TraceJob<FieldH4B>& J, bool twist, Schedule sched, long long n_host,
                                  cudaStream_t st);
cudaError_t launch_trace_fast_h8c(const TraceJob<FieldH8C>& J, bool twist, Schedule sched, long long n_host,
                                  cudaStream_t st);
// trace_fast_h4bw.cu
cudaError_t launch_trace_fast_h4bw(const TraceJob<FieldH4BW>& J, bool twist, Schedule sched, long long n_host,
                                   cudaStream_t st);

// Scott tracer (one line per thread); exact arithmetic uses GRAD_FD
cudaError_t launch_scott_exact(const ScottJob<FieldSoA>& J, bool twist, long long n_grid, cudaStream_t st);
cudaError_t launch_scott_fast_soa(const ScottJob<FieldSoA>& J, int grad, bool twist, long long n_grid,
                                  cudaStream_t st);
cudaError_t launch_scott_fast_f4(const ScottJob<FieldF4>& J, int grad, bool twist, long long n_grid, cudaStream_t st);
cudaError_t launch_scott_fast_h4b(const ScottJob<FieldH4B>& J, int grad, bool twist, long long n_grid,
                                  cudaStream_t st);
cudaError_t launch_scott_fast_h8c(const ScottJob<FieldH8C>& J, int grad, bool twist, long long n_grid,
                                  cudaStream_t st);

// Batched trace over a job table in device memory (trace_fast_<store>.cu)
cudaError_t launch_trace_batch_soa(const TraceJob<FieldSoA>* jobs, const long long* begin, int njobs,
                                   long long total, bool twist, unsigned long long* samples, int max_blocks,
                                   long long line_lo, long long line_hi, int occupancy, cudaStream_t st);
cudaError_t launch_trace_batch_f4(const TraceJob<FieldF4>* jobs, const long long* begin, int njobs, long long total,
                                  bool twist, unsigned long long* samples, int max_blocks,
                                   long long line_lo, long long line_hi, int occupancy, cudaStream_t st);
cudaError_t launch_trace_batch_h4b(const TraceJob<FieldH4B>* jobs, const long long* begin, int njobs,
                                   long long total, bool twist, unsigned long long* samples, int max_blocks,
                                   long long line_lo, long long line_hi, int occupancy, cudaStream_t st);
cudaError_t launch_trace_batch_h8c(const TraceJob<FieldH8C>* jobs, const long long* begin, int njobs,
                                   long long total, bool twist, unsigned long long* samples, int max_blocks,
                                   long long line_lo, long long line_hi, int occupancy, cudaStream_t st);

// curl.cu (compiled with -fmad=false)
cudaError_t launch_curl(const float* bx, const float* by, const float* bz, const float* ax, const float* ay,
                        const float* az, int nx, int ny, int nz, double* cx, double* cy, double* cz, cudaStream_t st);

// path.cu (compiled with -fmad=false)
cudaError_t launch_trace_path(const float* bx, const float* by, const float* bz, int nx, int ny, int nz,
                              const double* seeds, long long n, long long start, long long stop, long long stride,
                              double dr, float* ox, float* oy, float* oz, long long out_len, cudaStream_t st);
cudaError_t launch_sample_points(const float* bx, const float* by, const float* bz, int nx, int ny, int nz,
                                 const double* pts, long long n, int normalize, double* out, cudaStream_t st);

// hybrid.cu
cudaError_t launch_hybrid_select(const int* bflag, const double* q, long long n0, long long n1, long long nplanes,
                                 unsigned* seeds, unsigned long long* count, cudaStream_t st);
cudaError_t launch_hybrid_merge(const int* bflag, const float* qperp, long long n0, long long n1, long long nplanes,
                                double* q, cudaStream_t st);

// field_store.cu
cudaError_t launch_pack_f4(const float* bx, const float* by, const float* bz, Dims d, float4* out, cudaStream_t st);
cudaError_t launch_pack_f4x2(const float* bx, const float* by, const float* bz, Dims d, float4* out,
                             cudaStream_t st);
cudaError_t launch_stretch_tables(const float* ax, const float* ay, const float* az, Dims d, float4* srec,
                                  float4* sbin, cudaStream_t st);
cudaError_t launch_pack_h4b(const float* bx, const float* by, const float* bz, Dims d, int nbx, int nby, int nbz,
                            uint4* bricks, float* scale, cudaStream_t st);
cudaError_t launch_pack_h8c(const float* bx, const float* by, const float* bz, Dims d, int nbx, int nby, int nbz,
                            uint4* cells, cudaStream_t st);

}  // namespace qsl
