// Fast tracer kernels on the fp16 cell-record store (FieldH8C).
#include "qsl_kernels.cuh"

namespace qsl {

cudaError_t launch_trace_fast_h8c(const TraceJob<FieldH8C>& J, bool twist, Schedule sched, long long n_host,
                                  cudaStream_t st) {
    return launch_fast(J, twist, sched, n_host, st);
}

cudaError_t launch_scott_fast_h8c(const ScottJob<FieldH8C>& J, int grad, bool twist, long long n_grid,
                                  cudaStream_t st) {
    return launch_scott(J, grad, twist, n_grid, st);
}

cudaError_t launch_trace_batch_h8c(const TraceJob<FieldH8C>* jobs, const long long* begin, int njobs,
                                   long long total, bool twist, unsigned long long* samples, int max_blocks,
                                   long long line_lo, long long line_hi, int occupancy, cudaStream_t st) {
    return launch_batch(jobs, begin, njobs, total, twist, samples, max_blocks, line_lo, line_hi, occupancy, st);
}

}  // namespace qsl
