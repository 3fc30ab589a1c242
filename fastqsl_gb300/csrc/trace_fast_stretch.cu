// Fast tracer kernels on a stretched grid (FieldStretch), in the same
// resident-block variants as the uniform stores (the compiler's register
// choice leaves 3 blocks per SM for this gather-latency-bound loop).
#include "qsl_kernels.cuh"

namespace qsl {

cudaError_t launch_trace_fast_stretch(const TraceJob<FieldStretch>& J, bool twist, Schedule sched, long long n_host,
                                      cudaStream_t st) {
    return launch_fast(J, twist, sched, n_host, st);
}

cudaError_t launch_trace_fast_stretch_packed(const TraceJob<FieldStretchP>& J, bool twist, Schedule sched,
                                             long long n_host, cudaStream_t st) {
    return launch_fast(J, twist, sched, n_host, st);
}

}  // namespace qsl
