// Fast tracer kernels on a stretched grid (FieldStretch).  One resident-block
// variant (the compiler's register choice): the stretched path is not a
// throughput path.
#include "qsl_kernels.cuh"

namespace qsl {

cudaError_t launch_trace_fast_stretch(const TraceJob<FieldStretch>& J, bool twist, Schedule sched, long long n_host,
                                      cudaStream_t st) {
    return launch_fast_minb<FieldStretch, 1>(J, twist, sched, n_host, st);
}

}  // namespace qsl
