// Fast tracer kernels on a stretched grid with the nodes in an interleaved
// float4 copy (FieldStretchP, the native entry); the same two resident-block
// variants as trace_fast_stretch.cu.
#include "qsl_kernels.cuh"

namespace qsl {

cudaError_t launch_trace_fast_stretch_packed(const TraceJob<FieldStretchP>& J, bool twist, Schedule sched,
                                             long long n_host, cudaStream_t st) {
    return J.occupancy == 6 ? launch_fast_minb<FieldStretchP, 6>(J, twist, sched, n_host, st)
                            : launch_fast_minb<FieldStretchP, 1>(J, twist, sched, n_host, st);
}

}  // namespace qsl
