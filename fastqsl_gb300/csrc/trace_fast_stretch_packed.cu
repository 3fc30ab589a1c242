// Fast tracer kernels on a stretched grid with the nodes in an interleaved
// float4 copy and the cells found through the search tables (FieldStretchP,
// the native entry).  Two resident-block variants: the compiler's register
// choice held to 3 blocks per SM (168 registers; it would take 170-180 and
// drop to 2 blocks), and the 6-block budget.  The uniform-spacing form
// (FieldStretchPU) is in trace_fast_stretch_packed_uni.cu.
#include "qsl_kernels.cuh"

namespace qsl {

cudaError_t launch_trace_fast_stretch_packed(const TraceJob<FieldStretchP>& J, bool twist, Schedule sched,
                                             long long n_host, cudaStream_t st) {
    return J.occupancy == 6 ? launch_fast_minb<FieldStretchP, 6>(J, twist, sched, n_host, st)
                            : launch_fast_minb<FieldStretchP, 3>(J, twist, sched, n_host, st);
}

}  // namespace qsl
