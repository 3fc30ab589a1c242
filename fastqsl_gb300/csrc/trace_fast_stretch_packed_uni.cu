// Fast tracer kernels on a stretched grid with the nodes in an interleaved
// float4 copy and the cells found by the uniform-spacing formula
// (FieldStretchPU, the native entry with uni set): a translation unit of its
// own so that it compiles beside the table form; the same two resident-block
// variants (3 and 6 blocks per SM).
#include "qsl_kernels.cuh"

namespace qsl {

cudaError_t launch_trace_fast_stretch_packed_uni(const TraceJob<FieldStretchPU>& J, bool twist, Schedule sched,
                                                 long long n_host, cudaStream_t st) {
    return J.occupancy == 6 ? launch_fast_minb<FieldStretchPU, 6>(J, twist, sched, n_host, st)
                            : launch_fast_minb<FieldStretchPU, 3>(J, twist, sched, n_host, st);
}

}  // namespace qsl
