// Fast tracer kernels on a stretched grid with the nodes in an interleaved
// float4 copy and the cells found by the uniform-spacing formula
// (FieldStretchPU, the native entry with uni set): a translation unit of its
// own so that it compiles beside the table form; the same resident-block
// variants (4, 5 and 6 blocks per SM; 5 by default).
#include "qsl_kernels.cuh"

namespace qsl {

cudaError_t launch_trace_fast_stretch_packed_uni(const TraceJob<FieldStretchPU>& J, bool twist, Schedule sched,
                                                 long long n_host, cudaStream_t st) {
    switch (J.occupancy) {
        case 4: return launch_fast_minb<FieldStretchPU, 4>(J, twist, sched, n_host, st);
        case 6: return launch_fast_minb<FieldStretchPU, 6>(J, twist, sched, n_host, st);
        default: return launch_fast_minb<FieldStretchPU, 5>(J, twist, sched, n_host, st);
    }
}

}  // namespace qsl
