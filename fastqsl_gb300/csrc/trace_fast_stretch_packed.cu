// Fast tracer kernels on a stretched grid with the nodes in an interleaved
// float4 copy and the cells found through the search tables (FieldStretchP,
// the native entry).  Register budgets for 4, 5 and 6 resident blocks per
// SM; 5 is the default (the compiler's own choice, ~160 registers, holds 3
// blocks; on 1024x1024 seeds of a 256x256x128 grid: 9.3 ms at 3 blocks, 8.3
// at 4, 7.95 at 5, 8.4 at 6, seeds in 8x8 tiles).  The uniform-spacing form
// (FieldStretchPU) is in trace_fast_stretch_packed_uni.cu.
#include "qsl_kernels.cuh"

namespace qsl {

cudaError_t launch_trace_fast_stretch_packed(const TraceJob<FieldStretchP>& J, bool twist, Schedule sched,
                                             long long n_host, cudaStream_t st) {
    switch (J.occupancy) {
        case 4: return launch_fast_minb<FieldStretchP, 4>(J, twist, sched, n_host, st);
        case 6: return launch_fast_minb<FieldStretchP, 6>(J, twist, sched, n_host, st);
        default: return launch_fast_minb<FieldStretchP, 5>(J, twist, sched, n_host, st);
    }
}

}  // namespace qsl
