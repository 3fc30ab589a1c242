// Fast tracer kernels on a stretched grid, reading the caller's three arrays
// (the drop-in, and the native entry beyond the packed stores' limits): the
// reference's search (FieldStretch) and the uniform-spacing formula
// (FieldStretchU), each compiled apart.  Two resident-block variants: the
// compiler's register choice and the 6-block budget; the others spill
// without gain on this gather-latency-bound loop, and each variant costs
// compile time.
#include "qsl_kernels.cuh"

namespace qsl {

cudaError_t launch_trace_fast_stretch(const TraceJob<FieldStretch>& J, bool twist, Schedule sched, long long n_host,
                                      cudaStream_t st) {
    return J.occupancy == 6 ? launch_fast_minb<FieldStretch, 6>(J, twist, sched, n_host, st)
                            : launch_fast_minb<FieldStretch, 1>(J, twist, sched, n_host, st);
}

cudaError_t launch_trace_fast_stretch_uni(const TraceJob<FieldStretchU>& J, bool twist, Schedule sched,
                                          long long n_host, cudaStream_t st) {
    return J.occupancy == 6 ? launch_fast_minb<FieldStretchU, 6>(J, twist, sched, n_host, st)
                            : launch_fast_minb<FieldStretchU, 1>(J, twist, sched, n_host, st);
}

}  // namespace qsl
