// Fast tracer kernels on the fp16 brick store sampled with fp16 x weights
// (FieldH4BW, the QSL_ARITH_FAST_W16 option of qsl_trace).
#include "qsl_kernels.cuh"

namespace qsl {

cudaError_t launch_trace_fast_h4bw(const TraceJob<FieldH4BW>& J, bool twist, Schedule sched, long long n_host,
                                   cudaStream_t st) {
    return launch_fast(J, twist, sched, n_host, st);
}

}  // namespace qsl
