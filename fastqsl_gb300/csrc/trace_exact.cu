// Reference-parity tracer kernels.
//
// This translation unit is compiled with -fmad=false: no multiply and add are
// fused, so each float expression rounds exactly where the reference's does
// when built without contraction (the oracle's rule).  Together with the
// double-precision corner weights and IEEE divide / sqrt of the exact
// sampler, the results agree with the reference tracing routine bit for bit
// except where powf differs by an ulp.
#include "qsl_internal.h"

namespace qsl {

template <bool TWIST, bool QUEUE, class F>
__global__ void __launch_bounds__(kTraceBlock) k_trace_exact(const TraceJob<F> J) {
    trace_kernel_body<true, TWIST, QUEUE>(J);
}

template <class F>
static cudaError_t launch_exact(const TraceJob<F>& J, bool twist, Schedule sched, long long n_host, cudaStream_t st) {
    const bool q = sched == SCHED_QUEUE;
    const void* k = q ? (twist ? (const void*)k_trace_exact<true, true, F> : (const void*)k_trace_exact<false, true, F>)
                      : (twist ? (const void*)k_trace_exact<true, false, F> : (const void*)k_trace_exact<false, false, F>);
    int grid;
    if (q) {
        grid = persistent_grid(k, kTraceBlock);
    } else {
        long long g = (n_host + kTraceBlock - 1) / kTraceBlock;
        grid = (int)(g < 1 ? 1 : (g > (1 << 30) ? (1 << 30) : g));
    }
    if (grid <= 0) return cudaErrorInvalidConfiguration;
    if (q) {
        if (twist) k_trace_exact<true, true, F><<<grid, kTraceBlock, 0, st>>>(J);
        else k_trace_exact<false, true, F><<<grid, kTraceBlock, 0, st>>>(J);
    } else {
        if (twist) k_trace_exact<true, false, F><<<grid, kTraceBlock, 0, st>>>(J);
        else k_trace_exact<false, false, F><<<grid, kTraceBlock, 0, st>>>(J);
    }
    return cudaGetLastError();
}

cudaError_t launch_trace_exact(const TraceJob<FieldSoA>& J, bool twist, Schedule sched, long long n_host,
                               cudaStream_t st) {
    return launch_exact(J, twist, sched, n_host, st);
}

cudaError_t launch_trace_exact_stretch(const TraceJob<FieldStretch>& J, bool twist, Schedule sched, long long n_host,
                                       cudaStream_t st) {
    return launch_exact(J, twist, sched, n_host, st);
}

cudaError_t launch_trace_exact_stretch_uni(const TraceJob<FieldStretchU>& J, bool twist, Schedule sched,
                                           long long n_host, cudaStream_t st) {
    return launch_exact(J, twist, sched, n_host, st);
}

template <bool TWIST>
__global__ void __launch_bounds__(kTraceBlock) k_scott_exact(const ScottJob<FieldSoA> J) {
    scott_kernel_body<true, GRAD_FD, TWIST>(J);
}

static int grid_for_lines(long long n) {
    long long g = (n + kTraceBlock - 1) / kTraceBlock;
    return (int)(g < 1 ? 1 : (g > (1 << 30) ? (1 << 30) : g));
}

cudaError_t launch_scott_exact(const ScottJob<FieldSoA>& J, bool twist, long long n_grid, cudaStream_t st) {
    const int grid = grid_for_lines(n_grid);
    if (twist) k_scott_exact<true><<<grid, kTraceBlock, 0, st>>>(J);
    else k_scott_exact<false><<<grid, kTraceBlock, 0, st>>>(J);
    return cudaGetLastError();
}

}  // namespace qsl
