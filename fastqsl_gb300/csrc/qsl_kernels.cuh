// Kernel templates of the fast tracers and their launchers, instantiated per
// field store by one translation unit each (trace_fast_soa.cu, trace_fast_f4.cu,
// trace_fast_h4b.cu, trace_fast_h8c.cu), compiled in parallel.
#pragma once
#include "qsl_internal.h"

namespace qsl {

// MINB: minimum resident blocks per SM the register allocation must allow
// (1 = compiler's choice).  Higher values trade registers (possibly spills)
// for resident warps; the autotuner measures and picks.
template <bool TWIST, bool QUEUE, class F, int MINB>
__global__ void __launch_bounds__(kTraceBlock, MINB) k_trace_fast(const TraceJob<F> J) {
    trace_kernel_body<false, TWIST, QUEUE>(J);
}

template <class F, int MINB>
static cudaError_t launch_fast_minb(const TraceJob<F>& J, bool twist, Schedule sched, long long n_host,
                                    cudaStream_t st) {
    const bool q = sched == SCHED_QUEUE;
    const void* k = q ? (twist ? (const void*)k_trace_fast<true, true, F, MINB>
                               : (const void*)k_trace_fast<false, true, F, MINB>)
                      : (twist ? (const void*)k_trace_fast<true, false, F, MINB>
                               : (const void*)k_trace_fast<false, false, F, MINB>);
    int grid;
    if (q) {
        grid = persistent_grid(k, kTraceBlock);
    } else {
        long long g = (n_host + kTraceBlock - 1) / kTraceBlock;
        // a device-side count (n_host is only the capacity): two resident
        // waves of blocks stride over the lines instead of a grid over the
        // whole capacity whose surplus blocks would each start and exit
        if (J.s.n_dev) {
            const long long cap = 2LL * persistent_grid(k, kTraceBlock);
            if (cap > 0 && g > cap) g = cap;
        }
        grid = (int)(g < 1 ? 1 : (g > (1 << 30) ? (1 << 30) : g));
    }
    if (grid <= 0) return cudaErrorInvalidConfiguration;
    if (q) {
        if (twist) k_trace_fast<true, true, F, MINB><<<grid, kTraceBlock, 0, st>>>(J);
        else k_trace_fast<false, true, F, MINB><<<grid, kTraceBlock, 0, st>>>(J);
    } else {
        if (twist) k_trace_fast<true, false, F, MINB><<<grid, kTraceBlock, 0, st>>>(J);
        else k_trace_fast<false, false, F, MINB><<<grid, kTraceBlock, 0, st>>>(J);
    }
    return cudaGetLastError();
}

template <class F>
static cudaError_t launch_fast(const TraceJob<F>& J, bool twist, Schedule sched, long long n_host, cudaStream_t st) {
    switch (J.occupancy) {
        case 6: return launch_fast_minb<F, 6>(J, twist, sched, n_host, st);
        case 7: return launch_fast_minb<F, 7>(J, twist, sched, n_host, st);
        case 8: return launch_fast_minb<F, 8>(J, twist, sched, n_host, st);
        case 9: return launch_fast_minb<F, 9>(J, twist, sched, n_host, st);
        case 10: return launch_fast_minb<F, 10>(J, twist, sched, n_host, st);
        default: return launch_fast_minb<F, 1>(J, twist, sched, n_host, st);
    }
}

// (held to 3 blocks per SM: 168 registers; the twist form would take ~210)
template <int GRAD, bool TWIST, class F>
__global__ void __launch_bounds__(kTraceBlock, 3) k_scott_fast(const ScottJob<F> J) {
    scott_kernel_body<false, GRAD, TWIST>(J);
}

template <class F>
static cudaError_t launch_scott(const ScottJob<F>& J, int grad, bool twist, long long n_grid, cudaStream_t st) {
    long long g = (n_grid + kTraceBlock - 1) / kTraceBlock;
    const int grid = (int)(g < 1 ? 1 : (g > (1 << 30) ? (1 << 30) : g));
    if (grad == GRAD_ANALYTIC) {
        if (twist) k_scott_fast<GRAD_ANALYTIC, true, F><<<grid, kTraceBlock, 0, st>>>(J);
        else k_scott_fast<GRAD_ANALYTIC, false, F><<<grid, kTraceBlock, 0, st>>>(J);
    } else {
        if (twist) k_scott_fast<GRAD_FD, true, F><<<grid, kTraceBlock, 0, st>>>(J);
        else k_scott_fast<GRAD_FD, false, F><<<grid, kTraceBlock, 0, st>>>(J);
    }
    return cudaGetLastError();
}

// Batched trace: one line per thread; MINB resident blocks per SM the
// register allocation must allow (6-10; the autotuner picks, 8 by default).
template <bool TWIST, class F, int MINB>
__global__ void __launch_bounds__(kTraceBlock, MINB) k_trace_batch(const TraceJob<F>* __restrict__ jobs,
                                                                    const long long* __restrict__ begin, int njobs,
                                                                    unsigned long long* samples, long long line_lo,
                                                                    long long line_hi) {
    batch_kernel_body<TWIST>(jobs, begin, njobs, samples, line_lo, line_hi);
}

template <class F, int MINB>
static void launch_batch_minb(int grid, const TraceJob<F>* jobs, const long long* begin, int njobs, bool twist,
                              unsigned long long* samples, long long line_lo, long long line_hi, cudaStream_t st) {
    if (twist) k_trace_batch<true, F, MINB><<<grid, kTraceBlock, 0, st>>>(jobs, begin, njobs, samples, line_lo, line_hi);
    else k_trace_batch<false, F, MINB><<<grid, kTraceBlock, 0, st>>>(jobs, begin, njobs, samples, line_lo, line_hi);
}

template <class F>
static cudaError_t launch_batch(const TraceJob<F>* jobs, const long long* begin, int njobs, long long total,
                                bool twist, unsigned long long* samples, int max_blocks, long long line_lo,
                                long long line_hi, int occupancy, cudaStream_t st) {
    if (njobs <= 0 || total <= 0) return cudaSuccess;
    if (line_lo < 0) line_lo = 0;
    if (line_hi < 0 || line_hi > total) line_hi = total;
    if (line_lo >= line_hi) return cudaSuccess;
    long long g = (line_hi - line_lo + kTraceBlock - 1) / kTraceBlock;
    if (max_blocks > 0 && g > max_blocks) g = max_blocks;  // the grid-stride loop covers the rest
    const int grid = (int)(g > (1 << 30) ? (1 << 30) : g);
    switch (occupancy) {
        case 6: launch_batch_minb<F, 6>(grid, jobs, begin, njobs, twist, samples, line_lo, line_hi, st); break;
        case 7: launch_batch_minb<F, 7>(grid, jobs, begin, njobs, twist, samples, line_lo, line_hi, st); break;
        case 9: launch_batch_minb<F, 9>(grid, jobs, begin, njobs, twist, samples, line_lo, line_hi, st); break;
        case 10: launch_batch_minb<F, 10>(grid, jobs, begin, njobs, twist, samples, line_lo, line_hi, st); break;
        default: launch_batch_minb<F, 8>(grid, jobs, begin, njobs, twist, samples, line_lo, line_hi, st); break;
    }
    return cudaGetLastError();
}

}  // namespace qsl
