// One launch over many trace jobs: different fields (of one store type),
// seed sets, integrators and tolerances.  Each job's lines occupy a
// warp-aligned range [begin[j], begin[j] + n_j) of the launch's line space, so
// no warp mixes two jobs; a thread finds its job by binary search over the
// (small) begin table and traces one line with that job's settings, forward
// then backward, lanes in lockstep.  Used for batched uneven solves (many
// fields in one captured graph) and by the serving loop to merge the work of
// concurrently admitted requests into one launch.
#pragma once
#include "qsl_trace.cuh"

namespace qsl {

template <bool TWIST, class F>
__device__ __forceinline__ void batch_line(const TraceJob<F>& J, long long line, unsigned& ns) {
    F f = J.f;
    if (f.d.nx < 2 || f.d.ny < 2 || f.d.nz < 2) return;
    long long n = J.s.n;
    if (J.s.n_dev) {  // count produced on the device; the range was sized by n
        const long long nd = (long long)__ldg(J.s.n_dev);
        n = nd < n ? nd : n;
    }
    if (line >= n) return;  // padding lane of the job's warp-aligned range
    const long long i = J.order ? (long long)__ldg(J.order + line) : line;
    const float s_len = J.s.s_len, tol_coef = J.s.tol_coef;
    const float3 nrm = v3(J.s.cross[0], J.s.cross[1], J.s.cross[2]);
    const bool tw_on = TWIST && J.s.twist_on != 0;
    store_prepare(f);
    float len_lim;
    if constexpr (std::is_same<F, FieldH4B>::value || std::is_same<F, FieldH4BW>::value || std::is_same<F, FieldF4>::value ||
                  std::is_same<F, FieldH8C>::value)
        len_lim = J.lim.len_lim;
    else
        len_lim = (float)(J.prm.len_ratio * len_scale(f));
    Lane<false> L;
    lane_begin<false>(f, J, L, i, +1, s_len, tol_coef, nrm, ns);
    const TraceOut& o = J.o;
    while (true) {
        if (!lane_step<false, TWIST>(f, J, L, len_lim, tw_on, ns)) continue;
        if (L.dsign == 0) {
            const float3 be = sample_endpoint<false>(f, L.out);
            ns += 1;
            o.end_x[i] = L.out.x; o.end_y[i] = L.out.y; o.end_z[i] = L.out.z;
            o.flag_end[i] = lane_flag(L.flag);
            if (o.status_end) o.status_end[i] = lane_status(L.flag);
            o.bend_x[i] = be.x; o.bend_y[i] = be.y; o.bend_z[i] = be.z;
            o.line_len[i] = (double)L.len;
            if (TWIST && tw_on) o.twist[i] = L.tw;
            lane_begin<false>(f, J, L, i, -1, s_len, tol_coef, nrm, ns);
            continue;
        }
        const float3 bs = sample_endpoint<false>(f, L.out);
        const float3 p0 = v3(__ldg(J.inp_x + i), __ldg(J.inp_y + i), __ldg(J.inp_z + i));
        const float3 b0 = sample_endpoint<false>(f, p0);
        ns += 2;
        o.start_x[i] = L.out.x; o.start_y[i] = L.out.y; o.start_z[i] = L.out.z;
        o.flag_start[i] = lane_flag(L.flag);
        if (o.status_start) o.status_start[i] = lane_status(L.flag);
        o.bstart_x[i] = bs.x; o.bstart_y[i] = bs.y; o.bstart_z[i] = bs.z;
        o.bthis_x[i] = b0.x; o.bthis_y[i] = b0.y; o.bthis_z[i] = b0.z;
        o.line_len[i] = o.line_len[i] + (double)L.len;
        if (TWIST && tw_on) o.twist[i] = o.twist[i] + L.tw;
        const float bn = b0.x * nrm.x + b0.y * nrm.y + b0.z * nrm.z;
        const float bm = sqrtf(b0.x * b0.x + b0.y * b0.y + b0.z * b0.z);
        o.b_flag[i] = ((double)fabsf(bn) * 100. < (double)bm) ? 1 : 0;
        break;
    }
}

// begin[j]: first line of job j (multiples of 32, increasing); begin[njobs]:
// the total.  Each job's TraceJob sits in device memory.  Only the lines of
// the window [line_lo, line_hi) run (a multiple of 32 for line_lo keeps every
// warp inside one job).
template <bool TWIST, class F>
__device__ __forceinline__ void batch_kernel_body(const TraceJob<F>* __restrict__ jobs,
                                                  const long long* __restrict__ begin, int njobs,
                                                  unsigned long long* samples, long long line_lo,
                                                  long long line_hi) {
    long long total = __ldg(begin + njobs);
    total = line_hi < total ? line_hi : total;
    const long long stride = (long long)gridDim.x * blockDim.x;
    unsigned ns = 0;
    unsigned long long ns_total = 0;
    for (long long g = line_lo + (long long)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += stride) {
        int lo = 0, hi = njobs - 1;  // last j with begin[j] <= g
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(begin + mid) <= g) lo = mid;
            else hi = mid - 1;
        }
        batch_line<TWIST>(jobs[lo], g - __ldg(begin + lo), ns);
        ns_total += ns;
        ns = 0;
    }
    if (samples) {
        __syncwarp();
        unsigned long long v = ns_total;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(samples, v);
    }
}

}  // namespace qsl
