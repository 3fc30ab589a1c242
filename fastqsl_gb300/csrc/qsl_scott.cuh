// Scott-method tracer: RKF45 on the 9-component state (position p and two
// deviation vectors u, v with du/ds = (u.grad) b, dv/ds = (v.grad) b), Q from
// the deviation vectors at both footpoints.  Semantics per seed follow
// TraceAllBlineScott / TraceBlineScott (fastqslpy/cu/TraceBlineScott.cu:
// 334-595) with tol = tol_param * tol_coef (the reference's tolerance
// variable is never initialised, :352,378).
//
// grad b comes in two forms:
//   GRAD_FD       — central differences with step 1e-3 (grad_unit_vec_B,
//                   :204-226): 6 extra samples per right-hand side.
//   GRAD_ANALYTIC — the exact derivative of the trilinear field's unit
//                   vector from the same 8 corners as b itself:
//                   d(b_i)/dx_j = (dB_i/dx_j - b_i (b . dB/dx_j)) / |B|,
//                   one cell fetch per right-hand side instead of seven.
#pragma once
#include "qsl_trace.cuh"

namespace qsl {

enum GradMode { GRAD_FD = 0, GRAD_ANALYTIC = 1 };

struct Vec9 {
    float3 p, u, v;
};
__device__ __forceinline__ Vec9 add9(const Vec9& a, const Vec9& b) { return {a.p + b.p, a.u + b.u, a.v + b.v}; }
__device__ __forceinline__ Vec9 mul9(float s, const Vec9& a) { return {s * a.p, s * a.u, s * a.v}; }
__device__ __forceinline__ Vec9 div9(const Vec9& a, float s) { return {a.p / s, a.u / s, a.v / s}; }

struct ScottOut {
    float *start_x, *start_y, *start_z;
    int* flag_start;
    float *end_x, *end_y, *end_z;
    int* flag_end;
    float *bthis_x, *bthis_y, *bthis_z;
    float *q0, *qperp;
    double* line_len;
    double* twist;
};

template <class F>
struct ScottJob {
    F f;
    const int* shape_dev;
    FieldSoA cur;
    const float *inp_x, *inp_y, *inp_z;
    ScottOut o;
    TraceScalars s;
    qsl_trace_params prm;
    const unsigned* order;
    unsigned long long* samples;
};

// (u.grad) b with g[j] = d b / d x_j  (f_scott, TraceBlineScott.cu:230-249)
__device__ __forceinline__ float3 along(float3 u, const float3 g[3]) {
    return v3(dot(u, v3(g[0].x, g[1].x, g[2].x)), dot(u, v3(g[0].y, g[1].y, g[2].y)),
              dot(u, v3(g[0].z, g[1].z, g[2].z)));
}

// Unit field and its gradient by central differences of the unit field at
// p +- 1e-3 e_j.  Exact arithmetic: the offset applied in double and
// narrowed, as `x -= 0.001` on a float does, and the difference divided by
// 0.002f.  Fast arithmetic: the offset 0.001f added in float and the
// difference multiplied by 500 (rounding-level differences; no FP64 add or
// IEEE divide, nine of each per right-hand side otherwise).
template <bool EXACT, class F>
__device__ __forceinline__ float3 unit_and_grad_fd(const F& f, float3 p, float3 g[3], unsigned& ns) {
    const float3 b = sample<EXACT>(f, p, true);
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        float3 lo = p, hi = p;
        if (EXACT) {
            if (j == 0) { lo.x = (float)((double)lo.x - 0.001); hi.x = (float)((double)hi.x + 0.001); }
            if (j == 1) { lo.y = (float)((double)lo.y - 0.001); hi.y = (float)((double)hi.y + 0.001); }
            if (j == 2) { lo.z = (float)((double)lo.z - 0.001); hi.z = (float)((double)hi.z + 0.001); }
        } else {
            if (j == 0) { lo.x = lo.x - 0.001f; hi.x = hi.x + 0.001f; }
            if (j == 1) { lo.y = lo.y - 0.001f; hi.y = hi.y + 0.001f; }
            if (j == 2) { lo.z = lo.z - 0.001f; hi.z = hi.z + 0.001f; }
        }
        const float3 b1 = sample<EXACT>(f, lo, true);
        const float3 b2 = sample<EXACT>(f, hi, true);
        g[j] = EXACT ? (b2 - b1) / 0.002f : 500.f * (b2 - b1);
    }
    ns += 7;
    return b;
}

// Unit field and its exact gradient from one cell (fast arithmetic).
template <class F>
__device__ __forceinline__ float3 unit_and_grad_analytic(const F& f, float3 p, float3 g[3], unsigned& ns) {
    int ix, iy, iz;
    float rx, ry, rz;
    locate_fast(p.x, f.d.nx, ix, rx);
    locate_fast(p.y, f.d.ny, iy, ry);
    locate_fast(p.z, f.d.nz, iz, rz);
    float3 c[8];
    f.corners(ix, iy, iz, c);
    const float ox = 1.f - rx, oy = 1.f - ry, oz = 1.f - rz;
    // B and dB/dx_j of the trilinear interpolant (corner q = (dx,dy,dz) bits)
    float3 B = v3(0.f, 0.f, 0.f), Dx = B, Dy = B, Dz = B;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const float wx = (q >> 2) & 1 ? rx : ox, wy = (q >> 1) & 1 ? ry : oy, wz = q & 1 ? rz : oz;
        const float sx = (q >> 2) & 1 ? 1.f : -1.f, sy = (q >> 1) & 1 ? 1.f : -1.f, sz = q & 1 ? 1.f : -1.f;
        const float w = wx * wy * wz;
        B = B + w * c[q];
        Dx = Dx + (sx * wy * wz) * c[q];
        Dy = Dy + (sy * wx * wz) * c[q];
        Dz = Dz + (sz * wx * wy) * c[q];
    }
    const float inv = rsqrt_fast(dot(B, B));
    const float3 b = inv * B;
    const float3 D[3] = {Dx, Dy, Dz};
#pragma unroll
    for (int j = 0; j < 3; ++j) g[j] = inv * (D[j] - dot(b, D[j]) * b);
    ns += 1;
    return b;
}

template <bool EXACT, int GRAD, class F>
__device__ __forceinline__ Vec9 scott_rhs(const F& f, const Vec9& s, unsigned& ns) {
    float3 g[3];
    float3 b;
    if (GRAD == GRAD_ANALYTIC && !EXACT) b = unit_and_grad_analytic(f, s.p, g, ns);
    else b = unit_and_grad_fd<EXACT>(f, s.p, g, ns);
    return {b, along(s.u, g), along(s.v, g)};
}

// Fehlberg step on the 9-vector; the error uses the position part only
// (RKF45_Scott, TraceBlineScott.cu:256-290): its norm in exact arithmetic,
// its square in fast arithmetic (the fast controller works with log2 of it).
template <bool EXACT, int GRAD, class F>
__device__ __forceinline__ Vec9 scott_step(const F& f, const Vec9& s, float h, float& err, unsigned& ns) {
    using C = Fehlberg;
    const Vec9 k1 = mul9(h, scott_rhs<EXACT, GRAD>(f, s, ns));
    const Vec9 k2 = mul9(h, scott_rhs<EXACT, GRAD>(f, add9(s, mul9(C::a21, k1)), ns));
    const Vec9 k3 = mul9(h, scott_rhs<EXACT, GRAD>(f, add9(s, add9(mul9(C::a31, k1), mul9(C::a32, k2))), ns));
    const Vec9 k4 = mul9(h, scott_rhs<EXACT, GRAD>(
                                f, add9(s, add9(add9(mul9(C::a41, k1), mul9(C::a42, k2)), mul9(C::a43, k3))), ns));
    const Vec9 k5 = mul9(
        h, scott_rhs<EXACT, GRAD>(
               f, add9(s, add9(add9(add9(mul9(C::a51, k1), mul9(C::a52, k2)), mul9(C::a53, k3)), mul9(C::a54, k4))),
               ns));
    const Vec9 k6 = mul9(
        h, scott_rhs<EXACT, GRAD>(
               f,
               add9(s, add9(add9(add9(add9(mul9(C::a61, k1), mul9(C::a62, k2)), mul9(C::a63, k3)), mul9(C::a64, k4)),
                            mul9(C::a65, k5))),
               ns));
    const float3 e = (((C::e1 * k1.p + C::e3 * k3.p) + C::e4 * k4.p) + C::e5 * k5.p) + C::e6 * k6.p;
    err = EXACT ? norm(e) : fmaf(e.x, e.x, fmaf(e.y, e.y, e.z * e.z));
    return add9(s, add9(add9(add9(add9(mul9(C::b1, k1), mul9(C::b3, k3)), mul9(C::b4, k4)), mul9(C::b5, k5)),
                        mul9(C::b6, k6)));
}

// The same Fehlberg step for the fast arithmetic with the six stages in a
// rolled loop, so that the right-hand side (seven samples for the central
// differences) is in the loop body once instead of six times: the unrolled
// step does not fit the instruction cache.
// After stage st, its k is added into the inputs of the stages still to come,
// held in a shift register of five 9-vectors (slot i = stage st + 1 + i), so
// every index is static.  Coefficients as Fehlberg's (float).
struct ScottTab {
    float a[6][5];  // a[st][i] = A(st + 1 + i, st)
    float b[6], e[6];
};
__device__ __forceinline__ Vec9 fma9(float a, const Vec9& x, const Vec9& y) {
    return {v3(fmaf(a, x.p.x, y.p.x), fmaf(a, x.p.y, y.p.y), fmaf(a, x.p.z, y.p.z)),
            v3(fmaf(a, x.u.x, y.u.x), fmaf(a, x.u.y, y.u.y), fmaf(a, x.u.z, y.u.z)),
            v3(fmaf(a, x.v.x, y.v.x), fmaf(a, x.v.y, y.v.y), fmaf(a, x.v.z, y.v.z))};
}
static __constant__ ScottTab kScottTab = {
    {{Fehlberg::a21, Fehlberg::a31, Fehlberg::a41, Fehlberg::a51, Fehlberg::a61},
     {Fehlberg::a32, Fehlberg::a42, Fehlberg::a52, Fehlberg::a62, 0.f},
     {Fehlberg::a43, Fehlberg::a53, Fehlberg::a63, 0.f, 0.f},
     {Fehlberg::a54, Fehlberg::a64, 0.f, 0.f, 0.f},
     {Fehlberg::a65, 0.f, 0.f, 0.f, 0.f},
     {0.f, 0.f, 0.f, 0.f, 0.f}},
    {Fehlberg::b1, 0.f, Fehlberg::b3, Fehlberg::b4, Fehlberg::b5, Fehlberg::b6},
    {Fehlberg::e1, 0.f, Fehlberg::e3, Fehlberg::e4, Fehlberg::e5, Fehlberg::e6}};

template <int GRAD, class F>
__device__ __forceinline__ Vec9 scott_step_rolled(const F& f, const Vec9& s, float h, float& err, unsigned& ns) {
    const Vec9 zero = {v3(0.f, 0.f, 0.f), v3(0.f, 0.f, 0.f), v3(0.f, 0.f, 0.f)};
    Vec9 slot[5] = {zero, zero, zero, zero, zero};
    Vec9 sol = zero;
    float3 e = v3(0.f, 0.f, 0.f);
    Vec9 in = s;
#pragma unroll 1
    for (int st = 0; st < 6; ++st) {
        const Vec9 k = mul9(h, scott_rhs<false, GRAD>(f, in, ns));
#pragma unroll
        for (int i = 0; i < 5; ++i) slot[i] = fma9(kScottTab.a[st][i], k, slot[i]);
        sol = fma9(kScottTab.b[st], k, sol);
        const float ce = kScottTab.e[st];
        e = v3(fmaf(ce, k.p.x, e.x), fmaf(ce, k.p.y, e.y), fmaf(ce, k.p.z, e.z));
        in = add9(s, slot[0]);
#pragma unroll
        for (int i = 0; i < 4; ++i) slot[i] = slot[i + 1];
        slot[4] = zero;
    }
    err = fmaf(e.x, e.x, fmaf(e.y, e.y, e.z * e.z));  // squared (fast arithmetic)
    return add9(s, sol);
}

// v / |v| with the host rsqrtf of the reference's helper_math (1/sqrtf) in
// exact arithmetic, the hardware rsqrt otherwise.
template <bool EXACT>
__device__ __forceinline__ float3 unit_rsq(float3 a) {
    const float inv = EXACT ? 1.0f / sqrtf(dot(a, a)) : rsqrt_fast(dot(a, a));
    return v3(a.x * inv, a.y * inv, a.z * inv);
}

// One seed's Scott trace (TraceBlineScott, TraceBlineScott.cu:334-519).
template <bool EXACT, int GRAD, bool TWIST, class F>
__device__ void scott_line(const F& f, const ScottJob<F>& J, long long i, float s_len, float tol_coef, bool tw_on,
                           unsigned& ns) {
    const qsl_trace_params& pr = J.prm;
    const ScottOut& o = J.o;
    const float3 p0 = v3(__ldg(J.inp_x + i), __ldg(J.inp_y + i), __ldg(J.inp_z + i));
    const float3 bt = sample_endpoint<EXACT>(f, p0);
    o.bthis_x[i] = bt.x; o.bthis_y[i] = bt.y; o.bthis_z[i] = bt.z;
    if ((double)p0.z < -1e-8) {  // the reference skips seeds below z = 0
        o.start_x[i] = 0.f; o.start_y[i] = 0.f; o.start_z[i] = 0.f; o.flag_start[i] = 0;
        o.end_x[i] = 0.f; o.end_y[i] = 0.f; o.end_z[i] = 0.f; o.flag_end[i] = 0;
        o.q0[i] = 0.f; o.qperp[i] = 0.f; o.line_len[i] = 0.0;
        if (TWIST && tw_on) o.twist[i] = 0.0;
        return;
    }
    const double len_lim = pr.len_ratio * (double)(f.d.nx + f.d.ny + f.d.nz);
    // fast arithmetic: the controller in the log domain (no divide, exact
    // power or square root per step), the step limits narrowed to float
    // (the same clamps, as StepLimits argues), the length in Kahan-
    // compensated float (FP64 adds are slow on this GPU)
    typedef typename std::conditional<EXACT, double, float>::type len_t;
    const float h_max_f = (float)pr.h_max, h_min_f = (float)pr.h_min, reject_f = (float)pr.reject_factor;
    const len_t len_lim_t = (len_t)len_lim;
    const float3 b0 = sample<EXACT>(f, p0, true);
    const float nb0 = norm(sample<EXACT>(f, p0, false));
    ns += 2;
    const float tol = (float)(pr.tol * (double)tol_coef);
    const float ltol = EXACT ? 0.f : 0.2f * log2f(tol * (float)(1.0 / 11.09));
    float3 v0 = v3(b0.y, -b0.x, 0.f);
    v0 = unit_rsq<EXACT>(v0 - dot(v0, b0) * b0);
    float3 u0 = v3(b0.y * v0.z - b0.z * v0.y, b0.z * v0.x - b0.x * v0.z, b0.x * v0.y - b0.y * v0.x);
    u0 = unit_rsq<EXACT>(u0);
    const bool z0 = (double)p0.z < 1e-6;
    len_t len = 0;
    float lc = 0.f;  // Kahan compensation of len (fast arithmetic)
    double tw = 0.0;
    auto len_add = [&](double x_exact, float x_fast) {
        if (EXACT) {
            len = len + (len_t)x_exact;
        } else {
            const float y = x_fast - lc;
            const float t = (float)len + y;
            lc = (t - (float)len) - y;
            len = (len_t)t;
        }
    };
    long long steps = 0;
    Vec9 es = {p0, u0, v0}, ee = es;
    int fs = 0, fe = 0;
    float h = s_len;
    bool early = false;
    for (int sgn = -1; sgn < 2 && !early; sgn += 2) {
        Vec9 a = {p0, u0, v0};
        if (z0 && b0.z * (float)sgn < 0.f) {
            if (sgn < 0) { es = a; fs = 5; } else { ee = a; fe = 5; }
            continue;
        }
        h = fabsf(h);
        int flag = 0;
        while ((flag == 0) & (len < len_lim_t) & (steps < pr.max_steps)) {
            float err;
            Vec9 b;
            // the rolled stages pay for the central differences' seven
            // samples per stage (12.5 -> 10.7 ms on the Scott form); the
            // analytic gradient's one fetch keeps the unrolled step (3.4 ms
            // against 3.8 rolled)
            if constexpr (EXACT || GRAD == GRAD_ANALYTIC) b = scott_step<EXACT, GRAD>(f, a, h * (float)sgn, err, ns);
            else b = scott_step_rolled<GRAD>(f, a, h * (float)sgn, err, ns);
            if (EXACT) {
                const float scale = pow_cr((float)((double)(tol / err) / 11.09), 0.2f);
                if ((double)scale < 0.618) {
                    h = (float)((double)h * pr.reject_factor);
                    continue;
                }
                h = h * scale;
                if ((double)h > pr.h_max) h = (float)pr.h_max;
                if ((double)h < pr.h_min) h = (float)pr.h_min;
            } else {
                // (tol / (11.09 err))^0.2 = 2^(0.2 log2(tol / 11.09) - 0.1 log2(err^2))
                const float scale = ex2_approx(fmaf(-0.1f, lg2_approx(err), ltol));
                if (scale < 0.618f) {
                    h = h * reject_f;
                    continue;
                }
                h = h * scale;
                if (h > h_max_f) h = h_max_f;
                if (h < h_min_f) h = h_min_f;
            }
            const float dl = EXACT ? norm(b.p - a.p) : norm_fast(b.p - a.p);
            len_add((double)dl, dl);
            float td = 0.f;
            float3 bp1 = v3(0.f, 0.f, 0.f);
            if (TWIST && tw_on) {
                const float3 j1 = sample<EXACT>(current_view(f, J.cur), b.p, false);
                bp1 = sample<EXACT>(f, b.p, false);
                ns += 2;
                // fast arithmetic: the main tracer's integrand and one
                // float product (no FP64 divide per step)
                td = twist_density<EXACT>(j1, bp1);
                tw = tw + (EXACT ? (double)td / 4.0 / kRefPi * (double)dl : (double)(td * dl * kInv4PiF));
            }
            flag = box_flag(f.d, b.p);
            if (flag > 0) {
                len_add(-(double)dl, -dl);
                if (TWIST && tw_on)
                    tw = tw - (EXACT ? (double)td / 4.0 / kRefPi * (double)dl : (double)(td * dl * kInv4PiF));
                if (flag <= 6) {
                    const int d = (flag - 1) / 2;
                    const float q1 = comp(a.p, d), q2 = comp(b.p, d);
                    float qmid = q1;
                    Vec9 e;
                    if (fabsf(q1 - q2) > 0.f) {
                        qmid = (flag % 2 == 1) ? 0.f : (float)f.d.n(d);
                        e = div9(add9(mul9(q2 - qmid, a), mul9(qmid - q1, b)), q2 - q1);
                        // the exit segment's length divides by the field's
                        // component along the exit axis (B_P1, :448): with
                        // the twist on, B at the point past the face as the
                        // reference sets it (:425); with the twist off the
                        // reference leaves B_P1 unset and the unit field at
                        // the last inside point stands in (as in
                        // TraceBlineAdaptive.cu:404).  The length gates the
                        // second direction (the budget is shared).
                        float3 ua;
                        if (TWIST && tw_on) {
                            ua = bp1;
                        } else {
                            ua = sample<EXACT>(f, a.p, true);
                            ns += 1;
                        }
                        len_add((double)fabsf(qmid - q1) / (1e-4 + (double)fabsf(comp(ua, d))),
                                fabsf(qmid - q1) / (1e-4f + fabsf(comp(ua, d))));
                    } else {
                        e = a;
                    }
                    if (sgn < 0) { es = e; fs = flag; } else { ee = e; fe = flag; }
                    if (TWIST && tw_on)
                        tw = tw + (double)td / 4.0 / kRefPi * (double)fabsf(qmid - q1) /
                                      (1e-4 + (double)fabsf(comp(bp1, d)));
                } else {
                    if (sgn < 0) { es = a; fs = flag; } else { ee = a; fe = flag; }
                    early = true;  // flag 42: the reference returns with Q = 0
                    break;
                }
            }
            // on a face exit the reference still advances and counts the step
            // before its loop test ends the direction (the counter is shared)
            a = b;
            steps = steps + 1;
        }
        if (!early && flag == 0) {
            if (sgn < 0) { es = a; fs = 0; } else { ee = a; fe = 0; }
        }
    }
    float q0 = 0.f, qp = 0.f;
    if (!early) {
        // Q from the deviation vectors at both footpoints (:475-508)
        const int ds = (fs - 1) / 2, de = (fe - 1) / 2;
        const int dsc = (ds >= 0 && ds < 3) ? ds : 2, dec = (de >= 0 && de < 3) ? de : 2;
        const float3 Bs = sample<EXACT>(f, es.p, false), Be = sample<EXACT>(f, ee.p, false);
        ns += 2;
        const float BNs = comp(Bs, dsc), BNe = comp(Be, dec);
        const float3 us1 = es.u - (comp(es.u, dsc) / comp(Bs, dsc)) * Bs;
        const float3 vs1 = es.v - (comp(es.v, dsc) / comp(Bs, dsc)) * Bs;
        const float3 ue1 = ee.u - (comp(ee.u, dec) / comp(Be, dec)) * Be;
        const float3 ve1 = ee.v - (comp(ee.v, dec) / comp(Be, dec)) * Be;
        {
            const double num = (double)(dot(ue1, ue1) * dot(vs1, vs1) + dot(us1, us1) * dot(ve1, ve1)) -
                               2.0 * (double)dot(ue1, ve1) * (double)dot(us1, vs1);
            q0 = (float)(fabs(num) / fabs((double)((nb0 * nb0) / (BNs * BNe))));
        }
        {
            const float lBe = norm(Be), lBs = norm(Bs);
            const float3 ue2 = ee.u - (dot(ee.u, Be) / lBe) * (Be / lBe);
            const float3 ve2 = ee.v - (dot(ee.v, Be) / lBe) * (Be / lBe);
            const float3 us2 = es.u - (dot(es.u, Bs) / lBs) * (Bs / lBs);
            const float3 vs2 = es.v - (dot(es.v, Bs) / lBs) * (Bs / lBs);
            const double num = (double)(dot(ue2, ue2) * dot(vs2, vs2) + dot(us2, us2) * dot(ve2, ve2)) -
                               2.0 * (double)dot(ue2, ve2) * (double)dot(us2, vs2);
            qp = (float)(fabs(num) / (double)((nb0 * nb0) / (lBs * lBe)));
        }
    }
    o.start_x[i] = es.p.x; o.start_y[i] = es.p.y; o.start_z[i] = es.p.z; o.flag_start[i] = fs;
    o.end_x[i] = ee.p.x; o.end_y[i] = ee.p.y; o.end_z[i] = ee.p.z; o.flag_end[i] = fe;
    o.q0[i] = q0;
    o.qperp[i] = qp;
    o.line_len[i] = len;
    if (TWIST && tw_on) o.twist[i] = tw;
}

// One line per thread (lockstep lanes on neighbouring seeds when J.order is
// a tile order).
template <bool EXACT, int GRAD, bool TWIST, class F>
__device__ __forceinline__ void scott_kernel_body(const ScottJob<F>& J) {
    F f = J.f;
    if (J.shape_dev) {
        f.d.nx = __ldg(J.shape_dev);
        f.d.ny = __ldg(J.shape_dev + 1);
        f.d.nz = __ldg(J.shape_dev + 2);
    }
    if (f.d.nx < 2 || f.d.ny < 2 || f.d.nz < 2) return;
    const float s_len = J.s.s_len_dev ? __ldg(J.s.s_len_dev) : J.s.s_len;
    const float tol_coef = J.s.tol_coef_dev ? __ldg(J.s.tol_coef_dev) : J.s.tol_coef;
    long long n = J.s.n_dev ? (long long)__ldg(J.s.n_dev) : J.s.n;
    if (J.s.n_cap >= 0 && n > J.s.n_cap) n = J.s.n_cap;
    const bool tw_on = TWIST && (J.s.twist_flag_dev ? *J.s.twist_flag_dev : (J.s.twist_on != 0));
    unsigned ns = 0;
    unsigned long long ns_total = 0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long line = (long long)blockIdx.x * blockDim.x + threadIdx.x; line < n; line += stride) {
        const long long i = J.order ? (long long)__ldg(J.order + line) : line;
        scott_line<EXACT, GRAD, TWIST>(f, J, i, s_len, tol_coef, tw_on, ns);
        ns_total += ns;
        ns = 0;
    }
    if (J.samples) {
        __syncwarp();
        unsigned long long v = ns_total;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(J.samples, v);
    }
}

}  // namespace qsl
