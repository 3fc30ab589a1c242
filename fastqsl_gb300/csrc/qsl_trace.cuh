// Field-line tracer kernels (RK4 / RKF45), templated on the field store and
// the arithmetic.  Semantics per seed follow the reference's TraceAllBline
// (fastqslpy/cu/TraceBlineAdaptive.cu:429-510, fastqslpy/cu/TraceBline.cu:
// 383-464): forward trace -> end footpoint, backward trace -> start footpoint,
// B at both footpoints and at the seed, B_flag, line length, optional twist.
//
// Scheduling: a persistent grid (a multiple of the SM count) in which every
// lane owns one line at a time and, the moment its line finishes, takes the
// next one from a device work counter (one warp-aggregated atomic per refill).
// Lines whose lengths differ by orders of magnitude (RKF45 near nulls and
// separators) therefore never hold a warp's other lanes idle.  A static mode
// (one line per thread, no counter) is the plain baseline.
#pragma once
#include <type_traits>
#include "qsl_field.cuh"
#include "../../include/fastqsl_gb300.h"

namespace qsl {

constexpr double kRefPi = 3.14159265;  // the reference's M_PI (TraceBlineAdaptive.cu:10)
// 1 / (4 pi) for the fast twist increment: one float product per step and a
// single double add, instead of the reference's double divides (the FP64
// pipe is narrow on this GPU)
constexpr float kInv4PiF = (float)(1.0 / (4.0 * kRefPi));

struct TraceOut {
    float *start_x, *start_y, *start_z;
    int* flag_start;
    float *end_x, *end_y, *end_z;
    int* flag_end;
    float *bthis_x, *bthis_y, *bthis_z;
    int* b_flag;
    float *bstart_x, *bstart_y, *bstart_z;
    float *bend_x, *bend_y, *bend_z;
    double* line_len;
    double* twist;
    int* status_start;  // optional qsl_line_status per direction
    int* status_end;
};

// Scalars the reference passes as one-element device arrays are read from
// device memory when the *_dev pointer is set, else taken by value.
struct TraceScalars {
    const float* s_len_dev;
    const float* tol_coef_dev;
    const unsigned long long* n_dev;
    const float* cross_dev;
    const bool* twist_flag_dev;
    long long n_cap;  // >= 0: lines beyond this index are never touched (array capacity)
    float s_len;
    float tol_coef;
    long long n;
    float cross[3];
    int twist_on;
};

// Step-size limits of the adaptive controller narrowed to float once on the
// host.  For a float h and a double bound H, `h > H` and `h > (float)H` clamp
// h to the same value (the only float between H and its rounding is the
// rounding itself), so the fast kernels compare in float and keep the FP64
// pipe off the per-step path.  max_steps is clamped to the int range of the
// lane's step counter.
struct StepLimits {
    float h_min, h_max, reject;
    int max_steps;
    float len_lim;  // len_ratio x (nx + ny + nz) in float, formed on the host (packed stores)
};

template <class F>
struct TraceJob {
    F f;
    const int* shape_dev;  // when set, the field dims are read from here (nx, ny, nz)
    FieldSoA cur;  // current density for the twist integral (the caller's arrays)
    F cur_store;   // or, when cur_packed, the current density in a store of F's layout
    int cur_packed;
    const float *inp_x, *inp_y, *inp_z;
    TraceOut o;
    TraceScalars s;
    qsl_trace_params prm;
    StepLimits lim;               // prm's controller limits in float (fast arithmetic)
    unsigned long long* queue;    // work counter, zero at launch; null = static
    unsigned long long* samples;  // optional: total field samples
    const unsigned* order;        // optional: line k traces seed order[k] and writes its outputs there
    int chunk;                    // lines a warp takes from the queue at a time (QUEUE)
    int occupancy;                // resident-block variant of the fast kernels (0 = default)
};

// Fehlberg 4(5) coefficients, stored to float as the reference does
// (TraceBlineAdaptive.cu:224-235).
struct Fehlberg {
    static constexpr float a21 = (float)(1. / 4.);
    static constexpr float a31 = (float)(3. / 32.), a32 = (float)(9. / 32.);
    static constexpr float a41 = (float)(1932. / 2197.), a42 = (float)(-7200. / 2197.), a43 = (float)(7296. / 2197.);
    static constexpr float a51 = (float)(439. / 216.), a52 = -8.f, a53 = (float)(3680. / 513.),
                           a54 = (float)(-845. / 4104.);
    static constexpr float a61 = (float)(-8. / 27.), a62 = 2.f, a63 = (float)(-3544. / 2565.),
                           a64 = (float)(1859. / 4104.), a65 = (float)(-11. / 40.);
    static constexpr float b1 = (float)(16. / 135.), b3 = (float)(6656. / 12825.), b4 = (float)(28561. / 56430.),
                           b5 = (float)(-9. / 50.), b6 = (float)(2. / 55.);
    static constexpr float e1 = (float)(1. / 360.), e3 = (float)(-128. / 4275.), e4 = (float)(-2197. / 75240.),
                           e5 = (float)(1. / 50.), e6 = (float)(2. / 55.);
};

// One Fehlberg step (RKF45, TraceBlineAdaptive.cu:215-254): returns the
// 5th-order increment (the reference adds it to P0 in one rounding) and the
// error estimate: its norm in exact arithmetic; in fast arithmetic its
// square, h^2 |e|^2 (the fast controller works with log2 of it, so no square
// root is taken).
// Vector as an (x, y) pair for the packed f32x2 pipe plus a scalar z.
struct PV {
    float2 xy;
    float z;
};
__device__ __forceinline__ PV pv(float3 a) { return {make_float2(a.x, a.y), a.z}; }
__device__ __forceinline__ float3 f3(PV a) { return v3(a.xy.x, a.xy.y, a.z); }
// a*x + y
__device__ __forceinline__ PV axpy(float a, PV x, PV y) {
    return {__ffma2_rn(make_float2(a, a), x.xy, y.xy), fmaf(a, x.z, y.z)};
}
__device__ __forceinline__ PV scal(float a, PV x) { return {__fmul2_rn(make_float2(a, a), x.xy), a * x.z}; }

// Fast-arithmetic Fehlberg step: the same stages on the unit field b with
// the step folded in once per stage (p + h * sum a_ij b_j), combinations on
// packed (x, y) pairs.  Differs from the reference's rounding sequence only
// in rounding.  err2: the squared error estimate h^2 |e|^2.
template <class F>
__device__ __forceinline__ float3 step_rkf45_fast(const F& f, float3 p, float h, float& err2, unsigned& ns,
                                                 float3* b_raw = nullptr) {
    using C = Fehlberg;
    const PV P = pv(p);
    // b_raw: also return B itself at p (from the same interpolation)
    const PV b1 = pv(b_raw ? sample_unit_raw(f, p, *b_raw) : sample<false>(f, p, true));
    const PV b2 = pv(sample<false>(f, f3(axpy(h * C::a21, b1, P)), true));
    PV c = axpy(C::a32, b2, scal(C::a31, b1));
    const PV b3 = pv(sample<false>(f, f3(axpy(h, c, P)), true));
    c = axpy(C::a43, b3, axpy(C::a42, b2, scal(C::a41, b1)));
    const PV b4 = pv(sample<false>(f, f3(axpy(h, c, P)), true));
    c = axpy(C::a54, b4, axpy(C::a53, b3, axpy(C::a52, b2, scal(C::a51, b1))));
    const PV b5 = pv(sample<false>(f, f3(axpy(h, c, P)), true));
    c = axpy(C::a65, b5, axpy(C::a64, b4, axpy(C::a63, b3, axpy(C::a62, b2, scal(C::a61, b1)))));
    const PV b6 = pv(sample<false>(f, f3(axpy(h, c, P)), true));
    const PV e = axpy(C::e6, b6, axpy(C::e5, b5, axpy(C::e4, b4, axpy(C::e3, b3, scal(C::e1, b1)))));
    err2 = (h * h) * fmaf(e.xy.x, e.xy.x, fmaf(e.xy.y, e.xy.y, e.z * e.z));
    ns += 6;
    return f3(scal(h, axpy(C::b6, b6, axpy(C::b5, b5, axpy(C::b4, b4, axpy(C::b3, b3, scal(C::b1, b1)))))));
}

// The fast Fehlberg step with its six stages in a rolled loop, for the
// stretched-grid stores: their sample (three axis searches, eight corner
// loads and the blend) inlined six times makes a loop body that does not fit
// the instruction cache.  The sums of the stages still to come are held in
// a shift register of five vectors: entering stage st, slot[i] is the sum
// of stage st + i (slot[0] complete); after its sample each slot takes the
// next one's sum plus this stage's term, so the shift costs no moves and
// every index is static.  Coefficients from constant memory.  The same sums
// in the same order as step_rkf45_fast except that the step multiplies each
// stage's sum (h * sum a_ij b_j) instead of being folded into a21.
struct FehlbergTab {
    float a[6][5];  // a[st][i] = A(st + 1 + i, st)
    float b[6], e[6];
};
static __constant__ FehlbergTab kFehlbergTab = {
    {{Fehlberg::a21, Fehlberg::a31, Fehlberg::a41, Fehlberg::a51, Fehlberg::a61},
     {Fehlberg::a32, Fehlberg::a42, Fehlberg::a52, Fehlberg::a62, 0.f},
     {Fehlberg::a43, Fehlberg::a53, Fehlberg::a63, 0.f, 0.f},
     {Fehlberg::a54, Fehlberg::a64, 0.f, 0.f, 0.f},
     {Fehlberg::a65, 0.f, 0.f, 0.f, 0.f},
     {0.f, 0.f, 0.f, 0.f, 0.f}},
    {Fehlberg::b1, 0.f, Fehlberg::b3, Fehlberg::b4, Fehlberg::b5, Fehlberg::b6},
    {Fehlberg::e1, 0.f, Fehlberg::e3, Fehlberg::e4, Fehlberg::e5, Fehlberg::e6}};

template <class F>
struct RolledStages : std::false_type {};
template <int M>
struct RolledStages<FieldStretchT<M>> : std::true_type {};

template <class F>
__device__ __forceinline__ float3 step_rkf45_fast_rolled(const F& f, float3 p, float h, float& err2, unsigned& ns,
                                                        float3* b_raw) {
    const PV P = pv(p);
    const PV zero = {make_float2(0.f, 0.f), 0.f};
    PV slot[5] = {zero, zero, zero, zero, zero};
    PV sol = zero, e = zero;
    // b_raw (twist kernels): the first stage's B itself, from its own
    // interpolation before the loop so that the loop holds one sample
    PV b = pv(b_raw ? sample_unit_raw(f, p, *b_raw) : sample<false>(f, p, true));
#pragma unroll 1
    for (int st = 0; st < 6; ++st) {
        if (st > 0) b = pv(sample<false>(f, f3(axpy(h, slot[0], P)), true));
#pragma unroll
        for (int i = 0; i < 4; ++i) slot[i] = axpy(kFehlbergTab.a[st][i], b, slot[i + 1]);
        slot[4] = scal(kFehlbergTab.a[st][4], b);
        sol = axpy(kFehlbergTab.b[st], b, sol);
        e = axpy(kFehlbergTab.e[st], b, e);
    }
    err2 = (h * h) * fmaf(e.xy.x, e.xy.x, fmaf(e.xy.y, e.xy.y, e.z * e.z));
    ns += 6;
    return f3(scal(h, sol));
}

template <bool EXACT, class F>
__device__ __forceinline__ float3 step_rkf45(const F& f, float3 p, float h, float& err, unsigned& ns,
                                            float3* b_raw = nullptr) {
    if constexpr (!EXACT && RolledStages<F>::value) return step_rkf45_fast_rolled(f, p, h, err, ns, b_raw);
    if (!EXACT) return step_rkf45_fast(f, p, h, err, ns, b_raw);
    using C = Fehlberg;
    const float3 k1 = h * sample<EXACT>(f, p, true);
    const float3 k2 = h * sample<EXACT>(f, p + C::a21 * k1, true);
    const float3 k3 = h * sample<EXACT>(f, p + (C::a31 * k1 + C::a32 * k2), true);
    const float3 k4 = h * sample<EXACT>(f, p + ((C::a41 * k1 + C::a42 * k2) + C::a43 * k3), true);
    const float3 k5 = h * sample<EXACT>(f, p + (((C::a51 * k1 + C::a52 * k2) + C::a53 * k3) + C::a54 * k4), true);
    const float3 k6 =
        h * sample<EXACT>(f, p + ((((C::a61 * k1 + C::a62 * k2) + C::a63 * k3) + C::a64 * k4) + C::a65 * k5), true);
    const float3 e = (((C::e1 * k1 + C::e3 * k3) + C::e4 * k4) + C::e5 * k5) + C::e6 * k6;
    err = norm(e);
    ns += 6;
    return (((C::b1 * k1 + C::b3 * k3) + C::b4 * k4) + C::b5 * k5) + C::b6 * k6;
}

// Classic RK4 on b (RK4, TraceBlineAdaptive.cu:259-267); returns the
// increment.  The 1/6 factor is formed as (1./6.)*h in double and narrowed.
template <bool EXACT, class F>
__device__ __forceinline__ float3 step_rk4(const F& f, float3 p, float h, unsigned& ns, float3* b_raw = nullptr) {
    const float3 k1 = (!EXACT && b_raw) ? sample_unit_raw(f, p, *b_raw) : sample<EXACT>(f, p, true);
    const float3 k2 = sample<EXACT>(f, p + (h * k1) / 2.f, true);
    const float3 k3 = sample<EXACT>(f, p + (h * k2) / 2.f, true);
    const float3 k4 = sample<EXACT>(f, p + h * k3, true);
    ns += 4;
    const float c = EXACT ? (float)(1.0 / 6.0 * (double)h) : h * (1.f / 6.f);
    return c * (((k1 + 2.f * k2) + 2.f * k3) + k4);
}

// RK4 in the face-normal coordinate, dx/dq = b / b_d over dq = h
// (RK4_boundary, TraceBlineAdaptive.cu:286-307).  Out of line (it runs once
// per line end); the store view is taken by value so that the caller's copy
// never has its address taken.  4 field samples.
template <bool EXACT, class F>
__device__ __noinline__ float3 step_rk4_normal(const F f, float3 p, float h, int d) {
    float3 b = sample_outlined<EXACT>(f, p, true);
    const float3 k1 = b / comp(b, d);
    b = sample_outlined<EXACT>(f, p + (h * k1) / 2.f, true);
    const float3 k2 = b / comp(b, d);
    b = sample_outlined<EXACT>(f, p + (h * k2) / 2.f, true);
    const float3 k3 = b / comp(b, d);
    b = sample_outlined<EXACT>(f, p + h * k3, true);
    const float3 k4 = b / comp(b, d);
    const float c = EXACT ? (float)(1.0 / 6.0 * (double)h) : h * (1.f / 6.f);
    return p + c * (((k1 + 2.f * k2) + 2.f * k3) + k4);
}

// The same boundary RK4 inlined, its four stages in a rolled loop, for the
// stretched-grid stores: the out-of-line form takes the store view by value,
// and for their large views (coordinate arrays, per-axis constants, search
// tables) the caller then keeps a copy of the view in local memory, which
// the hot loop reads too.  The same operations in the same order.
template <bool EXACT, class F>
__device__ __forceinline__ float3 step_rk4_normal_rolled(const F& f, float3 p, float h, int d) {
    float3 k1 = v3(0.f, 0.f, 0.f), k2 = k1, k3 = k1, k4 = k1, q = p;
#pragma unroll 1
    for (int st = 0; st < 4; ++st) {
        const float3 b = sample<EXACT>(f, q, true);
        const float3 k = b / comp(b, d);
        if (st == 0) {
            k1 = k;
            q = p + (h * k1) / 2.f;
        } else if (st == 1) {
            k2 = k;
            q = p + (h * k2) / 2.f;
        } else if (st == 2) {
            k3 = k;
            q = p + h * k3;
        } else {
            k4 = k;
        }
    }
    const float c = EXACT ? (float)(1.0 / 6.0 * (double)h) : h * (1.f / 6.f);
    return p + c * (((k1 + 2.f * k2) + 2.f * k3) + k4);
}

// Boundary classification (checkFlag, TraceBlineAdaptive.cu:309-331).
__device__ __forceinline__ int box_flag(const Dims& n, float3 p) {
    const float X = (float)(n.nx - 1), Y = (float)(n.ny - 1), Z = (float)(n.nz - 1);
    if ((p.x >= 0.f) & (p.y > 0.f) & (p.z >= 0.f) & (p.x <= X) & (p.y <= Y) & (p.z <= Z)) return 0;
    int f = 42;
    if ((p.x < 0.f) & (p.y >= 0.f) & (p.z >= 0.f) & (p.x < X) & (p.y < Y) & (p.z < Z)) f = 1;
    if ((p.x >= 0.f) & (p.y >= 0.f) & (p.z >= 0.f) & (p.x >= X) & (p.y < Y) & (p.z < Z)) f = 2;
    if ((p.x >= 0.f) & (p.y < 0.f) & (p.z >= 0.f) & (p.x < X) & (p.y < Y) & (p.z < Z)) f = 3;
    if ((p.x >= 0.f) & (p.y >= 0.f) & (p.z >= 0.f) & (p.x < X) & (p.y >= Y) & (p.z < Z)) f = 4;
    if ((p.x >= 0.f) & (p.y >= 0.f) & (p.z < 0.f) & (p.x < X) & (p.y < Y) & (p.z < Z)) f = 5;
    if ((p.x >= 0.f) & (p.y >= 0.f) & (p.z >= 0.f) & (p.x < X) & (p.y < Y) & (p.z >= Z)) f = 6;
    return f;
}

// ---------------------------------------------------------------------------
// Per-store geometry: the box tests, the length-limit scale, the kernel-start
// set-up and the view of the twist current density on the store's grid.
// ---------------------------------------------------------------------------
template <class F>
__device__ __forceinline__ bool box_inside(const F& f, float3 p) {
    return (p.x >= 0.f) & (p.y > 0.f) & (p.z >= 0.f) & (p.x <= (float)(f.d.nx - 1)) &
           (p.y <= (float)(f.d.ny - 1)) & (p.z <= (float)(f.d.nz - 1));
}
template <class F>
__device__ __forceinline__ int box_exit(const F& f, float3 p) {
    return box_flag(f.d, p);
}
// len_lim = len_ratio * this (the node counts' sum)
template <class F>
__device__ __forceinline__ double len_scale(const F& f) {
    return (double)(f.d.nx + f.d.ny + f.d.nz);
}
template <class F>
__device__ __forceinline__ void store_prepare(F&) {}
// Whether this launch's kernel does the work: always, except for the
// drop-in's two stretched kernels (search / uniform formula), of which only
// the one matching the caller's device flag runs.
template <class F>
__device__ __forceinline__ bool store_active(const F&) { return true; }
template <int M>
__device__ __forceinline__ bool store_active(const FieldStretchT<M>& f) {
    if constexpr (M == 4 || M == 5) {
        if (f.uni_dev) return (*f.uni_dev) == (M == 4);
    }
    return true;
}
// The current density shares the traced field's grid; J.cur carries only its
// three arrays, the geometry comes from the traced store (whose dims may have
// been read from the device at kernel start).
template <class F>
__device__ __forceinline__ FieldSoA current_view(const F& f, const FieldSoA& c) {
    return FieldSoA{c.bx, c.by, c.bz, f.d};
}

// Stretched grid (checkFlag, TraceBlineAdaptiveStretch.cu:309-331): the same
// tests against the first and last node coordinates.
template <int M>
__device__ __forceinline__ bool box_inside(const FieldStretchT<M>& f, float3 p) {
    return (p.x >= f.lo.x) & (p.y > f.lo.y) & (p.z >= f.lo.z) & (p.x <= f.hi.x) & (p.y <= f.hi.y) &
           (p.z <= f.hi.z);
}
template <int M>
__device__ __forceinline__ int box_exit(const FieldStretchT<M>& f, float3 p) {
    const float3 a = f.lo, b = f.hi;
    if ((p.x >= a.x) & (p.y > a.y) & (p.z >= a.z) & (p.x <= b.x) & (p.y <= b.y) & (p.z <= b.z)) return 0;
    int r = 42;
    if ((p.x < a.x) & (p.y >= a.y) & (p.z >= a.z) & (p.x < b.x) & (p.y < b.y) & (p.z < b.z)) r = 1;
    if ((p.x >= a.x) & (p.y >= a.y) & (p.z >= a.z) & (p.x >= b.x) & (p.y < b.y) & (p.z < b.z)) r = 2;
    if ((p.x >= a.x) & (p.y < a.y) & (p.z >= a.z) & (p.x < b.x) & (p.y < b.y) & (p.z < b.z)) r = 3;
    if ((p.x >= a.x) & (p.y >= a.y) & (p.z >= a.z) & (p.x < b.x) & (p.y >= b.y) & (p.z < b.z)) r = 4;
    if ((p.x >= a.x) & (p.y >= a.y) & (p.z < a.z) & (p.x < b.x) & (p.y < b.y) & (p.z < b.z)) r = 5;
    if ((p.x >= a.x) & (p.y >= a.y) & (p.z >= a.z) & (p.x < b.x) & (p.y < b.y) & (p.z >= b.z)) r = 6;
    return r;
}
// the summed coordinate extents, in float as the reference (:337-339)
template <int M>
__device__ __forceinline__ double len_scale(const FieldStretchT<M>& f) {
    return (double)(((f.hi.x + f.hi.y) + f.hi.z) - ((f.lo.x + f.lo.y) + f.lo.z));
}
template <int M>
__device__ __forceinline__ void store_prepare(FieldStretchT<M>& f) {
    // the packed stores' constants are formed on the host (qsl_trace_stretch)
    // in this same arithmetic and stay kernel parameters
    if constexpr (M == 1 || M == 2) return;
    f.lo = v3(__ldg(f.ax), __ldg(f.ay), __ldg(f.az));
    f.hi = v3(__ldg(f.ax + f.d.nx - 1), __ldg(f.ay + f.d.ny - 1), __ldg(f.az + f.d.nz - 1));
    // per-sample constants of the cell search, formed once (the FP64 pipe
    // is narrow on this GPU)
    f.clo = v3((float)((double)f.lo.x + 1e-6), (float)((double)f.lo.y + 1e-6), (float)((double)f.lo.z + 1e-6));
    f.chi = v3((float)((double)f.hi.x - 1e-6), (float)((double)f.hi.y - 1e-6), (float)((double)f.hi.z - 1e-6));
    f.us = v3((f.hi.x - f.lo.x) / __int2float_rd(f.d.nx), (f.hi.y - f.lo.y) / __int2float_rd(f.d.ny),
              (f.hi.z - f.lo.z) / __int2float_rd(f.d.nz));
    if constexpr (M == 1) {
        // the bin width of the search tables (only picks the bin; the
        // tables' ranges absorb its rounding)
        f.sbinv = v3((float)(STRETCH_BINS_PER_CELL * (f.d.nx - 1)) / (f.hi.x - f.lo.x),
                     (float)(STRETCH_BINS_PER_CELL * (f.d.ny - 1)) / (f.hi.y - f.lo.y),
                     (float)(STRETCH_BINS_PER_CELL * (f.d.nz - 1)) / (f.hi.z - f.lo.z));
    } else if constexpr (M == 4) {
        // the uniform formula's reciprocal spacing (fast arithmetic)
        f.sbinv = v3(1.f / f.us.x, 1.f / f.us.y, 1.f / f.us.z);
    }
}
// The current density is always the caller's arrays: a view of them on the
// store's grid that finds cells the way the store does (a packed store's
// tables or formula, else the drop-in's run-time choice).
template <int M>
__device__ __forceinline__ auto current_view(const FieldStretchT<M>& f, const FieldSoA& c) {
    FieldStretchT<M == 1 ? 3 : (M == 2 ? 4 : M)> r;
    r.bx = c.bx;
    r.by = c.by;
    r.bz = c.bz;
    r.d = f.d;
    r.ax = f.ax;
    r.ay = f.ay;
    r.az = f.az;
    r.uni_dev = nullptr;
    r.lo = f.lo;
    r.hi = f.hi;
    r.clo = f.clo;
    r.chi = f.chi;
    r.us = f.us;
    r.b4 = nullptr;
    r.srec = f.srec;
    r.sbin = f.sbin;
    r.sbinv = f.sbinv;
    return r;
}

// x^y correctly rounded to float: the double-precision power narrowed once
// (its error is far below half a float ulp except within ~2^-28 of a float
// rounding boundary).  The exact kernels use it so that the step controller's
// decisions do not depend on one library's powf rounding.
__device__ __forceinline__ float pow_cr(float x, float y) { return (float)pow((double)x, (double)y); }

// J.B / |B|^2, the twist integrand.  The fast form fixes its rounding
// sequence with explicit multiply-adds: left as plain expressions, the
// compiler is free to fuse the products in an order that depends on the code
// around them, and two kernels tracing the same line would then differ in
// the last bit.  (The exact form is compiled without fusion.)
template <bool EXACT>
__device__ __forceinline__ float twist_density(float3 j, float3 b) {
    if (EXACT) return dot(j, b) / dot(b, b);
    const float jb = fmaf(j.z, b.z, fmaf(j.y, b.y, __fmul_rn(j.x, b.x)));
    const float bb = fmaf(b.z, b.z, fmaf(b.y, b.y, __fmul_rn(b.x, b.x)));
    return jb / bb;
}

// Per-lane state of one direction of one line.  The length accumulates in
// double for exact arithmetic (as the reference does) and in Kahan-
// compensated float otherwise (FP64 adds are slow on GB300).
template <bool EXACT>
struct Lane {
    typedef typename std::conditional<EXACT, double, float>::type len_t;
    float3 p;      // current point
    float3 pc;     // Kahan compensation of p (fast arithmetic)
    float h;       // current step
    float tol;     // local error tolerance (fast arithmetic: 0.2 log2(tol / 11.09), the controller's form)
    len_t len;     // accumulated length
    float lc;      // Kahan compensation of len (fast arithmetic)
    double tw;     // accumulated twist
    int steps;     // accepted steps
    int rej;       // trial steps rejected in a row
    unsigned dsign;  // sign bit of the step: 0 forward, 0x80000000 backward
    long long line;
    float3 out;    // footpoint of this direction when finished
    int flag;      // reference flag; bits 8.. hold the qsl_line_status when finished
};

// The reference flag and the qsl_line_status of a finished direction
// (packed into Lane::flag so that the status costs no register in the loop).
__device__ __forceinline__ int lane_flag(int packed) { return packed & 0xff; }
__device__ __forceinline__ int lane_status(int packed) { return packed >> 8; }
__device__ __forceinline__ int pack_flag(int flag, int status) { return flag | (status << 8); }

template <bool EXACT>
__device__ __forceinline__ void len_add(Lane<EXACT>& L, double x_exact, float x_fast) {
    if (EXACT) {
        L.len = L.len + x_exact;
    } else {
        const float y = x_fast - L.lc;
        const float t = (float)L.len + y;
        L.lc = (t - (float)L.len) - y;
        L.len = t;
    }
}

template <bool EXACT, class F>
__device__ __forceinline__ void lane_begin(const F& f, const TraceJob<F>& J, Lane<EXACT>& L, long long line, int dir,
                                           float s_len, float tol_coef, const float3 nrm, unsigned& ns) {
    L.line = line;
    L.dsign = dir > 0 ? 0u : 0x80000000u;
    L.p = v3(__ldg(J.inp_x + line), __ldg(J.inp_y + line), __ldg(J.inp_z + line));
    L.pc = v3(0.f, 0.f, 0.f);
    L.h = s_len;
    L.len = 0;
    L.lc = 0.f;
    L.tw = 0.0;
    L.steps = 0;
    L.rej = 0;
    L.flag = 0;
    L.out = L.p;
    L.tol = 0.f;
    if (J.prm.integrator == QSL_RKF45) {
        // tolerance law (TraceBlineAdaptive.cu:351-359)
        const float3 b0 = sample<EXACT>(f, L.p, true);
        ns += 1;
        const float bn = fabsf(dot(b0, nrm));
        float tol;
        if (J.prm.tol_law == QSL_TOL_REFERENCE) {
            if ((double)bn <= 0.05) tol = (float)(J.prm.tol / 8e3);
            else tol = (float)(J.prm.tol * (double)(EXACT ? pow_cr(bn, 1.5f) : powf(bn, 1.5f)));
        } else {
            tol = (float)J.prm.tol;
        }
        L.tol = tol * tol_coef;
        // the fast controller's power (tol / (11.09 err))^0.2 as
        // 2^(0.2 log2(tol / 11.09) - 0.1 log2(err^2)): the first term once
        if (!EXACT) L.tol = 0.2f * log2f(L.tol * (float)(1.0 / 11.09));
    }
}

// 2^x and log2 x by the hardware approximations (ex2/lg2.approx.ftz.f32):
// the fast step controller only needs the next step size to a few digits.
__device__ __forceinline__ float ex2_approx(float x) {
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float lg2_approx(float x) {
    float r;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// a - b on the packed f32x2 pipe
__device__ __forceinline__ float2 fsub2(float2 a, float2 b) {
    float2 d;
    asm("{\n\t"
        ".reg .b64 ra, rb, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\t"
        "mov.b64 rb, {%4, %5};\n\t"
        "sub.rn.f32x2 rd, ra, rb;\n\t"
        "mov.b64 {%0, %1}, rd;\n\t"
        "}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}

// The limits checked before a trial step: true (direction finished, L.out
// and L.flag set) when the length or step limit stops it.
template <bool EXACT, class F>
__device__ __forceinline__ bool lane_limits(const TraceJob<F>& J, Lane<EXACT>& L,
                                            typename Lane<EXACT>::len_t len_lim) {
    const bool more_steps = EXACT ? ((long long)L.steps < J.prm.max_steps) : (L.steps < J.lim.max_steps);
    const bool more_len = L.len < len_lim;
    if (!(more_len & more_steps)) {
        L.out = L.p;
        L.flag = pack_flag(0, more_len ? QSL_LINE_MAX_STEPS : QSL_LINE_MAX_LENGTH);
        return true;
    }
    return false;
}

// the signed step: h with the direction's sign bit (h x +-1 exactly)
template <bool EXACT>
__device__ __forceinline__ float lane_hd(const Lane<EXACT>& L) {
    return __int_as_float(__float_as_int(L.h) ^ (int)L.dsign);
}

// The RKF45 step controller after a trial step with error estimate err (its
// norm in exact arithmetic, h^2 |e|^2 in fast): 0 = accepted (L.h is the
// next step), 1 = rejected (L.h shrunk; try again), 2 = rejected and the
// direction finished by the reject limit.
template <bool EXACT, class F>
__device__ __forceinline__ int lane_control(const TraceJob<F>& J, Lane<EXACT>& L, float err) {
    const qsl_trace_params& pr = J.prm;
    float scale;
    if (EXACT) {
        scale = pow_cr((float)((double)(L.tol / err) / 11.09), 0.2f);
        if ((double)scale < 0.618) {
            L.h = (float)((double)L.h * pr.reject_factor);
            if (pr.max_rejects > 0 && ++L.rej >= pr.max_rejects) {
                L.out = L.p;
                L.flag = pack_flag(0, QSL_LINE_REJECT_LIMIT);
                return 2;
            }
            return 1;
        }
    } else {
        // only the next step size depends on this power: hardware
        // log2 / exp2 are accurate enough (err is h^2 |e|^2 here, L.tol
        // 0.2 log2(tol / 11.09))
        scale = ex2_approx(fmaf(-0.1f, lg2_approx(err), L.tol));
        if (scale < 0.618f) {
            L.h = L.h * J.lim.reject;
            if (pr.max_rejects > 0 && ++L.rej >= pr.max_rejects) {
                L.out = L.p;
                L.flag = pack_flag(0, QSL_LINE_REJECT_LIMIT);
                return 2;
            }
            return 1;
        }
    }
    L.rej = 0;
    float h = L.h * scale;
    if (EXACT) {
        if ((double)h > pr.h_max) h = (float)pr.h_max;
        if ((double)h < pr.h_min) h = (float)pr.h_min;
    } else {
        if (h > J.lim.h_max) h = J.lim.h_max;  // a NaN step stays NaN, as above
        if (h < J.lim.h_min) h = J.lim.h_min;
    }
    L.h = h;
    return 0;
}

template <bool EXACT, bool TWIST, class F>
__device__ __forceinline__ bool lane_move(const F& f, const TraceJob<F>& J, Lane<EXACT>& L, float3 inc,
                                          float3 b_at_p, bool tw_on, unsigned& ns);

// One trial step of the current direction.  Returns true when the direction
// is finished (left the box, or stopped by the length / step limit) with
// L.out, L.flag, L.len, L.tw final.  Reference: TraceBlineAdap,
// TraceBlineAdaptive.cu:361-421 and TraceBline, TraceBline.cu:320-373.
template <bool EXACT, bool TWIST, class F>
__device__ __forceinline__ bool lane_step(const F& f, const TraceJob<F>& J, Lane<EXACT>& L,
                                          typename Lane<EXACT>::len_t len_lim, bool tw_on,
                                          unsigned& ns) {
    if (lane_limits(J, L, len_lim)) return true;
    const float hd = lane_hd(L);
    float3 inc;
    // fast twist kernels: B at L.p comes out of the step's first sample
    float3 b_at_p = v3(0.f, 0.f, 0.f);
    float3* const want_b = (!EXACT && TWIST && tw_on) ? &b_at_p : nullptr;
    if (J.prm.integrator == QSL_RKF45) {
        float err;
        inc = step_rkf45<EXACT>(f, L.p, hd, err, ns, want_b);
        const int c = lane_control(J, L, err);
        if (c != 0) return c == 2;
    } else {
        inc = step_rk4<EXACT>(f, L.p, hd, ns, want_b);
    }
    return lane_move<EXACT, TWIST>(f, J, L, inc, b_at_p, tw_on, ns);
}

// The accepted step's move: the position update (Kahan-compensated in fast
// arithmetic), the length, the twist increment and the exit test with the
// footpoint on the face.  True when the direction is finished.
template <bool EXACT, bool TWIST, class F>
__device__ __forceinline__ bool lane_move(const F& f, const TraceJob<F>& J, Lane<EXACT>& L, float3 inc,
                                          float3 b_at_p, bool tw_on, unsigned& ns) {
    const qsl_trace_params& pr = J.prm;
    // the twist integrand at the step's start point, before the position
    // update (fewer values live during the current density's sample)
    float td = 0.f;
    float3 b1 = v3(0.f, 0.f, 0.f), j1 = v3(0.f, 0.f, 0.f);
    if (TWIST && tw_on) {
        j1 = J.cur_packed ? sample<EXACT>(J.cur_store, L.p, false) : sample<EXACT>(current_view(f, J.cur), L.p, false);
        if (EXACT) {
            b1 = sample<EXACT>(f, L.p, false);
            ns += 2;
        } else {
            b1 = b_at_p;
            ns += 1;
        }
        td = twist_density<EXACT>(j1, b1);
    }
    float3 p2;
    float dl;
    if (EXACT) {
        p2 = L.p + inc;
        dl = norm(L.p - p2);
    } else {
        // Kahan-compensated position update: the rounding lost in p + inc is
        // carried into the next step, so long lines of short steps do not
        // drift by accumulated float rounding.  (x, y) on the packed pipe;
        // t = p2 - p, the increment as applied, also gives the step length.
        const float2 pxy = make_float2(L.p.x, L.p.y);
        const float2 yxy = fsub2(make_float2(inc.x, inc.y), make_float2(L.pc.x, L.pc.y));
        const float yz = inc.z - L.pc.z;
        const float2 qxy = __fadd2_rn(pxy, yxy);
        const float qz = L.p.z + yz;
        const float2 txy = fsub2(qxy, pxy);
        const float tz = qz - L.p.z;
        const float2 cxy = fsub2(txy, yxy);
        L.pc = v3(cxy.x, cxy.y, tz - yz);
        p2 = v3(qxy.x, qxy.y, qz);
        dl = norm_fast(v3(txy.x, txy.y, tz));
    }
    len_add(L, (double)dl, dl);
    if (TWIST && tw_on)
        L.tw = L.tw + (EXACT ? (double)td / 4.0 / kRefPi * (double)dl : (double)(td * dl * kInv4PiF));
    // inside test first: the full face classification only runs on exit
    const int flag = box_inside(f, p2) ? 0 : box_exit(f, p2);
    if (flag > 0) {
        len_add(L, -(double)dl, -dl);
        if (TWIST && tw_on)
            L.tw = L.tw - (EXACT ? (double)td / 4.0 / kRefPi * (double)dl : (double)(td * dl * kInv4PiF));
        if (flag <= 6) {
            const int d = (flag - 1) / 2;
            const float q1 = comp(L.p, d), q2 = comp(p2, d);
            float qmid = q1;
            if ((double)fabsf(q1 - q2) > 1e-3) {
                qmid = (flag % 2 == 1) ? 0.f : (float)f.d.n(d);
                const float3 u1 = sample<EXACT>(f, L.p, true);
                const float3 u2 = sample<EXACT>(f, p2, true);
                ns += 2;
                if (((double)fabsf(comp(u1, d)) < 0.2) | ((double)fabsf(comp(u2, d)) < 0.2)) {
                    L.out.x = (L.p.x * (q2 - qmid) + p2.x * (qmid - q1)) / (q2 - q1);
                    L.out.y = (L.p.y * (q2 - qmid) + p2.y * (qmid - q1)) / (q2 - q1);
                    L.out.z = (L.p.z * (q2 - qmid) + p2.z * (qmid - q1)) / (q2 - q1);
                } else {
                    if constexpr (RolledStages<F>::value) L.out = step_rk4_normal_rolled<EXACT>(f, L.p, qmid - q1, d);
                    else L.out = step_rk4_normal<EXACT>(f, L.p, qmid - q1, d);
                    ns += 4;
                }
                len_add(L, (double)fabsf(qmid - q1) / (1e-4 + (double)fabsf(comp(u1, d))),
                        fabsf(qmid - q1) / (1e-4f + fabsf(comp(u1, d))));
                b1 = u1;
            } else {
                L.out = L.p;
            }
            if (TWIST && tw_on && pr.boundary_twist) {
                L.tw = L.tw + (double)twist_density<EXACT>(j1, b1) / 4.0 / kRefPi * (double)fabsf(qmid - q1) /
                                  (1e-4 + (double)fabsf(comp(b1, d)));
            }
        } else {
            L.out = p2;
        }
        const bool finite = isfinite(p2.x) & isfinite(p2.y) & isfinite(p2.z);
        L.flag = pack_flag(flag, flag <= 6 ? QSL_LINE_FACE : (finite ? QSL_LINE_EDGE : QSL_LINE_NAN));
        L.p = p2;
        L.steps++;
        return true;
    }
    L.p = p2;
    L.steps++;
    return false;
}

// A finished direction's outputs, as the reference writes them
// (TraceBlineAdaptive.cu:466-501): after the forward direction its end
// footpoint, flag, B and length, then the backward direction begins (returns
// true); after the backward one the start footpoint, B at the seed and
// B_flag (returns false: the line is done).  The per-line scalars come from
// functors so that they are re-read rather than held in registers.
template <bool EXACT, bool TWIST, class F, class SL, class TC, class NR>
__device__ __forceinline__ bool lane_finish(const F& f, const TraceJob<F>& J, Lane<EXACT>& L, bool tw_on,
                                            unsigned& ns, const SL& s_len_of, const TC& tol_coef_of,
                                            const NR& nrm_of) {
    const long long i = L.line;
    const TraceOut& o = J.o;
    if (L.dsign == 0) {
        const float3 pe = L.out;
        const float3 be = sample_endpoint<EXACT>(f, pe);
        ns += 1;
        o.end_x[i] = pe.x; o.end_y[i] = pe.y; o.end_z[i] = pe.z;
        o.flag_end[i] = lane_flag(L.flag);
        if (o.status_end) o.status_end[i] = lane_status(L.flag);
        o.bend_x[i] = be.x; o.bend_y[i] = be.y; o.bend_z[i] = be.z;
        o.line_len[i] = (double)L.len;
        if (TWIST && tw_on) o.twist[i] = L.tw;
        lane_begin<EXACT>(f, J, L, i, -1, s_len_of(), tol_coef_of(), nrm_of(), ns);
        return true;
    }
    const float3 ps = L.out;
    const float3 bs = sample_endpoint<EXACT>(f, ps);
    const float3 p0 = v3(__ldg(J.inp_x + i), __ldg(J.inp_y + i), __ldg(J.inp_z + i));
    const float3 b0 = sample_endpoint<EXACT>(f, p0);
    ns += 2;
    o.start_x[i] = ps.x; o.start_y[i] = ps.y; o.start_z[i] = ps.z;
    o.flag_start[i] = lane_flag(L.flag);
    if (o.status_start) o.status_start[i] = lane_status(L.flag);
    o.bstart_x[i] = bs.x; o.bstart_y[i] = bs.y; o.bstart_z[i] = bs.z;
    o.bthis_x[i] = b0.x; o.bthis_y[i] = b0.y; o.bthis_z[i] = b0.z;
    o.line_len[i] = o.line_len[i] + (double)L.len;
    if (TWIST && tw_on) o.twist[i] = o.twist[i] + L.tw;
    // B nearly in the seed plane (TraceBlineAdaptive.cu:498-501)
    const float3 nrm = nrm_of();
    const float bn = b0.x * nrm.x + b0.y * nrm.y + b0.z * nrm.z;
    const float bm = sqrtf(b0.x * b0.x + b0.y * b0.y + b0.z * b0.z);
    o.b_flag[i] = ((double)fabsf(bn) * 100. < (double)bm) ? 1 : 0;
    return false;
}

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// The tracer kernel.  QUEUE = true: persistent grid; each warp takes chunks
// of J.chunk consecutive lines from the device counter J.queue and its lanes
// refill from the warp's current chunk the moment their line ends, so a
// warp's lanes stay on neighbouring seeds (spatially coherent gathers) while
// uneven line lengths never idle them.  QUEUE = false: line = global thread
// index + k * total threads.  Lines are visited in J.order when it is set.
// TWIST compiles the twist integral in; it runs when the runtime flag is set.
template <bool EXACT, bool TWIST, bool QUEUE, class F>
__device__ __forceinline__ void trace_kernel_body(const TraceJob<F>& J) {
    F f = J.f;
    // only the drop-in stores (the caller's arrays) take their shape from the
    // device; the packed stores' dims stay kernel parameters
    if constexpr (std::is_same<F, FieldSoA>::value || std::is_same<F, FieldStretch>::value ||
                  std::is_same<F, FieldStretchU>::value) {
        if (J.shape_dev) {
            f.d.nx = __ldg(J.shape_dev);
            f.d.ny = __ldg(J.shape_dev + 1);
            f.d.nz = __ldg(J.shape_dev + 2);
        }
    }
    // a grid needs two nodes per axis for a trilinear cell (uniform exit)
    if (f.d.nx < 2 || f.d.ny < 2 || f.d.nz < 2) return;
    // Loop invariants that are used once per line are re-read at each use
    // (kernel parameters or one cached load) rather than held in registers:
    // registers set how many blocks stay resident, and the gathers need
    // every resident warp to hide their latency.
    auto s_len_of = [&J]() { return J.s.s_len_dev ? __ldg(J.s.s_len_dev) : J.s.s_len; };
    auto tol_coef_of = [&J]() { return J.s.tol_coef_dev ? __ldg(J.s.tol_coef_dev) : J.s.tol_coef; };
    auto nrm_of = [&J]() {
        return J.s.cross_dev ? v3(__ldg(J.s.cross_dev), __ldg(J.s.cross_dev + 1), __ldg(J.s.cross_dev + 2))
                             : v3(J.s.cross[0], J.s.cross[1], J.s.cross[2]);
    };
    long long n = J.s.n_dev ? (long long)__ldg(J.s.n_dev) : J.s.n;
    if (J.s.n_cap >= 0 && n > J.s.n_cap) n = J.s.n_cap;
    const bool tw_on = TWIST && (J.s.twist_flag_dev ? *J.s.twist_flag_dev : (J.s.twist_on != 0));
    if (!store_active(f)) return;
    store_prepare(f);
    // the packed stores' dims (and the stretched stores' coordinate
    // extents) are known on the host: their length limit is a kernel
    // parameter (a register would be re-formed from the double
    // product at every step once the loop runs short of registers)
    typename Lane<EXACT>::len_t len_lim;
    if constexpr (!EXACT && (std::is_same<F, FieldH4B>::value || std::is_same<F, FieldH4BW>::value ||
                             std::is_same<F, FieldF4>::value || std::is_same<F, FieldH8C>::value ||
                             std::is_same<F, FieldStretchP>::value || std::is_same<F, FieldStretchPU>::value))
        len_lim = J.lim.len_lim;
    else
        len_lim = (typename Lane<EXACT>::len_t)(J.prm.len_ratio * len_scale(f));
    unsigned ns = 0;
    const int lane_id = threadIdx.x & 31;

    Lane<EXACT> L;
    bool active = false;
    bool drained = false;
    // warp-uniform chunk window [c_next, c_end) of the work queue
    long long c_next = 0, c_end = 0;
    bool q_empty = false;
    const long long chunk = J.chunk > 0 ? J.chunk : 256;
    long long next_static = (long long)blockIdx.x * blockDim.x + threadIdx.x;

    while (true) {
        // ---- give lanes without a line the next ones ----
        if (QUEUE) {
            bool need = !active && !drained;
            unsigned m = __ballot_sync(0xffffffffu, need);
            while (m) {
                if (c_next >= c_end) {
                    if (q_empty) {
                        drained = drained || need;
                        break;
                    }
                    unsigned long long base = 0;
                    if (lane_id == 0) base = atomicAdd(J.queue, (unsigned long long)chunk);
                    base = __shfl_sync(0xffffffffu, base, 0);
                    if ((long long)base >= n) {
                        q_empty = true;
                        drained = drained || need;
                        break;
                    }
                    c_next = (long long)base;
                    c_end = min((long long)base + chunk, n);
                }
                const long long avail = c_end - c_next;
                const int take = (int)min((long long)__popc(m), avail);
                const int rank = __popc(m & lanemask_lt());
                if (need && rank < take) {
                    const long long line = c_next + rank;
                    const long long sidx = J.order ? (long long)__ldg(J.order + line) : line;
                    lane_begin<EXACT>(f, J, L, sidx, +1, s_len_of(), tol_coef_of(), nrm_of(), ns);
                    active = true;
                    need = false;
                }
                c_next += take;
                m = __ballot_sync(0xffffffffu, need);
            }
            if (!__any_sync(0xffffffffu, active)) break;
            if (!active) continue;
        } else {
            if (!active) {
                if (next_static >= n) break;
                const long long sidx = J.order ? (long long)__ldg(J.order + next_static) : next_static;
                lane_begin<EXACT>(f, J, L, sidx, +1, s_len_of(), tol_coef_of(), nrm_of(), ns);
                next_static += (long long)gridDim.x * blockDim.x;
                active = true;
            }
        }

        // ---- advance this lane's line by one trial step ----
        if (lane_step<EXACT, TWIST>(f, J, L, len_lim, tw_on, ns)) {
            // a lane's sample count nears 32 bits: hand it over (checked at
            // direction ends only; exact while one direction takes fewer than
            // 5e8 trial steps)
            if (ns > (1u << 30)) {
                if (J.samples) atomicAdd(J.samples, (unsigned long long)ns);
                ns = 0;
            }
            active = lane_finish<EXACT, TWIST>(f, J, L, tw_on, ns, s_len_of, tol_coef_of, nrm_of);
        }
    }
    if (J.samples) {
        // one atomic per warp (blocks are whole warps; every lane gets here)
        __syncwarp();
        unsigned long long v = ns;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane_id == 0) atomicAdd(J.samples, v);
    }
}

}  // namespace qsl
