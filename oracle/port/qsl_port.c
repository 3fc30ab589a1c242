/*
 * CPU ORACLE (test infrastructure, not part of the fastqsl_gb300 product).
 *
 * A restatement in C of the reference's field-line tracer and Scott
 * deviation-vector tracer (peijin94/FastQSL, fastqslpy/cu/TraceBline.cu,
 * TraceBlineAdaptive.cu, TraceBlineScott.cu) and of the stretched-grid
 * tracer (TraceBlineAdaptiveStretch.cu).  Compiled three times:
 *
 *   QO_REAL=float  (prefix qo32_): reference-parity arithmetic.  Every
 *       expression rounds where the reference's does: FP32 state, corner
 *       weights evaluated in FP64 then stored to FP32, FP64 line length, the
 *       double literals of the step controller.  Built with
 *       -ffp-contract=off it reproduces the reference's host build bit for
 *       bit (checked by the tests against oracle/_ref).  With
 *       params->tol_law / h_min / h_max / ... set to non-reference values it
 *       is also the CPU baseline for the benchmark settings.
 *   QO_REAL=float, QO_CRPOW=1 (prefix qo32cr_): the same with a correctly
 *       rounded power function, the rounding of the GPU's exact kernels;
 *   QO_REAL=double (prefix qo64_): the FP64 oracle — the same algorithm with
 *       every quantity in double, used to state the error of each GPU form.
 *
 * Deliberate, documented departures from the reference:
 *   - a direction stopped by the step or length limit (flag 0) reports the
 *     last point reached; the reference reports whatever its per-thread
 *     scratch buffer held (TraceBlineAdaptive.cu:448-452, P_out is written only
 *     on exit, :380-418);
 *   - the RK4 exit-segment twist term uses p_mid = p1 (term 0) when the exit
 *     step is shorter than 1e-3 in the normal coordinate; the reference reads
 *     p_mid uninitialised there (TraceBline.cu:343-365);
 *   - the Scott tracer uses tol = 1e-3*tol_coef; the reference reads its
 *     tolerance uninitialised (TraceBlineScott.cu:352,378), and its line
 *     length uses B at the previous exit point only when twist is on (:448);
 *     here the exit-segment length term uses the unit field at the last
 *     inside point.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "fastqsl_gb300.h"

#ifndef QO_REAL
#define QO_REAL float
#endif
typedef QO_REAL R;

#if QO_DOUBLE
#define PFX(n) qo64_##n
#define RSQRT_(x) sqrt(x)
#define RFLOOR(x) floor(x)
#define RFABS(x) fabs(x)
#define RPOW(x, y) pow((x), (y))
#elif QO_CRPOW
/* FP32 parity arithmetic with a correctly rounded power (the double-precision
 * pow narrowed to float), the rounding the GPU's exact kernels use.  glibc's
 * powf (what the reference's host build calls) misses correct rounding in
 * ~6e-4 of calls; on the reference's loose tolerance that flips some
 * accept/reject decisions. */
#define PFX(n) qo32cr_##n
#define RSQRT_(x) sqrtf(x)
#define RFLOOR(x) floorf(x)
#define RFABS(x) fabsf(x)
#define RPOW(x, y) ((float)pow((double)(x), (double)(y)))
#else
#define PFX(n) qo32_##n
#define RSQRT_(x) sqrtf(x)
#define RFLOOR(x) floorf(x)
#define RFABS(x) fabsf(x)
#define RPOW(x, y) powf((x), (y))
#endif

#define QO_API __attribute__((visibility("default")))

/* The reference redefines M_PI to this 9-digit value (TraceBlineAdaptive.cu:10). */
static const double kRefPi = 3.14159265;

typedef struct { R x, y, z; } v3;
typedef struct { v3 p, u, v; } v9; /* position and two deviation vectors */

static inline v3 mk3(R x, R y, R z) { v3 r = {x, y, z}; return r; }
static inline v3 add3(v3 a, v3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub3(v3 a, v3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 mul3(R s, v3 a) { return mk3(s * a.x, s * a.y, s * a.z); }
static inline v3 div3(v3 a, R s) { return mk3(a.x / s, a.y / s, a.z / s); }
static inline R dot3(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline R norm3(v3 a) { return RSQRT_(a.x * a.x + a.y * a.y + a.z * a.z); }
static inline R comp3(v3 a, int d) { return d == 0 ? a.x : (d == 1 ? a.y : a.z); }

static inline v9 add9(v9 a, v9 b) { v9 r = {add3(a.p, b.p), add3(a.u, b.u), add3(a.v, b.v)}; return r; }
static inline v9 mul9(R s, v9 a) { v9 r = {mul3(s, a.p), mul3(s, a.u), mul3(s, a.v)}; return r; }
static inline v9 div9(v9 a, R s) { v9 r = {div3(a.p, s), div3(a.u, s), div3(a.v, s)}; return r; }

typedef struct {
    const float *bx, *by, *bz;
    int n[3];
    int64_t samples; /* trilinear vector samples taken (for the roofline count) */
    /* stretched grid (TraceBlineAdaptiveStretch.cu): node coordinates per
     * axis, NULL for the integer grid; uni selects the uniform-spacing index
     * formula instead of the search */
    const float *ax[3];
    int uni;
} fld;

/* Floor to int with the device conversion's edge behaviour: NaN -> 0,
 * saturation outside the int range. */
static inline int floor_int(R x)
{
    if (x != x) return 0;
    if (x >= (R)2147483647.0) return 2147483647;
    if (x <= (R)-2147483648.0) return -2147483647 - 1;
    return (int)RFLOOR(x);
}

static inline int64_t node(const int n[3], int i, int j, int k)
{
    return (int64_t)i + (int64_t)n[0] * ((int64_t)j + (int64_t)n[1] * (int64_t)k);
}

/* Stretched grid: cell index of coordinate c on the node coordinates a[n].
 * The reference's search (GetIndexBiSearch, TraceBlineAdaptiveStretch.cu:
 * 42-64) narrows [i0, i1] by halving while the interval spans more than 3
 * nodes, then takes mid or mid - 1 on one comparison; for a point in the upper
 * part of the last interval that is the cell below the point's (the fraction
 * then exceeds 1 and the sample extrapolates).  Restated as is. */
static int stretch_bisect(R c, int n, const float *a)
{
    int i0 = 0, i1 = n - 1, mid = n / 2;
    while (i1 - i0 > 3) {
        if (c > a[mid]) i0 = mid;
        else i1 = mid;
        mid = (i0 + i1) / 2;
    }
    int r = (c > a[mid]) ? mid : mid - 1;
    if (r > n - 2) r = n - 2;
    return r;
}

/* Uniform-spacing formula (GetIndexUniStretch, :67-74): the spacing is taken
 * as (a[n-1] - a[0]) / n (the node count, not n - 1), restated as is. */
static int stretch_uni(R c, int n, const float *a)
{
    int r = floor_int((c - a[0]) / ((a[n - 1] - a[0]) / (R)n));
    if (r < 0) r = 0;
    if (r > n - 2) r = n - 2;
    return r;
}

/* Stretched-grid cell and fraction of coordinate c along axis d: c clamped to
 * (a[0] + 1e-6, a[n-1] - 1e-6) (the offsets applied in double and narrowed),
 * then the index and r = (c - a[i]) / (a[i+1] - a[i]).
 * Reference: Interp3dxyzn, TraceBlineAdaptiveStretch.cu:100-122. */
static void stretch_locate(const fld *f, int d, R c, int *ix, R *fr)
{
    const float *a = f->ax[d];
    const int n = f->n[d];
    c = (c > a[0]) ? c : (R)((double)a[0] + 1e-6);
    c = (c < a[n - 1]) ? c : (R)((double)a[n - 1] - 1e-6);
    const int i = f->uni ? stretch_uni(c, n, a) : stretch_bisect(c, n, a);
    *ix = i;
    *fr = (c - a[i]) / ((R)a[i + 1] - a[i]);
}

/* Trilinear B (optionally unit b = B/|B|) at p; a coordinate at or beyond a
 * face is pinned to that face's cell with fraction 0 or 1.
 * Reference: Interp3dxyzn, TraceBlineAdaptive.cu:95-201 (integer grid) and
 * TraceBlineAdaptiveStretch.cu:82-201 (stretched grid: stretch_locate). */
static v3 sample_b(fld *f, v3 p, int unit)
{
    const int *n = f->n;
    R fr[3], c[3] = {p.x, p.y, p.z};
    int ix[3];
    for (int d = 0; d < 3; ++d) {
        if (f->ax[0]) {
            stretch_locate(f, d, c[d], &ix[d], &fr[d]);
            continue;
        }
        fr[d] = c[d] - RFLOOR(c[d]);
        ix[d] = floor_int(c[d]);
        if (c[d] <= 0.) { fr[d] = 0; ix[d] = 0; }
        if (c[d] >= n[d] - 1) { fr[d] = 1; ix[d] = n[d] - 2; }
    }
    /* Corner weights.  The reference forms (1.-r) in double, multiplies left
     * to right and stores to float; the two products of bare fractions
     * (rx*ry) are float products. */
    const R rx = fr[0], ry = fr[1], rz = fr[2];
    const double ox = 1. - rx, oy = 1. - ry, oz = 1. - rz;
    R w[8];
    w[0] = (R)(ox * oy * oz);
    w[1] = (R)(ox * oy * rz);
    w[2] = (R)(ox * ry * oz);
    w[3] = (R)(ox * ry * rz);
    w[4] = (R)(rx * oy * oz);
    w[5] = (R)(rx * oy * rz);
    w[6] = (R)((R)(rx * ry) * oz);
    w[7] = (R)((R)(rx * ry) * rz);
    /* corner order 000,001,010,011,100,101,110,111 = (dx,dy,dz) bits */
    int64_t idx[8];
    for (int q = 0; q < 8; ++q)
        idx[q] = node(n, ix[0] + ((q >> 2) & 1), ix[1] + ((q >> 1) & 1), ix[2] + (q & 1));
    const float *arr[3] = {f->bx, f->by, f->bz};
    R out[3];
    for (int m = 0; m < 3; ++m) {
        R acc = (R)arr[m][idx[0]] * w[0];
        for (int q = 1; q < 8; ++q) acc = acc + (R)arr[m][idx[q]] * w[q];
        out[m] = acc;
    }
    f->samples++;
    v3 r = mk3(out[0], out[1], out[2]);
    if (unit) {
        R nb = norm3(r);
        r = mk3(r.x / nb, r.y / nb, r.z / nb);
    }
    return r;
}

/* One field component at p, position clamped into [1e-4, n-1-1e-4].
 * Reference: Interp3d, TraceBlineAdaptive.cu:47-93. */
static R sample_scalar(const float *A, const int n[3], R x, R y, R z)
{
    R c[3] = {x, y, z};
    for (int d = 0; d < 3; ++d) {
        c[d] = (c[d] > 0) ? c[d] : (R)0.0001;
        c[d] = (c[d] < (R)(n[d] - 1)) ? c[d] : (R)((double)((R)n[d] - 1) - 0.0001);
    }
    R fr[3];
    int ix[3];
    for (int d = 0; d < 3; ++d) {
        fr[d] = c[d] - RFLOOR(c[d]);
        ix[d] = floor_int(c[d]);
    }
    const R rx = fr[0], ry = fr[1], rz = fr[2];
    const double ox = 1. - rx, oy = 1. - ry, oz = 1. - rz;
    R a[8];
    for (int q = 0; q < 8; ++q)
        a[q] = (R)A[node(n, ix[0] + ((q >> 2) & 1), ix[1] + ((q >> 1) & 1), ix[2] + (q & 1))];
    /* Each term multiplies the corner value by the three factors left to
     * right; factors that are bare float fractions stay float products until
     * a double factor appears. */
    double s = a[0] * ox * oy * oz;
    s = s + a[1] * ox * oy * rz;
    s = s + a[2] * ox * ry * oz;
    s = s + a[3] * ox * ry * rz;
    s = s + (R)(a[4] * rx) * oy * oz;
    s = s + (R)(a[5] * rx) * oy * rz;
    s = s + (R)((R)(a[6] * rx) * ry) * oz;
    s = s + (R)((R)((R)(a[7] * rx) * ry) * rz);
    return (R)s;
}

/* Reference: checkFlag, TraceBlineAdaptive.cu:309-331.  Inside needs y > 0
 * strictly (x and z allow 0); a face flag needs the other two coordinates
 * strictly below their maxima. */
static int box_flag(const int n[3], v3 p)
{
    const double X = n[0] - 1., Y = n[1] - 1., Z = n[2] - 1.;
    if ((p.x >= 0.) & (p.y > 0.) & (p.z >= 0.) & (p.x <= X) & (p.y <= Y) & (p.z <= Z)) return 0;
    int f = 42;
    if ((p.x < 0.) & (p.y >= 0.) & (p.z >= 0.) & (p.x < X) & (p.y < Y) & (p.z < Z)) f = 1;
    if ((p.x >= 0.) & (p.y >= 0.) & (p.z >= 0.) & (p.x >= X) & (p.y < Y) & (p.z < Z)) f = 2;
    if ((p.x >= 0.) & (p.y < 0.) & (p.z >= 0.) & (p.x < X) & (p.y < Y) & (p.z < Z)) f = 3;
    if ((p.x >= 0.) & (p.y >= 0.) & (p.z >= 0.) & (p.x < X) & (p.y >= Y) & (p.z < Z)) f = 4;
    if ((p.x >= 0.) & (p.y >= 0.) & (p.z < 0.) & (p.x < X) & (p.y < Y) & (p.z < Z)) f = 5;
    if ((p.x >= 0.) & (p.y >= 0.) & (p.z >= 0.) & (p.x < X) & (p.y < Y) & (p.z >= Z)) f = 6;
    return f;
}

/* checkFlag on the stretched grid (TraceBlineAdaptiveStretch.cu:309-331):
 * the same tests against the first and last node coordinates. */
static int box_flag_stretch(const fld *f, v3 p)
{
    const float *a = f->ax[0], *b = f->ax[1], *c = f->ax[2];
    const R x0 = a[0], y0 = b[0], z0 = c[0];
    const R X = a[f->n[0] - 1], Y = b[f->n[1] - 1], Z = c[f->n[2] - 1];
    if ((p.x >= x0) & (p.y > y0) & (p.z >= z0) & (p.x <= X) & (p.y <= Y) & (p.z <= Z)) return 0;
    int r = 42;
    if ((p.x < x0) & (p.y >= y0) & (p.z >= z0) & (p.x < X) & (p.y < Y) & (p.z < Z)) r = 1;
    if ((p.x >= x0) & (p.y >= y0) & (p.z >= z0) & (p.x >= X) & (p.y < Y) & (p.z < Z)) r = 2;
    if ((p.x >= x0) & (p.y < y0) & (p.z >= z0) & (p.x < X) & (p.y < Y) & (p.z < Z)) r = 3;
    if ((p.x >= x0) & (p.y >= y0) & (p.z >= z0) & (p.x < X) & (p.y >= Y) & (p.z < Z)) r = 4;
    if ((p.x >= x0) & (p.y >= y0) & (p.z < z0) & (p.x < X) & (p.y < Y) & (p.z < Z)) r = 5;
    if ((p.x >= x0) & (p.y >= y0) & (p.z >= z0) & (p.x < X) & (p.y < Y) & (p.z >= Z)) r = 6;
    return r;
}

static inline int exit_flag(const fld *f, v3 p) { return f->ax[0] ? box_flag_stretch(f, p) : box_flag(f->n, p); }

/* Length limit: len_ratio x (nx + ny + nz) on the integer grid; on the
 * stretched grid len_ratio x the summed coordinate extents
 * (TraceBlineAdaptiveStretch.cu:337-339, evaluated in float). */
static double len_limit(const fld *f, double ratio)
{
    if (!f->ax[0]) return ratio * (double)(f->n[0] + f->n[1] + f->n[2]);
    const R hi = (R)((R)f->ax[0][f->n[0] - 1] + f->ax[1][f->n[1] - 1]) + f->ax[2][f->n[2] - 1];
    const R lo = (R)((R)f->ax[0][0] + f->ax[1][0]) + f->ax[2][0];
    return ratio * (double)(R)(hi - lo);
}

/* Classic RK4 on the unit field.  Reference: RK4, TraceBlineAdaptive.cu:259-267.
 * `(1./6.)*h` is formed in double and narrowed before scaling the sum. */
static v3 step_rk4(fld *f, v3 p, R h)
{
    v3 k1 = sample_b(f, p, 1);
    v3 k2 = sample_b(f, add3(p, div3(mul3(h, k1), (R)2.)), 1);
    v3 k3 = sample_b(f, add3(p, div3(mul3(h, k2), (R)2.)), 1);
    v3 k4 = sample_b(f, add3(p, mul3(h, k3)), 1);
    v3 s = add3(add3(add3(k1, mul3((R)2., k2)), mul3((R)2., k3)), k4);
    return add3(p, mul3((R)(1. / 6. * h), s));
}

/* RK4 in the face-normal coordinate: dx/dp = b/b_d over dp = h.
 * Reference: RK4_boundary, TraceBlineAdaptive.cu:286-307. */
static v3 step_rk4_normal(fld *f, v3 p, R h, int d)
{
    v3 b1 = sample_b(f, p, 1);
    v3 k1 = div3(b1, comp3(b1, d));
    v3 b2 = sample_b(f, add3(p, div3(mul3(h, k1), (R)2.)), 1);
    v3 k2 = div3(b2, comp3(b2, d));
    v3 b3 = sample_b(f, add3(p, div3(mul3(h, k2), (R)2.)), 1);
    v3 k3 = div3(b3, comp3(b3, d));
    v3 b4 = sample_b(f, add3(p, mul3(h, k3)), 1);
    v3 k4 = div3(b4, comp3(b4, d));
    v3 s = add3(add3(add3(k1, mul3((R)2., k2)), mul3((R)2., k3)), k4);
    return add3(p, mul3((R)(1. / 6. * h), s));
}

/* Fehlberg 4(5) tableau (coefficients narrowed to the working type as the
 * reference stores them in float variables, TraceBlineAdaptive.cu:224-235). */
typedef struct {
    R a21, a31, a32, a41, a42, a43, a51, a52, a53, a54, a61, a62, a63, a64, a65;
    R b1, b3, b4, b5, b6, e1, e3, e4, e5, e6;
} fehlberg_t;

static fehlberg_t fehlberg(void)
{
    fehlberg_t c;
    c.a21 = (R)(1. / 4.);
    c.a31 = (R)(3. / 32.); c.a32 = (R)(9. / 32.);
    c.a41 = (R)(1932. / 2197.); c.a42 = (R)(-7200. / 2197.); c.a43 = (R)(7296. / 2197.);
    c.a51 = (R)(439. / 216.); c.a52 = (R)(-8.); c.a53 = (R)(3680. / 513.); c.a54 = (R)(-845. / 4104.);
    c.a61 = (R)(-8. / 27.); c.a62 = (R)(2.); c.a63 = (R)(-3544. / 2565.); c.a64 = (R)(1859. / 4104.);
    c.a65 = (R)(-11. / 40.);
    c.b1 = (R)(16. / 135.); c.b3 = (R)(6656. / 12825.); c.b4 = (R)(28561. / 56430.);
    c.b5 = (R)(-9. / 50.); c.b6 = (R)(2. / 55.);
    c.e1 = (R)(1. / 360.); c.e3 = (R)(-128. / 4275.); c.e4 = (R)(-2197. / 75240.);
    c.e5 = (R)(1. / 50.); c.e6 = (R)(2. / 55.);
    return c;
}

/* One Fehlberg step of size h; returns the 5th-order point and the norm of
 * the embedded error estimate.  Reference: RKF45, TraceBlineAdaptive.cu:215-254. */
static v3 step_rkf45(fld *f, v3 p, R h, R *err)
{
    const fehlberg_t c = fehlberg();
    v3 k1 = mul3(h, sample_b(f, p, 1));
    v3 k2 = mul3(h, sample_b(f, add3(p, mul3(c.a21, k1)), 1));
    v3 k3 = mul3(h, sample_b(f, add3(p, add3(mul3(c.a31, k1), mul3(c.a32, k2))), 1));
    v3 s4 = add3(add3(mul3(c.a41, k1), mul3(c.a42, k2)), mul3(c.a43, k3));
    v3 k4 = mul3(h, sample_b(f, add3(p, s4), 1));
    v3 s5 = add3(add3(add3(mul3(c.a51, k1), mul3(c.a52, k2)), mul3(c.a53, k3)), mul3(c.a54, k4));
    v3 k5 = mul3(h, sample_b(f, add3(p, s5), 1));
    v3 s6 = add3(add3(add3(add3(mul3(c.a61, k1), mul3(c.a62, k2)), mul3(c.a63, k3)), mul3(c.a64, k4)),
                 mul3(c.a65, k5));
    v3 k6 = mul3(h, sample_b(f, add3(p, s6), 1));
    v3 hi = add3(add3(add3(add3(mul3(c.b1, k1), mul3(c.b3, k3)), mul3(c.b4, k4)), mul3(c.b5, k5)), mul3(c.b6, k6));
    v3 er = add3(add3(add3(add3(mul3(c.e1, k1), mul3(c.e3, k3)), mul3(c.e4, k4)), mul3(c.e5, k5)), mul3(c.e6, k6));
    *err = norm3(er);
    return add3(p, hi);
}

static inline R twist_density(fld *f, fld *cur, v3 p, v3 *b_out, v3 *j_out)
{
    v3 j = sample_b(cur, p, 0);
    v3 b = sample_b(f, p, 0);
    *b_out = b;
    *j_out = j;
    return dot3(j, b) / dot3(b, b);
}

typedef struct {
    v3 end;
    int flag;
    double len;
    double twist;
} dir_result;

/* Traces one direction (dir = +1 along b, -1 against) from p0 until the
 * line leaves the box or a limit stops it.  Reference: TraceBlineAdap,
 * TraceBlineAdaptive.cu:333-426 (RKF45) and TraceBline, TraceBline.cu:300-378
 * (RK4). */
static dir_result trace_direction(fld *f, fld *cur, int twist_on, const qsl_trace_params *pr, v3 p0, v3 nrm,
                                  R h, R dir, R tol_coef)
{
    const int *n = f->n;
    const double len_lim = len_limit(f, pr->len_ratio);
    const int rkf = pr->integrator == QSL_RKF45;
    dir_result res;
    v3 p1 = p0, out = p0;
    v3 j1 = mk3(0, 0, 0), b1 = mk3(0, 0, 0);
    double len = 0, tw = 0;
    int64_t steps = 0;
    int flag = 0;
    R tol = 0;

    v3 bstart = sample_b(f, p1, 1);
    if (rkf) {
        R bn = RFABS(dot3(bstart, nrm));
        if (pr->tol_law == QSL_TOL_REFERENCE) {
            if (bn <= 0.05) tol = (R)(pr->tol / 8e3);
            else tol = (R)(pr->tol * RPOW(bn, (R)1.5));
        } else {
            tol = (R)pr->tol;
        }
        tol = tol * tol_coef;
    }

    int rej = 0; /* trial steps rejected in a row (max_rejects > 0 ends the direction there) */
    while ((flag == 0) & (len < len_lim) & (steps < pr->max_steps)) {
        v3 p2;
        if (rkf) {
            R err;
            p2 = step_rkf45(f, p1, h * dir, &err);
            R scale = RPOW((R)((tol / err) / 11.09), (R)0.2);
            if (scale < 0.618) {
                h = (R)(h * pr->reject_factor);
                if (pr->max_rejects > 0 && ++rej >= pr->max_rejects) break;
                continue;
            }
            rej = 0;
            h = h * scale;
            if (h > pr->h_max) h = (R)pr->h_max;
            if (h < pr->h_min) h = (R)pr->h_min;
        } else {
            p2 = step_rk4(f, p1, h * dir);
        }
        const R dl = norm3(sub3(p1, p2));
        len = len + dl;
        R td = 0;
        if (twist_on) {
            td = twist_density(f, cur, p1, &b1, &j1);
            tw = tw + td / 4.0 / kRefPi * dl;
        }
        flag = exit_flag(f, p2);
        if (flag > 0) {
            len = len - dl;
            if (twist_on) tw = tw - td / 4.0 / kRefPi * dl;
            if (flag <= 6) {
                const int d = (flag - 1) / 2;
                const R q1 = comp3(p1, d), q2 = comp3(p2, d);
                R qmid = q1;
                if (RFABS(q1 - q2) > 1e-3) {
                    qmid = (flag % 2 == 1) ? (R)0 : (R)n[d];
                    v3 u1 = sample_b(f, p1, 1);
                    v3 u2 = sample_b(f, p2, 1);
                    if ((RFABS(comp3(u1, d)) < 0.2) | (RFABS(comp3(u2, d)) < 0.2)) {
                        out.x = (p1.x * (q2 - qmid) + p2.x * (qmid - q1)) / (q2 - q1);
                        out.y = (p1.y * (q2 - qmid) + p2.y * (qmid - q1)) / (q2 - q1);
                        out.z = (p1.z * (q2 - qmid) + p2.z * (qmid - q1)) / (q2 - q1);
                    } else {
                        out = step_rk4_normal(f, p1, qmid - q1, d);
                    }
                    len = len + RFABS(qmid - q1) / (1e-4 + RFABS(comp3(u1, d)));
                    b1 = u1;
                } else {
                    out = p1;
                }
                if (twist_on && pr->boundary_twist) {
                    tw = tw + dot3(j1, b1) / dot3(b1, b1) / 4.0 / kRefPi * RFABS(qmid - q1) /
                                  (1e-4 + RFABS(comp3(b1, d)));
                }
            } else {
                out = p2;
            }
        }
        p1 = p2;
        steps = steps + 1;
    }
    if (flag == 0) out = p1;
    res.end = out;
    res.flag = flag;
    res.len = len;
    res.twist = tw;
    return res;
}

/* B at an endpoint or at the seed: the clamped scalar interpolator per
 * component on the integer grid (TraceBlineAdaptive.cu:466-509), the vector
 * interpolator on the stretched grid (TraceBlineAdaptiveStretch.cu:466-499). */
static v3 sample_end(fld *f, v3 p)
{
    if (f->ax[0]) {
        const int64_t s0 = f->samples;
        v3 r = sample_b(f, p, 0);
        f->samples = s0;
        return r;
    }
    return mk3(sample_scalar(f->bx, f->n, p.x, p.y, p.z), sample_scalar(f->by, f->n, p.x, p.y, p.z),
               sample_scalar(f->bz, f->n, p.x, p.y, p.z));
}

/* The whole per-seed job of TraceAllBline (TraceBlineAdaptive.cu:429-510,
 * TraceBlineAdaptiveStretch.cu:422-508): forward trace -> end footpoint,
 * backward -> start footpoint, B at both footpoints and at the seed, B_flag
 * (field within ~0.57 deg of the seed plane), line length and twist summed
 * over both directions.  ax (NULL: integer grid) and uni describe a
 * stretched grid. */
static int trace_seeds(const float *Bx, const float *By, const float *Bz, const int *shape,
                       const float *const ax[3], int uni,
                       const float *cBx, const float *cBy, const float *cBz, double *twist, int twist_on,
                       const float *inp_x, const float *inp_y, const float *inp_z, const float *cross_dir,
                       float *start_x, float *start_y, float *start_z, int *flag_start,
                       float *end_x, float *end_y, float *end_z, int *flag_end,
                       float *B_this_x, float *B_this_y, float *B_this_z, int *B_flag,
                       float *B_start_x, float *B_start_y, float *B_start_z,
                       float *B_end_x, float *B_end_y, float *B_end_z,
                       float s_len, int64_t n_seeds, double *LineLen, float tol_coef,
                       const qsl_trace_params *pr, int64_t *samples_out)
{
    if (!Bx || !By || !Bz || !shape || !pr) return QSL_ERR_INVALID;
    if (shape[0] < 2 || shape[1] < 2 || shape[2] < 2) return QSL_ERR_INVALID;
    if (twist_on && (!cBx || !cBy || !cBz || !twist)) return QSL_ERR_INVALID;
    int64_t total = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : total)
    for (int64_t i = 0; i < n_seeds; ++i) {
        fld f = {Bx, By, Bz, {shape[0], shape[1], shape[2]}, 0, {ax[0], ax[1], ax[2]}, uni};
        fld cur = {cBx, cBy, cBz, {shape[0], shape[1], shape[2]}, 0, {ax[0], ax[1], ax[2]}, uni};
        const v3 p0 = mk3((R)inp_x[i], (R)inp_y[i], (R)inp_z[i]);
        const v3 nrm = mk3((R)cross_dir[0], (R)cross_dir[1], (R)cross_dir[2]);
        dir_result fw = trace_direction(&f, &cur, twist_on, pr, p0, nrm, (R)s_len, (R)1.0, (R)tol_coef);
        v3 be = sample_end(&f, fw.end);
        B_end_x[i] = (float)be.x;
        B_end_y[i] = (float)be.y;
        B_end_z[i] = (float)be.z;
        end_x[i] = (float)fw.end.x;
        end_y[i] = (float)fw.end.y;
        end_z[i] = (float)fw.end.z;
        flag_end[i] = fw.flag;
        dir_result bw = trace_direction(&f, &cur, twist_on, pr, p0, nrm, (R)s_len, (R)-1.0, (R)tol_coef);
        v3 bs = sample_end(&f, bw.end);
        B_start_x[i] = (float)bs.x;
        B_start_y[i] = (float)bs.y;
        B_start_z[i] = (float)bs.z;
        start_x[i] = (float)bw.end.x;
        start_y[i] = (float)bw.end.y;
        start_z[i] = (float)bw.end.z;
        flag_start[i] = bw.flag;
        LineLen[i] = fw.len + bw.len;
        if (twist_on) twist[i] = fw.twist + bw.twist;
        v3 b0 = sample_end(&f, p0);
        const R bx = b0.x, by = b0.y, bz = b0.z;
        B_this_x[i] = (float)bx;
        B_this_y[i] = (float)by;
        B_this_z[i] = (float)bz;
        const R bn = bx * nrm.x + by * nrm.y + bz * nrm.z;
        B_flag[i] = (RFABS(bn) * 100. < RSQRT_(bx * bx + by * by + bz * bz)) ? 1 : 0;
        total += f.samples + cur.samples;
    }
    if (samples_out) *samples_out = total;
    return 0;
}

QO_API int PFX(trace_all)(const float *Bx, const float *By, const float *Bz, const int *shape,
                          const float *cBx, const float *cBy, const float *cBz, double *twist, int twist_on,
                          const float *inp_x, const float *inp_y, const float *inp_z, const float *cross_dir,
                          float *start_x, float *start_y, float *start_z, int *flag_start,
                          float *end_x, float *end_y, float *end_z, int *flag_end,
                          float *B_this_x, float *B_this_y, float *B_this_z, int *B_flag,
                          float *B_start_x, float *B_start_y, float *B_start_z,
                          float *B_end_x, float *B_end_y, float *B_end_z,
                          float s_len, int64_t n_seeds, double *LineLen, float tol_coef,
                          const qsl_trace_params *pr, int64_t *samples_out)
{
    const float *const none[3] = {NULL, NULL, NULL};
    return trace_seeds(Bx, By, Bz, shape, none, 0, cBx, cBy, cBz, twist, twist_on, inp_x, inp_y, inp_z, cross_dir,
                       start_x, start_y, start_z, flag_start, end_x, end_y, end_z, flag_end, B_this_x, B_this_y,
                       B_this_z, B_flag, B_start_x, B_start_y, B_start_z, B_end_x, B_end_y, B_end_z, s_len,
                       n_seeds, LineLen, tol_coef, pr, samples_out);
}

/* Stretched grid: node coordinates xa[nx], ya[ny], za[nz] (increasing). */
QO_API int PFX(trace_all_stretch)(const float *Bx, const float *By, const float *Bz, const int *shape,
                                  const float *xa, const float *ya, const float *za, int uni,
                                  const float *cBx, const float *cBy, const float *cBz, double *twist, int twist_on,
                                  const float *inp_x, const float *inp_y, const float *inp_z, const float *cross_dir,
                                  float *start_x, float *start_y, float *start_z, int *flag_start,
                                  float *end_x, float *end_y, float *end_z, int *flag_end,
                                  float *B_this_x, float *B_this_y, float *B_this_z, int *B_flag,
                                  float *B_start_x, float *B_start_y, float *B_start_z,
                                  float *B_end_x, float *B_end_y, float *B_end_z,
                                  float s_len, int64_t n_seeds, double *LineLen, float tol_coef,
                                  const qsl_trace_params *pr, int64_t *samples_out)
{
    if (!xa || !ya || !za) return QSL_ERR_INVALID;
    const float *const ax[3] = {xa, ya, za};
    return trace_seeds(Bx, By, Bz, shape, ax, uni, cBx, cBy, cBz, twist, twist_on, inp_x, inp_y, inp_z, cross_dir,
                       start_x, start_y, start_z, flag_start, end_x, end_y, end_z, flag_end, B_this_x, B_this_y,
                       B_this_z, B_flag, B_start_x, B_start_y, B_start_z, B_end_x, B_end_y, B_end_z, s_len,
                       n_seeds, LineLen, tol_coef, pr, samples_out);
}

/* Single-function probes of the stretched grid (unit-level pinning against
 * the reference build). */
QO_API int PFX(index_bisect)(float p, int n, const float *a) { return stretch_bisect((R)p, n, a); }
QO_API int PFX(index_uni)(float p, int n, const float *a) { return stretch_uni((R)p, n, a); }

QO_API void PFX(interp_stretch)(const float *Bx, const float *By, const float *Bz, const int *shape,
                                const float *xa, const float *ya, const float *za, int uni, const float *p, int norm,
                                float *out)
{
    fld f = {Bx, By, Bz, {shape[0], shape[1], shape[2]}, 0, {xa, ya, za}, uni};
    v3 r = sample_b(&f, mk3((R)p[0], (R)p[1], (R)p[2]), norm);
    out[0] = (float)r.x; out[1] = (float)r.y; out[2] = (float)r.z;
}

QO_API int PFX(checkflag_stretch)(const int *shape, const float *xa, const float *ya, const float *za, int uni,
                                  const float *p)
{
    fld f = {NULL, NULL, NULL, {shape[0], shape[1], shape[2]}, 0, {xa, ya, za}, uni};
    return box_flag_stretch(&f, mk3((R)p[0], (R)p[1], (R)p[2]));
}

/* ---------------------------------------------------------------------- */
/* Scott deviation-vector tracer (TraceBlineScott.cu).                     */
/* ---------------------------------------------------------------------- */

/* d(b)/dx_j by central differences with step 1e-3: row j of the result is
 * (b(p + 1e-3 e_j) - b(p - 1e-3 e_j)) / 2e-3.
 * Reference: grad_unit_vec_B, TraceBlineScott.cu:204-226. */
static void grad_unit_b(fld *f, v3 p, v3 g[3])
{
    for (int j = 0; j < 3; ++j) {
        v3 lo = p, hi = p;
        /* `x -= 0.001` on a float: the offset is applied in double and the
         * result narrowed. */
        if (j == 0) { lo.x = (R)(lo.x - 0.001); hi.x = (R)(hi.x + 0.001); }
        if (j == 1) { lo.y = (R)(lo.y - 0.001); hi.y = (R)(hi.y + 0.001); }
        if (j == 2) { lo.z = (R)(lo.z - 0.001); hi.z = (R)(hi.z + 0.001); }
        v3 b1 = sample_b(f, lo, 1);
        v3 b2 = sample_b(f, hi, 1);
        g[j] = div3(sub3(b2, b1), (R)0.002);
    }
}

/* Right-hand side of the 9-component system: dp/ds = b, du/ds = (u.grad) b,
 * dv/ds = (v.grad) b.  Reference: f_scott, TraceBlineScott.cu:230-249. */
static v9 scott_rhs(fld *f, v9 s)
{
    v9 r;
    v3 g[3];
    r.p = sample_b(f, s.p, 1);
    grad_unit_b(f, s.p, g);
    /* component m of (u.grad) b = sum_j u_j * g[j].m */
    r.u.x = dot3(s.u, mk3(g[0].x, g[1].x, g[2].x));
    r.u.y = dot3(s.u, mk3(g[0].y, g[1].y, g[2].y));
    r.u.z = dot3(s.u, mk3(g[0].z, g[1].z, g[2].z));
    r.v.x = dot3(s.v, mk3(g[0].x, g[1].x, g[2].x));
    r.v.y = dot3(s.v, mk3(g[0].y, g[1].y, g[2].y));
    r.v.z = dot3(s.v, mk3(g[0].z, g[1].z, g[2].z));
    return r;
}

/* Fehlberg step on the 9-vector; the error estimate uses the position part
 * only.  Reference: RKF45_Scott, TraceBlineScott.cu:256-290. */
static v9 step_rkf45_scott(fld *f, v9 s, R h, R *err)
{
    const fehlberg_t c = fehlberg();
    v9 k1 = mul9(h, scott_rhs(f, s));
    v9 k2 = mul9(h, scott_rhs(f, add9(s, mul9(c.a21, k1))));
    v9 k3 = mul9(h, scott_rhs(f, add9(s, add9(mul9(c.a31, k1), mul9(c.a32, k2)))));
    v9 k4 = mul9(h, scott_rhs(f, add9(s, add9(add9(mul9(c.a41, k1), mul9(c.a42, k2)), mul9(c.a43, k3)))));
    v9 k5 = mul9(h, scott_rhs(f, add9(s, add9(add9(add9(mul9(c.a51, k1), mul9(c.a52, k2)), mul9(c.a53, k3)),
                                               mul9(c.a54, k4)))));
    v9 k6 = mul9(h, scott_rhs(f, add9(s, add9(add9(add9(add9(mul9(c.a61, k1), mul9(c.a62, k2)), mul9(c.a63, k3)),
                                                    mul9(c.a64, k4)),
                                               mul9(c.a65, k5)))));
    v9 hi = add9(add9(add9(add9(mul9(c.b1, k1), mul9(c.b3, k3)), mul9(c.b4, k4)), mul9(c.b5, k5)), mul9(c.b6, k6));
    v3 er = add3(add3(add3(add3(mul3(c.e1, k1.p), mul3(c.e3, k3.p)), mul3(c.e4, k4.p)), mul3(c.e5, k5.p)),
                 mul3(c.e6, k6.p));
    *err = norm3(er);
    return add9(s, hi);
}

static inline v3 unit3_rsq(v3 a)
{
    /* helper_math normalize(): v * rsqrtf(dot(v,v)), host rsqrtf = 1/sqrtf */
    R inv = (R)1.0 / RSQRT_(dot3(a, a));
    return mk3(a.x * inv, a.y * inv, a.z * inv);
}

typedef struct {
    v3 start, end;
    int flag_start, flag_end;
    R q0, qperp;
    double len;
    double twist;
    int valid;
} scott_result;

/* Reference: TraceBlineScott, TraceBlineScott.cu:334-519.  One step counter
 * (limit max_steps) and one length budget are shared by both directions;
 * the first direction traced is backward.  Seeds below z = 0 are skipped
 * (valid = 0); a seed on z ~ 0 whose field points down is its own footpoint
 * in that direction (flag 5). */
static scott_result trace_scott(fld *f, fld *cur, int twist_on, const qsl_trace_params *pr, v3 p0, R h_in,
                                R tol_coef)
{
    const int *n = f->n;
    scott_result res;
    memset(&res, 0, sizeof(res));
    const double len_lim = pr->len_ratio * (double)(n[0] + n[1] + n[2]);
    if (p0.z < -1e-8) return res;
    res.valid = 1;
    v3 b0 = sample_b(f, p0, 1);
    R nb0 = norm3(sample_b(f, p0, 0));
    R tol = (R)(pr->tol * tol_coef);
    v3 v0 = mk3(b0.y, -b0.x, 0);
    v0 = unit3_rsq(sub3(v0, mul3(dot3(v0, b0), b0)));
    v3 u0 = mk3(b0.y * v0.z - b0.z * v0.y, b0.z * v0.x - b0.x * v0.z, b0.x * v0.y - b0.y * v0.x);
    u0 = unit3_rsq(u0);
    const int z0 = p0.z < 1e-6;
    double len = 0, tw = 0;
    int64_t steps = 0;
    v9 es = {p0, u0, v0}, ee = {p0, u0, v0};
    int fs = 0, fe = 0;
    R h = h_in;
    v3 bp1 = mk3(0, 0, 0), jp1 = mk3(0, 0, 0);
    for (int sgn = -1; sgn < 2; sgn += 2) {
        v9 a = {p0, u0, v0};
        if (z0 && b0.z * sgn < 0) {
            if (sgn == -1) { es = a; fs = 5; } else { ee = a; fe = 5; }
            continue;
        }
        h = RFABS(h);
        int flag = 0;
        while ((flag == 0) & (len < len_lim) & (steps < pr->max_steps)) {
            R err;
            v9 b = step_rkf45_scott(f, a, h * sgn, &err);
            R scale = RPOW((R)((tol / err) / 11.09), (R)0.2);
            if (scale < 0.618) {
                h = (R)(h * pr->reject_factor);
                continue;
            }
            h = h * scale;
            if (h > pr->h_max) h = (R)pr->h_max;
            if (h < pr->h_min) h = (R)pr->h_min;
            R dl = norm3(sub3(b.p, a.p));
            len = len + dl;
            R td = 0;
            if (twist_on) {
                td = twist_density(f, cur, b.p, &bp1, &jp1);
                tw = tw + td / 4.0 / kRefPi * dl;
            }
            flag = box_flag(n, b.p);
            if (flag > 0) {
                len = len - dl;
                if (twist_on) tw = tw - td / 4.0 / kRefPi * dl;
                if (flag <= 6) {
                    const int d = (flag - 1) / 2;
                    const R q1 = comp3(a.p, d), q2 = comp3(b.p, d);
                    R qmid = q1;
                    v9 e;
                    if (RFABS(q1 - q2) > 0) {
                        qmid = (flag % 2 == 1) ? (R)0 : (R)n[d];
                        e = div9(add9(mul9(q2 - qmid, a), mul9(qmid - q1, b)), q2 - q1);
                        /* the exit segment's length divides by the field's
                         * component along the exit axis, B_P1 in the
                         * reference (:448): with the twist on it is B at the
                         * point past the face (:425); with it off the
                         * reference leaves B_P1 unset, and the unit field at
                         * the last inside point stands in (as in
                         * TraceBlineAdaptive.cu:404) */
                        v3 ua = twist_on ? bp1 : sample_b(f, a.p, 1);
                        len = len + RFABS(qmid - q1) / (1e-4 + RFABS(comp3(ua, d)));
                    } else {
                        e = a;
                    }
                    if (sgn == -1) { es = e; fs = flag; } else { ee = e; fe = flag; }
                    if (twist_on) tw = tw + td / 4.0 / kRefPi * RFABS(qmid - q1) / (1e-4 + RFABS(comp3(bp1, d)));
                } else {
                    if (sgn == -1) { es = a; fs = flag; } else { ee = a; fe = flag; }
                    res.start = es.p; res.end = ee.p;
                    res.flag_start = fs; res.flag_end = fe;
                    res.q0 = 0; res.qperp = 0;
                    res.len = len; res.twist = tw;
                    return res;
                }
            }
            a = b;
            steps = steps + 1;
        }
        if (flag == 0) {
            if (sgn == -1) { es = a; fs = 0; } else { ee = a; fe = 0; }
        }
    }
    /* Q from the deviation vectors at both footpoints.  Reference:
     * TraceBlineScott.cu:475-508. */
    const int ds = (fs - 1) / 2, de = (fe - 1) / 2;
    const int dsc = (ds >= 0 && ds < 3) ? ds : 2, dec = (de >= 0 && de < 3) ? de : 2;
    v3 Bs = sample_b(f, es.p, 0), Be = sample_b(f, ee.p, 0);
    R BNs = comp3(Bs, dsc), BNe = comp3(Be, dec);
    v3 us = es.u, vs = es.v, ue = ee.u, ve = ee.v;
    v3 us1 = sub3(us, mul3(comp3(us, dsc) / comp3(Bs, dsc), Bs));
    v3 vs1 = sub3(vs, mul3(comp3(vs, dsc) / comp3(Bs, dsc), Bs));
    v3 ue1 = sub3(ue, mul3(comp3(ue, dec) / comp3(Be, dec), Be));
    v3 ve1 = sub3(ve, mul3(comp3(ve, dec) / comp3(Be, dec), Be));
    {
        double num = dot3(ue1, ue1) * dot3(vs1, vs1) + dot3(us1, us1) * dot3(ve1, ve1)
                     - 2.0 * dot3(ue1, ve1) * dot3(us1, vs1);
        res.q0 = (R)(fabs(num) / fabs((double)((nb0 * nb0) / (BNs * BNe))));
    }
    {
        R lBe = norm3(Be), lBs = norm3(Bs);
        ue1 = sub3(ue, mul3(dot3(ue, Be) / lBe, div3(Be, lBe)));
        ve1 = sub3(ve, mul3(dot3(ve, Be) / lBe, div3(Be, lBe)));
        us1 = sub3(us, mul3(dot3(us, Bs) / lBs, div3(Bs, lBs)));
        vs1 = sub3(vs, mul3(dot3(vs, Bs) / lBs, div3(Bs, lBs)));
        double num = dot3(ue1, ue1) * dot3(vs1, vs1) + dot3(us1, us1) * dot3(ve1, ve1)
                     - 2.0 * dot3(ue1, ve1) * dot3(us1, vs1);
        res.qperp = (R)(fabs(num) / (double)((nb0 * nb0) / (lBs * lBe)));
    }
    res.start = es.p;
    res.end = ee.p;
    res.flag_start = fs;
    res.flag_end = fe;
    res.len = len;
    res.twist = tw;
    return res;
}

/* Reference: TraceAllBlineScott, TraceBlineScott.cu:521-595.  Outputs of a
 * skipped seed (z < 0) are zeros. */
QO_API int PFX(scott_all)(const float *Bx, const float *By, const float *Bz, const int *shape,
                          const float *cBx, const float *cBy, const float *cBz, double *twist, int twist_on,
                          const float *inp_x, const float *inp_y, const float *inp_z,
                          float *start_x, float *start_y, float *start_z, int *flag_start,
                          float *end_x, float *end_y, float *end_z, int *flag_end,
                          float *B_this_x, float *B_this_y, float *B_this_z,
                          float *q0, float *qperp,
                          float s_len, int64_t n_seeds, double *LineLen, float tol_coef,
                          const qsl_trace_params *pr, int64_t *samples_out)
{
    if (!Bx || !By || !Bz || !shape || !pr) return QSL_ERR_INVALID;
    if (twist_on && (!cBx || !cBy || !cBz || !twist)) return QSL_ERR_INVALID;
    int64_t total = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : total)
    for (int64_t i = 0; i < n_seeds; ++i) {
        fld f = {Bx, By, Bz, {shape[0], shape[1], shape[2]}, 0};
        fld cur = {cBx, cBy, cBz, {shape[0], shape[1], shape[2]}, 0};
        const v3 p0 = mk3((R)inp_x[i], (R)inp_y[i], (R)inp_z[i]);
        scott_result r = trace_scott(&f, &cur, twist_on, pr, p0, (R)s_len, (R)tol_coef);
        start_x[i] = (float)r.start.x; start_y[i] = (float)r.start.y; start_z[i] = (float)r.start.z;
        end_x[i] = (float)r.end.x; end_y[i] = (float)r.end.y; end_z[i] = (float)r.end.z;
        flag_start[i] = r.flag_start;
        flag_end[i] = r.flag_end;
        LineLen[i] = r.len;
        if (twist_on) twist[i] = r.twist;
        B_this_x[i] = (float)sample_scalar(Bx, f.n, p0.x, p0.y, p0.z);
        B_this_y[i] = (float)sample_scalar(By, f.n, p0.x, p0.y, p0.z);
        B_this_z[i] = (float)sample_scalar(Bz, f.n, p0.x, p0.y, p0.z);
        q0[i] = (float)r.q0;
        qperp[i] = (float)r.qperp;
        total += f.samples + cur.samples;
    }
    if (samples_out) *samples_out = total;
    return 0;
}

/* ---------------------------------------------------------------------- */
/* Single-function probes (unit-level pinning against the reference).      */
/* ---------------------------------------------------------------------- */
static fld mkfld(const float *Bx, const float *By, const float *Bz, const int *shape)
{
    fld f = {Bx, By, Bz, {shape[0], shape[1], shape[2]}, 0};
    return f;
}
static v3 ld3(const float *p) { return mk3((R)p[0], (R)p[1], (R)p[2]); }
static void st3(v3 a, float *o) { o[0] = (float)a.x; o[1] = (float)a.y; o[2] = (float)a.z; }
static v9 ld9(const float *p) { v9 r = {ld3(p), ld3(p + 3), ld3(p + 6)}; return r; }
static void st9(v9 a, float *o) { st3(a.p, o); st3(a.u, o + 3); st3(a.v, o + 6); }

QO_API void PFX(interp3dxyzn)(const float *Bx, const float *By, const float *Bz, const int *shape, const float *p,
                              int unit, float *out)
{
    fld f = mkfld(Bx, By, Bz, shape);
    st3(sample_b(&f, ld3(p), unit), out);
}
QO_API float PFX(interp3d)(const float *A, const int *shape, const float *p)
{
    return (float)sample_scalar(A, shape, (R)p[0], (R)p[1], (R)p[2]);
}
QO_API int PFX(checkflag)(const int *shape, const float *p) { return box_flag(shape, ld3(p)); }
QO_API void PFX(rk4_step)(const float *Bx, const float *By, const float *Bz, const int *shape, const float *p,
                          float h, float *out)
{
    fld f = mkfld(Bx, By, Bz, shape);
    st3(step_rk4(&f, ld3(p), (R)h), out);
}
QO_API void PFX(rk4_boundary)(const float *Bx, const float *By, const float *Bz, const int *shape, const float *p,
                              float h, int d, float *out)
{
    fld f = mkfld(Bx, By, Bz, shape);
    st3(step_rk4_normal(&f, ld3(p), (R)h, d), out);
}
QO_API void PFX(rkf45_step)(const float *Bx, const float *By, const float *Bz, const int *shape, const float *p,
                            float h, float *out4)
{
    fld f = mkfld(Bx, By, Bz, shape);
    R err;
    st3(step_rkf45(&f, ld3(p), (R)h, &err), out4);
    out4[3] = (float)err;
}
QO_API void PFX(grad_unit_vec_B)(const float *Bx, const float *By, const float *Bz, const int *shape,
                                 const float *p, float *out9)
{
    fld f = mkfld(Bx, By, Bz, shape);
    v3 g[3];
    grad_unit_b(&f, ld3(p), g);
    st3(g[0], out9); st3(g[1], out9 + 3); st3(g[2], out9 + 6);
}
QO_API void PFX(f_scott)(const float *Bx, const float *By, const float *Bz, const int *shape, const float *v9in,
                         float *out9)
{
    fld f = mkfld(Bx, By, Bz, shape);
    st9(scott_rhs(&f, ld9(v9in)), out9);
}
QO_API float PFX(rkf45_scott)(const float *Bx, const float *By, const float *Bz, const int *shape,
                              const float *v9in, float h, float *out9)
{
    fld f = mkfld(Bx, By, Bz, shape);
    R err;
    st9(step_rkf45_scott(&f, ld9(v9in), (R)h, &err), out9);
    return (float)err;
}
