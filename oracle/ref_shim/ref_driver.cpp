/*
 * Host driver around the reference's UNMODIFIED tracing kernels.
 *
 * Test infrastructure only (oracle): compiled by oracle/build_ref.sh from the
 * reference sources where they lie, never shipped in the fastqsl_gb300
 * package.  One shared object per kernel file:
 *   REF_KERNEL == 1  fastqslpy/cu/TraceBline.cu          (RK4)
 *   REF_KERNEL == 2  fastqslpy/cu/TraceBlineAdaptive.cu  (RKF45)
 *   REF_KERNEL == 3  fastqslpy/cu/TraceBlineScott.cu     (RKF45 + deviation vectors)
 *   REF_KERNEL == 4  fastqslpy/cu/TraceBlineAdaptiveStretch.cu (RKF45 on a stretched grid)
 *
 * qref_trace_all runs the reference kernel body TraceAllBline once per seed
 * (grid = block = 1, N = 1, pointer-offset slices) under an OpenMP loop, which
 * is exactly the work one GPU thread of the reference does for that seed.
 * The qref_* probes expose single device functions (interpolation, one
 * integrator step, the boundary test) for unit-level pinning.
 */
#include <cstddef>
#include <cstdlib>
#include <cstdio>
#include <new>
#include <omp.h>
#include "cuda_runtime.h"

#if REF_KERNEL == 1
#include "TraceBline.cu"
#elif REF_KERNEL == 2
#include "TraceBlineAdaptive.cu"
#elif REF_KERNEL == 3
#include "TraceBlineScott.cu"
#elif REF_KERNEL == 4
#include "TraceBlineAdaptiveStretch.cu"
#else
#error "REF_KERNEL must be 1, 2, 3 or 4"
#endif

thread_local uint3 threadIdx;
thread_local uint3 blockIdx;
thread_local dim3 blockDim;
thread_local dim3 gridDim;

/* The reference kernels keep per-thread scratch in `new float[3]` buffers and
 * write a line's footpoint into it only when the line leaves the box; a line
 * stopped by the step or length limit reports whatever the buffer held.  A
 * zero-filled allocation makes that case deterministic here (footpoint 0,0,0
 * for a forward trace, the forward footpoint for a backward trace). */
__attribute__((visibility("hidden"))) void *operator new[](std::size_t n)
{
    void *p = std::calloc(1, n ? n : 1);
    if (!p) std::abort();
    return p;
}
__attribute__((visibility("hidden"))) void operator delete[](void *p) noexcept { std::free(p); }
__attribute__((visibility("hidden"))) void operator delete[](void *p, std::size_t) noexcept { std::free(p); }

static void set_single_thread_launch()
{
    threadIdx = make_uint3(0, 0, 0);
    blockIdx = make_uint3(0, 0, 0);
    blockDim = dim3(1, 1, 1);
    gridDim = dim3(1, 1, 1);
}

#define QREF_API extern "C" __attribute__((visibility("default")))

QREF_API int qref_kernel_kind(void) { return REF_KERNEL; }

QREF_API int qref_set_threads(int n)
{
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
}

static inline int3 shape_of(const int *s) { return make_int3(s[0], s[1], s[2]); }

#if REF_KERNEL != 4
QREF_API void qref_interp3dxyzn(const float *Bx, const float *By, const float *Bz, const int *shape,
                                const float *p, int norm, float *out)
{
    float3 r = Interp3dxyzn((float *)Bx, (float *)By, (float *)Bz, shape_of(shape),
                            make_float3(p[0], p[1], p[2]), norm != 0);
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

QREF_API float qref_interp3d(const float *A, const int *shape, const float *p)
{
    return Interp3d((float *)A, shape_of(shape), p[0], p[1], p[2]);
}

QREF_API int qref_checkflag(const int *shape, const float *p)
{
    return checkFlag(shape_of(shape), make_float3(p[0], p[1], p[2]));
}
#endif

#if REF_KERNEL == 1 || REF_KERNEL == 2
QREF_API void qref_rk4_step(const float *Bx, const float *By, const float *Bz, const int *shape,
                            const float *p, float h, float *out)
{
    float3 r = RK4((float *)Bx, (float *)By, (float *)Bz, shape_of(shape), make_float3(p[0], p[1], p[2]), h);
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

QREF_API void qref_rk4_boundary(const float *Bx, const float *By, const float *Bz, const int *shape,
                                const float *p, float h, int dim, float *out)
{
    float3 r = RK4_boundary((float *)Bx, (float *)By, (float *)Bz, shape_of(shape),
                            make_float3(p[0], p[1], p[2]), h, dim);
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}
#endif

#if REF_KERNEL == 2
QREF_API void qref_rkf45_step(const float *Bx, const float *By, const float *Bz, const int *shape,
                              const float *p, float h, float *out4)
{
    float4 r = RKF45((float *)Bx, (float *)By, (float *)Bz, shape_of(shape), make_float3(p[0], p[1], p[2]), h);
    out4[0] = r.x; out4[1] = r.y; out4[2] = r.z; out4[3] = r.w;
}
#endif

#if REF_KERNEL == 1 || REF_KERNEL == 2
/* Runs TraceAllBline for seeds [0, n).  Argument order follows the kernel's
 * own (TraceBlineAdaptive.cu:429-437); scalars are passed by value here and
 * re-boxed into the one-element arrays the kernel reads. */
QREF_API int qref_trace_all(const float *Bx, const float *By, const float *Bz, const int *shape,
                            const float *curBx, const float *curBy, const float *curBz, double *twist,
                            int twist_flag,
                            const float *inp_x, const float *inp_y, const float *inp_z, const float *cross_dir,
                            float *start_x, float *start_y, float *start_z, int *flag_start,
                            float *end_x, float *end_y, float *end_z, int *flag_end,
                            float *B_this_x, float *B_this_y, float *B_this_z, int *B_flag,
                            float *B_start_x, float *B_start_y, float *B_start_z,
                            float *B_end_x, float *B_end_y, float *B_end_z,
                            float s_len, unsigned long long n, double *LineLen, float tol_coef)
{
    bool flag = twist_flag != 0;
    if (flag && (!curBx || !curBy || !curBz || !twist)) return -1;
    const float *cx = flag ? curBx : Bx, *cy = flag ? curBy : By, *cz = flag ? curBz : Bz;
#pragma omp parallel for schedule(dynamic, 64)
    for (long long i = 0; i < (long long)n; ++i) {
        set_single_thread_launch();
        int shp[3] = {shape[0], shape[1], shape[2]};
        float cd[3] = {cross_dir[0], cross_dir[1], cross_dir[2]};
        float sl = s_len, tc = tol_coef;
        unsigned long long one = 1;
        double tw_dummy = 0;
        bool f = flag;
        double *tw = flag ? twist + i : &tw_dummy;
#if REF_KERNEL == 2
        TraceAllBline((float *)Bx, (float *)By, (float *)Bz, shp, (float *)cx, (float *)cy, (float *)cz, tw, &f,
                      (float *)inp_x + i, (float *)inp_y + i, (float *)inp_z + i, cd,
                      start_x + i, start_y + i, start_z + i, flag_start + i,
                      end_x + i, end_y + i, end_z + i, flag_end + i,
                      B_this_x + i, B_this_y + i, B_this_z + i, B_flag + i,
                      B_start_x + i, B_start_y + i, B_start_z + i,
                      B_end_x + i, B_end_y + i, B_end_z + i,
                      &sl, &one, LineLen + i, &tc);
#else
        (void)tc;
        TraceAllBline((float *)Bx, (float *)By, (float *)Bz, shp, (float *)cx, (float *)cy, (float *)cz, tw, &f,
                      (float *)inp_x + i, (float *)inp_y + i, (float *)inp_z + i, cd,
                      start_x + i, start_y + i, start_z + i, flag_start + i,
                      end_x + i, end_y + i, end_z + i, flag_end + i,
                      B_this_x + i, B_this_y + i, B_this_z + i, B_flag + i,
                      B_start_x + i, B_start_y + i, B_start_z + i,
                      B_end_x + i, B_end_y + i, B_end_z + i,
                      &sl, &one, LineLen + i);
#endif
    }
    return 0;
}
#endif

#if REF_KERNEL == 3
/* Scott-method building blocks (TraceBlineScott.cu:204-290), and the
 * whole-line routine TraceBlineScott (:334-519) from the copy of the file
 * whose uninitialised tolerance (:352,378) build_ref.sh sets to
 * TOL*tol_coef. */
static float9 load9(const float *v)
{
    float9 r;
    r.x = make_float3(v[0], v[1], v[2]);
    r.y = make_float3(v[3], v[4], v[5]);
    r.z = make_float3(v[6], v[7], v[8]);
    return r;
}
static void store9(float9 r, float *v)
{
    v[0] = r.x.x; v[1] = r.x.y; v[2] = r.x.z;
    v[3] = r.y.x; v[4] = r.y.y; v[5] = r.y.z;
    v[6] = r.z.x; v[7] = r.z.y; v[8] = r.z.z;
}

QREF_API void qref_grad_unit_vec_B(const float *Bx, const float *By, const float *Bz, const int *shape,
                                   const float *p, float *out9)
{
    store9(grad_unit_vec_B((float *)Bx, (float *)By, (float *)Bz, shape_of(shape), make_float3(p[0], p[1], p[2])),
           out9);
}

QREF_API void qref_f_scott(const float *Bx, const float *By, const float *Bz, const int *shape,
                           const float *v9, float *out9)
{
    store9(f_scott((float *)Bx, (float *)By, (float *)Bz, shape_of(shape), load9(v9)), out9);
}

QREF_API float qref_rkf45_scott(const float *Bx, const float *By, const float *Bz, const int *shape,
                                const float *v9, float h, float *out9)
{
    float9 o;
    float err = RKF45_Scott((float *)Bx, (float *)By, (float *)Bz, shape_of(shape), load9(v9), &o, h);
    store9(o, out9);
    return err;
}

/* TraceBlineScott for seeds [0, n), as one thread of TraceAllBlineScott
 * (:521-595) runs it, with its per-seed locals initialised here: the
 * reference kernel leaves the exit flags unset when a line ends on the shared
 * step limit, and the footpoints and q unset when a line ends on an edge or
 * corner (flag 42), so those lines keep flag 0 and the footpoint/q outputs
 * of such lines are whatever the routine left in its locals (the caller
 * masks them).  B_this as the kernel computes it (:583-585).  The line
 * length is not reported: the routine adds a term with B_P1, which it
 * sets only when the twist is on (:448), so with the twist off it is not
 * defined. */
QREF_API int qref_scott_all(const float *Bx, const float *By, const float *Bz, const int *shape,
                            const float *curBx, const float *curBy, const float *curBz, double *twist,
                            int twist_flag, const float *inp_x, const float *inp_y, const float *inp_z,
                            const float *cross_dir, float *start_x, float *start_y, float *start_z,
                            int *flag_start, float *end_x, float *end_y, float *end_z, int *flag_end,
                            float *B_this_x, float *B_this_y, float *B_this_z, float *q_0, float *q_perp,
                            float s_len, unsigned long long n, float tol_coef)
{
    bool flag = twist_flag != 0;
    if (flag && (!curBx || !curBy || !curBz || !twist)) return -1;
    const float *cx = flag ? curBx : Bx, *cy = flag ? curBy : By, *cz = flag ? curBz : Bz;
#pragma omp parallel for schedule(dynamic, 16)
    for (long long i = 0; i < (long long)n; ++i) {
        set_single_thread_launch();
        int3 s3 = shape_of(shape);
        float cd[3] = {cross_dir[0], cross_dir[1], cross_dir[2]};
        float p0[3] = {inp_x[i], inp_y[i], inp_z[i]};
        double tw = 0, len = 0;
        bool f = flag;
        int fs = 0, fe = 0;
        float q0 = 0.f, qp = 0.f;
        float9 pv = TraceBlineScott((float *)Bx, (float *)By, (float *)Bz, s3, (float *)cx, (float *)cy,
                                    (float *)cz, &tw, &f, p0, cd, s_len, &fs, &fe, &q0, &qp, &len, tol_coef);
        start_x[i] = pv.x.x; start_y[i] = pv.x.y; start_z[i] = pv.x.z;
        end_x[i] = pv.z.x; end_y[i] = pv.z.y; end_z[i] = pv.z.z;
        flag_start[i] = fs;
        flag_end[i] = fe;
        if (flag) twist[i] = tw;
        B_this_x[i] = Interp3d((float *)Bx, s3, p0[0], p0[1], p0[2]);
        B_this_y[i] = Interp3d((float *)By, s3, p0[0], p0[1], p0[2]);
        B_this_z[i] = Interp3d((float *)Bz, s3, p0[0], p0[1], p0[2]);
        q_0[i] = q0;
        q_perp[i] = qp;
    }
    return 0;
}
#endif

#if REF_KERNEL == 4
/* Stretched-grid building blocks (TraceBlineAdaptiveStretch.cu:42-201,309-331). */
QREF_API int qref_index_bisect(float p, int n, const float *a) { return GetIndexBiSearch(p, n, (float *)a); }

QREF_API int qref_index_uni(float p, int n, const float *a) { return GetIndexUniStretch(p, n, (float *)a); }

QREF_API void qref_interp_stretch(const float *Bx, const float *By, const float *Bz, const int *shape,
                                  const float *xa, const float *ya, const float *za, int uni, const float *p,
                                  int norm, float *out)
{
    float3 r = Interp3dxyzn((float *)Bx, (float *)By, (float *)Bz, shape_of(shape), make_float3(p[0], p[1], p[2]),
                            norm != 0, (float *)xa, (float *)ya, (float *)za, uni != 0);
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

QREF_API int qref_checkflag_stretch(const int *shape, const float *xa, const float *ya, const float *za, int uni,
                                    const float *p)
{
    return checkFlag(shape_of(shape), make_float3(p[0], p[1], p[2]), (float *)xa, (float *)ya, (float *)za,
                     uni != 0);
}

/* TraceAllBline of the stretched-grid file (TraceBlineAdaptiveStretch.cu:422-508) for seeds [0, n), one
 * single-thread launch per seed as above. */
QREF_API int qref_trace_all_stretch(const float *Bx, const float *By, const float *Bz, const int *shape,
                                    const float *xa, const float *ya, const float *za, int uni,
                                    const float *curBx, const float *curBy, const float *curBz, double *twist,
                                    int twist_flag,
                                    const float *inp_x, const float *inp_y, const float *inp_z,
                                    const float *cross_dir,
                                    float *start_x, float *start_y, float *start_z, int *flag_start,
                                    float *end_x, float *end_y, float *end_z, int *flag_end,
                                    float *B_this_x, float *B_this_y, float *B_this_z, int *B_flag,
                                    float *B_start_x, float *B_start_y, float *B_start_z,
                                    float *B_end_x, float *B_end_y, float *B_end_z,
                                    float s_len, unsigned long long n, double *LineLen, float tol_coef)
{
    bool flag = twist_flag != 0;
    if (flag && (!curBx || !curBy || !curBz || !twist)) return -1;
    const float *cx = flag ? curBx : Bx, *cy = flag ? curBy : By, *cz = flag ? curBz : Bz;
#pragma omp parallel for schedule(dynamic, 64)
    for (long long i = 0; i < (long long)n; ++i) {
        set_single_thread_launch();
        int shp[3] = {shape[0], shape[1], shape[2]};
        float cd[3] = {cross_dir[0], cross_dir[1], cross_dir[2]};
        float sl = s_len, tc = tol_coef;
        unsigned long long one = 1;
        double tw_dummy = 0;
        bool f = flag, u = uni != 0;
        double *tw = flag ? twist + i : &tw_dummy;
        TraceAllBline((float *)Bx, (float *)By, (float *)Bz, shp, (float *)xa, (float *)ya, (float *)za, &u,
                      (float *)cx, (float *)cy, (float *)cz, tw, &f,
                      (float *)inp_x + i, (float *)inp_y + i, (float *)inp_z + i, cd,
                      start_x + i, start_y + i, start_z + i, flag_start + i,
                      end_x + i, end_y + i, end_z + i, flag_end + i,
                      B_this_x + i, B_this_y + i, B_this_z + i, B_flag + i,
                      B_start_x + i, B_start_y + i, B_start_z + i,
                      B_end_x + i, B_end_y + i, B_end_z + i,
                      &sl, &one, LineLen + i, &tc);
    }
    return 0;
}
#endif
