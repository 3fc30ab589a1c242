/*
 * fastqsl_gb300 — C ABI of the GB300 (sm_103a) field-line tracer and
 * squashing-factor (Q) assembly.
 *
 * Conventions
 *  - Every pointer argument is a DEVICE pointer unless its name ends in _h.
 *  - Field arrays Bx, By, Bz have shape (nx, ny, nz) with x fastest in memory:
 *    element (i, j, k) lives at i + nx*(j + ny*k)  (the layout of
 *    fastqslpy/cu/TraceBlineAdaptive.cu:36-39, get_Idx3d).
 *  - Every entry point returns 0 on success and a negative qsl_status on
 *    failure; work is enqueued on `stream` (0 = legacy default stream) and the
 *    call does not synchronise unless stated.
 *  - Per-line boundary flags keep the reference meaning
 *    (TraceBlineAdaptive.cu:309-331): 0 inside / stopped by a limit,
 *    1..6 left through x-min, x-max, y-min, y-max, z-min, z-max,
 *    42 edge, corner or non-finite position.
 */
#ifndef FASTQSL_GB300_H
#define FASTQSL_GB300_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *qsl_stream_t; /* == cudaStream_t */

enum qsl_status {
    QSL_OK = 0,
    QSL_ERR_INVALID = -1,   /* bad argument: null pointer, bad shape, bad enum */
    QSL_ERR_NOMEM = -2,     /* device allocation failed */
    QSL_ERR_CUDA = -3,      /* a CUDA call failed; qsl_last_error() has the text */
    QSL_ERR_TOO_LARGE = -4, /* request exceeds a stated maximum */
    QSL_ERR_NODEVICE = -5
};

enum qsl_integrator { QSL_RK4 = 0, QSL_RKF45 = 1 };

enum qsl_tol_law {
    /* tol*|b0.n|^1.5*tol_coef, or tol/8e3*tol_coef when |b0.n| <= 0.05, with b0
     * the unit field at the seed and n the seed-plane normal
     * (TraceBlineAdaptive.cu:354-359) */
    QSL_TOL_REFERENCE = 0,
    /* tol*tol_coef */
    QSL_TOL_ABSOLUTE = 1
};

/* Arithmetic of the tracing kernels. */
enum qsl_arith {
    /* Same operation order and rounding as the reference kernels built without
     * fused multiply-add: corner weights in FP64, IEEE divide and sqrt. */
    QSL_ARITH_EXACT = 0,
    /* FP32 with fused multiply-add, FP32 corner weights and rsqrt
     * normalisation.  On the fp16 stores the node values are widened exactly
     * and every lerp is FP32. */
    QSL_ARITH_FAST = 1,
    /* qsl_trace on the QSL_LAYOUT_H4B store only: QSL_ARITH_FAST with the x
     * weights (1 - r, r) rounded to fp16 and the x-lerps done by the
     * mixed-precision f16 x f16 + f32 multiply-add (fewer instructions per
     * sample; the x fraction is quantised to ~2^-11).  Rejected elsewhere. */
    QSL_ARITH_FAST_W16 = 2
};

/* Integrator settings.  qsl_params_reference_rk4/_rkf45 fill the values the
 * reference hard-wires (TraceBline.cu:10-12, TraceBlineAdaptive.cu:10-13). */
typedef struct qsl_trace_params {
    int32_t integrator;      /* qsl_integrator */
    int32_t tol_law;         /* qsl_tol_law (RKF45 only) */
    double tol;              /* base local-error tolerance; reference 1e-3 */
    double h_min;            /* accepted-step lower clamp; reference 0.1 */
    double h_max;            /* accepted-step upper clamp; reference 100 */
    double reject_factor;    /* step shrink on rejection; reference 0.618 */
    double len_ratio;        /* length limit = len_ratio*(nx+ny+nz); ref 3 (RKF45), 2 (RK4) */
    int64_t max_steps;       /* accepted steps per direction; ref 500000 (RKF45), 100000 (RK4) */
    int32_t boundary_twist;  /* add the exit-segment twist term (RK4 reference does, TraceBline.cu:362-365) */
    int32_t arith;           /* qsl_arith */
    int32_t max_rejects;     /* RKF45: this many rejected trial steps in a row end the direction where
                                it is (flag 0, status QSL_LINE_REJECT_LIMIT); 0 = no limit, as in the
                                reference, whose controller then only stops when the step size
                                underflows and the position turns non-finite (flag 42) */
} qsl_trace_params;

/* How one direction of a line ended (the optional status_start / status_end
 * outputs of qsl_trace_io; the reference reports only the flag, which is 0
 * for every limit and 42 for edges, corners and non-finite positions alike). */
enum qsl_line_status {
    QSL_LINE_FACE = 0,         /* left through a face: flag 1..6 */
    QSL_LINE_EDGE = 1,         /* left through an edge or corner: flag 42, finite position */
    QSL_LINE_NAN = 2,          /* the position became non-finite (NaN/Inf field or step): flag 42 */
    QSL_LINE_MAX_STEPS = 3,    /* stopped by max_steps: flag 0 */
    QSL_LINE_MAX_LENGTH = 4,   /* stopped by the length limit: flag 0 */
    QSL_LINE_REJECT_LIMIT = 5  /* stopped by max_rejects: flag 0 */
};

void qsl_params_reference_rk4(qsl_trace_params *p_h);
void qsl_params_reference_rkf45(qsl_trace_params *p_h);

/* Text of the last error on the calling host thread. */
const char *qsl_last_error(void);
const char *qsl_version(void);
int qsl_device_sm_count(int *sms_h);

/* ------------------------------------------------------------------------
 * Drop-in tracing entry points.
 *
 * These replace the CUDA kernel the reference compiles at run time and calls
 * through cupy.RawKernel (fastqslpy/kernels.py:10-29, returning
 * TraceAllBline):
 *   qsl_trace_all_bline_rkf45 <- TraceAllBline of
 *       fastqslpy/cu/TraceBlineAdaptive.cu:429-437 (35 arguments)
 *   qsl_trace_all_bline_rk4   <- TraceAllBline of
 *       fastqslpy/cu/TraceBline.cu:383-391 (34 arguments, no tol_coef)
 * Same argument order and meaning; scalars (BshapeN[3], inp_cross_dir[3],
 * s_len[1], N[1], tol_coef[1], curB_flag[1]) are device pointers as in the
 * reference; every array is caller-allocated device memory.  The launch
 * geometry the reference takes from the caller is chosen here (a persistent
 * grid sized to the GPU).  Arithmetic is QSL_ARITH_EXACT.  When *curB_flag
 * is false the curB_* arrays and `twist` are not read or written (they may be
 * null).  Asynchronous on `stream`.
 * ------------------------------------------------------------------------ */
int qsl_trace_all_bline_rkf45(const float *Bx, const float *By, const float *Bz, const int *BshapeN,
                              const float *curB_x, const float *curB_y, const float *curB_z, double *twist,
                              const bool *curB_flag, const float *inp_x, const float *inp_y, const float *inp_z,
                              const float *inp_cross_dir, float *start_x, float *start_y, float *start_z,
                              int *flag_start, float *end_x, float *end_y, float *end_z, int *flag_end,
                              float *B_this_x, float *B_this_y, float *B_this_z, int *B_flag, float *B_start_x,
                              float *B_start_y, float *B_start_z, float *B_end_x, float *B_end_y, float *B_end_z,
                              const float *s_len, const unsigned long long *N, double *LineLen,
                              const float *tol_coef, qsl_stream_t stream);

int qsl_trace_all_bline_rk4(const float *Bx, const float *By, const float *Bz, const int *BshapeN,
                            const float *curB_x, const float *curB_y, const float *curB_z, double *twist,
                            const bool *curB_flag, const float *inp_x, const float *inp_y, const float *inp_z,
                            const float *inp_cross_dir, float *start_x, float *start_y, float *start_z,
                            int *flag_start, float *end_x, float *end_y, float *end_z, int *flag_end,
                            float *B_this_x, float *B_this_y, float *B_this_z, int *B_flag, float *B_start_x,
                            float *B_start_y, float *B_start_z, float *B_end_x, float *B_end_y, float *B_end_z,
                            const float *s_len, const unsigned long long *N, double *LineLen, qsl_stream_t stream);

/* The two entries above with the integrator (qsl_integrator) and arithmetic
 * (qsl_arith) chosen by the caller; tol_coef may be null for QSL_RK4.
 * capacity >= 0: the number of elements every per-seed array holds; seeds at
 * or beyond it are never read or written even if *N is larger (0: nothing
 * is launched and the pointers may be null).  -1: trust *N as the
 * reference does. */
int qsl_trace_all_bline(int integrator, int arith, const float *Bx, const float *By, const float *Bz,
                        const int *BshapeN, const float *curB_x, const float *curB_y, const float *curB_z,
                        double *twist, const bool *curB_flag, const float *inp_x, const float *inp_y,
                        const float *inp_z, const float *inp_cross_dir, float *start_x, float *start_y,
                        float *start_z, int *flag_start, float *end_x, float *end_y, float *end_z, int *flag_end,
                        float *B_this_x, float *B_this_y, float *B_this_z, int *B_flag, float *B_start_x,
                        float *B_start_y, float *B_start_z, float *B_end_x, float *B_end_y, float *B_end_z,
                        const float *s_len, const unsigned long long *N, double *LineLen, const float *tol_coef,
                        int64_t capacity, qsl_stream_t stream);

/* ------------------------------------------------------------------------
 * Resident field stores (no reference counterpart: the reference keeps the
 * caller's three arrays).  A store converts the caller's field once into a
 * GB300 layout and owns that copy; QSL_LAYOUT_SOA borrows the caller's
 * arrays (they must outlive the store).
 * ------------------------------------------------------------------------ */
enum qsl_layout {
    QSL_LAYOUT_SOA = 0, /* the caller's Bx, By, Bz in place */
    QSL_LAYOUT_F4 = 1,  /* interleaved float4 per node (16 B/node) */
    QSL_LAYOUT_H4B = 2, /* fp16 8^3-cell bricks with a +1 apron and a float scale per brick, as x-pair
                           records (node i and i+1 in 16 B; ~20 B/node): the fastest store.  A
                           z-slab of bricks must hold < 2^32 records (nx, ny up to ~20,000) */
    QSL_LAYOUT_H8C = 3  /* fp16 cell records: each cell's 8 corner vectors in 64 B, power-of-two
                           scale per cell (~64 B per cell) */
};
typedef struct qsl_field qsl_field_t;

/* Device bytes a store of this shape and layout owns (0 for SOA). */
int64_t qsl_field_store_bytes(int nx, int ny, int nz, int layout);
int qsl_field_create(const float *Bx, const float *By, const float *Bz, int nx, int ny, int nz, int layout,
                     qsl_stream_t stream, qsl_field_t **out_h);
int qsl_field_destroy(qsl_field_t *field);
int64_t qsl_field_bytes(const qsl_field_t *field);
/* Refills a store from new arrays of the same shape (no reallocation). */
int qsl_field_update(qsl_field_t *field, const float *Bx, const float *By, const float *Bz, qsl_stream_t stream);

/* ------------------------------------------------------------------------
 * Native tracing entry (the drop-in entries are thin wrappers of the same
 * kernels).  Outputs keep the meaning of TraceAllBline's
 * (TraceBlineAdaptive.cu:429-510).
 * ------------------------------------------------------------------------ */
enum qsl_schedule {
    QSL_SCHED_QUEUE = 0, /* persistent grid, per-lane refill from a device work counter */
    QSL_SCHED_STATIC = 1 /* one line per thread; the grid covers n (with n_dev set, n is the capacity) */
};

typedef struct qsl_trace_io {
    const float *inp_x, *inp_y, *inp_z;
    float *start_x, *start_y, *start_z;
    int *flag_start;
    float *end_x, *end_y, *end_z;
    int *flag_end;
    float *B_this_x, *B_this_y, *B_this_z;
    int *B_flag;
    float *B_start_x, *B_start_y, *B_start_z;
    float *B_end_x, *B_end_y, *B_end_z;
    double *LineLen;
    double *twist; /* needed when curB is given */
    int *status_start, *status_end; /* optional (null = not written): qsl_line_status of the
                                       backward / forward direction */
} qsl_trace_io;

/* Scheduling of a trace launch (host struct; pointers are device pointers). */
typedef struct qsl_sched {
    int32_t schedule;            /* qsl_schedule */
    int32_t chunk;               /* QUEUE: lines a warp takes per refill (0 = 256) */
    const uint32_t *order;       /* optional: line k traces seed order[k] and writes its outputs at
                                    order[k] (a permutation of [0, n)); visiting seeds in compact
                                    tiles keeps a warp's gathers coherent */
    unsigned long long *queue;   /* optional 8-byte work counter; when null one is allocated on
                                    `stream` (stream-ordered) and freed after the launch */
    unsigned long long *samples; /* optional: accumulates the number of trilinear field samples */
    int32_t occupancy;           /* fast kernels: register budget for this many resident 128-thread
                                    blocks per SM (0 = compiler's choice, or 6, 7, 8, 9, 10) */
} qsl_sched;

/* Traces n seeds (or *n_dev seeds when n_dev is set; then the outputs must
 * hold n, the largest possible count).  cross_dir_h: the seed-plane normal
 * (host, 3 floats; null = z).  curB*: current density for the twist
 * integral, or null.  sched_h: null = QUEUE with defaults. */
int qsl_trace(const qsl_field_t *field, const qsl_trace_params *params_h, const qsl_trace_io *io_h, int64_t n,
              const unsigned long long *n_dev, float s_len, float tol_coef, const float *cross_dir_h,
              const float *curBx, const float *curBy, const float *curBz, const qsl_sched *sched_h,
              qsl_stream_t stream);

/* qsl_trace with the twist integral's current density held in a store of
 * the field's own layout and shape (qsl_field_create of curl B): one current
 * sample then costs what a field sample costs, instead of 24 scalar gathers
 * from the caller's arrays (TraceBlineAdaptive.cu:373-377 samples it at
 * every step).  io_h->twist receives the integral. */
int qsl_trace_cur(const qsl_field_t *field, const qsl_field_t *cur, const qsl_trace_params *params_h,
                  const qsl_trace_io *io_h, int64_t n, const unsigned long long *n_dev, float s_len, float tol_coef,
                  const float *cross_dir_h, const qsl_sched *sched_h, qsl_stream_t stream);

/* ------------------------------------------------------------------------
 * Batched trace plans (no reference counterpart: the reference launches one
 * kernel per seed set).  Many jobs — different fields (any store), seed
 * sets, RK4/RKF45 settings — traced by one launch per store type, each job's
 * lines in their own warp-aligned range.  qsl_batch_create uploads the job
 * table once (synchronises `stream`); qsl_batch_launch only launches kernels,
 * so it can be replayed or captured into a CUDA graph.  Jobs use fast
 * arithmetic; outputs as qsl_trace.
 * ------------------------------------------------------------------------ */
typedef struct qsl_batch_job {
    const qsl_field_t *field;
    qsl_trace_params params;  /* arith must be QSL_ARITH_FAST */
    qsl_trace_io io;
    int64_t n;
    float s_len;
    float tol_coef;
    float cross_dir[3];
    const float *curB[3];     /* twist current density, or nulls */
    const uint32_t *order;    /* optional seed visiting order (tile order) */
    const unsigned long long *n_dev; /* optional: seed count on the device (<= n, which sizes the range) */
} qsl_batch_job;
typedef struct qsl_batch qsl_batch_t;

/* Stateless form for callers that manage their own memory (a serving loop
 * must not synchronise): qsl_batch_pack serialises the job table into a host
 * buffer (table_h null: only fills info, including table_bytes); the caller
 * copies those bytes to device memory (256-byte aligned) by any means and
 * qsl_batch_run launches from it.  The table holds device addresses of the
 * jobs' fields and buffers, which must stay valid until the run completes. */
/* Per store type (index = enum qsl_layout): offsets into the table, lines
 * and job counts. */
typedef struct qsl_batch_info {
    int64_t jobs_offset[4], begin_offset[4], total[4];
    int32_t njobs[4], twist[4];
    int64_t table_bytes, lines;
} qsl_batch_info;
int qsl_batch_pack(const qsl_batch_job *jobs_h, int njobs, void *table_h, int64_t table_bytes,
                   qsl_batch_info *info_h);
/* qsl_batch_run over the lines [line_lo, line_hi) of each store type's line
 * space (line_hi < 0: to the end; line_lo a multiple of 32 keeps each warp
 * inside one job) with at most max_blocks resident 128-thread blocks per
 * launch (0 = no limit; the blocks then loop over the lines).  A serving loop
 * runs a large batch as a sequence of such windows, so that small requests
 * never share the GPU with more than a window of it, and caps its resident
 * blocks below the GPU's capacity.  occupancy: the register budget of the
 * batched kernels, for this many resident 128-thread blocks per SM (6-10;
 * 0 = 8). */
int qsl_batch_run_window(const void *table_dev, const qsl_batch_info *info_h, unsigned long long *samples_dev,
                         int64_t line_lo, int64_t line_hi, int max_blocks, int occupancy, qsl_stream_t stream);
int qsl_batch_run(const void *table_dev, const qsl_batch_info *info_h, unsigned long long *samples_dev,
                  qsl_stream_t stream);

int qsl_batch_create(const qsl_batch_job *jobs_h, int njobs, qsl_stream_t stream, qsl_batch_t **out_h);
int qsl_batch_launch(const qsl_batch_t *batch, unsigned long long *samples_dev, qsl_stream_t stream);
int64_t qsl_batch_lines(const qsl_batch_t *batch);
int qsl_batch_destroy(qsl_batch_t *batch);

/* ------------------------------------------------------------------------
 * Scott deviation-vector tracer: position plus two deviation vectors along
 * each line (RKF45 on 9 components), Q from the deviation vectors at both
 * footpoints (q_0: face-projected, q_perp: perpendicular-projected).
 * ------------------------------------------------------------------------ */
enum qsl_grad_mode {
    QSL_GRAD_FD = 0,       /* grad(B/|B|) by +-1e-3 central differences (reference) */
    QSL_GRAD_ANALYTIC = 1  /* exact derivative of the trilinear unit field, one cell fetch */
};

typedef struct qsl_scott_io {
    const float *inp_x, *inp_y, *inp_z;
    float *start_x, *start_y, *start_z;
    int *flag_start;
    float *end_x, *end_y, *end_z;
    int *flag_end;
    float *B_this_x, *B_this_y, *B_this_z;
    float *q_0, *q_perp;
    double *LineLen;
    double *twist; /* needed when curB is given */
} qsl_scott_io;

/* ------------------------------------------------------------------------
 * Stretched (rectilinear) grids — fastqslpy/cu/TraceBlineAdaptiveStretch.cu
 * ------------------------------------------------------------------------ */

/* Reference settings of the stretched-grid tracer (TraceBlineAdaptiveStretch.cu
 * :10-12,336-371): the RKF45 settings with len_ratio 2 applied to the summed
 * coordinate extents, no step limit (2^31-1 here), exit-segment twist term. */
void qsl_params_reference_stretch(qsl_trace_params *p_h);

/* Replaces TraceAllBline of fastqslpy/cu/TraceBlineAdaptiveStretch.cu:422-433
 * (compiled at run time by demo/Q_RKF45CuPyStretch.ipynb cell 9): the same 39
 * arguments in order — the field, BshapeN, the node coordinates x_arr[nx],
 * y_arr[ny], z_arr[nz] (increasing) and *flag_uni (true: the uniform-spacing
 * index formula instead of the search) before the twist arguments — with
 * arith in front and capacity (length of the per-seed arrays, -1 unknown) and
 * the stream behind.  Cells are found exactly as the reference does, including
 * its search's choice of the cell below the point near the top of its last
 * interval.  The footpoint of a direction that exits through a face is placed
 * on the plane q = 0 or q = n of the exit axis in INDEX units, as the
 * reference's exit code does (:375-400). */
int qsl_trace_all_bline_stretch(int arith, const float *Bx, const float *By, const float *Bz, const int *BshapeN,
                                const float *x_arr, const float *y_arr, const float *z_arr, const bool *flag_uni,
                                const float *curB_x, const float *curB_y, const float *curB_z, double *twist,
                                const bool *curB_flag, const float *inp_x, const float *inp_y, const float *inp_z,
                                const float *inp_cross_dir, float *start_x, float *start_y, float *start_z,
                                int *flag_start, float *end_x, float *end_y, float *end_z, int *flag_end,
                                float *B_this_x, float *B_this_y, float *B_this_z, int *B_flag, float *B_start_x,
                                float *B_start_y, float *B_start_z, float *B_end_x, float *B_end_y, float *B_end_z,
                                const float *s_len, const unsigned long long *N, double *LineLen,
                                const float *tol_coef, int64_t capacity, qsl_stream_t stream);

/* Native form: host scalars and settings; Bx/By/Bz of shape nx x ny x nz (x
 * fastest) on the device, the node coordinates (strictly increasing) on the
 * HOST (nx + ny + nz floats); uni as above.  The per-axis constants of the
 * cell location (first and last coordinate, their 1e-6 offsets, the
 * uniform spacing, the search-table bin width) and the length limit are
 * formed on the host, in the same arithmetic as the drop-in forms them on
 * the device, and reach the kernels as parameters.  sched may be NULL
 * (static one-line-per-thread grid) or give the schedule, order map, sample
 * counter and occupancy (4, 5 or 6: the register budget for that many
 * resident blocks per SM of the fast packed kernels, 5 by default; 6 or the
 * default for the fast kernels on the arrays; 0 or any other value: the
 * default).  The call allocates, stream-ordered on `stream`
 * (cudaMallocAsync, freed after the launch), a device copy of the
 * coordinates (copied from the host arrays before the call returns) and, in
 * fast arithmetic, a copy of the nodes as x-pair records (node o and o + 1
 * as two float4, 32 B per node; fewer than 2^31 nodes, else the arrays)
 * and, for the search, per-axis search tables (144 B per cell of each axis);
 * the outputs equal the drop-in's (fast arithmetic) bit for bit. */
int qsl_trace_stretch(const float *Bx, const float *By, const float *Bz, int nx, int ny, int nz,
                      const float *x_arr_h, const float *y_arr_h, const float *z_arr_h, int uni,
                      const qsl_trace_params *prm, const qsl_trace_io *io, int64_t n, float s_len, float tol_coef,
                      const float *cross_dir_h, const float *curBx, const float *curBy, const float *curBz,
                      const qsl_sched *sched_h, qsl_stream_t stream);

/* curl B of a field (x fastest, nx x ny x nz) on node coordinates x_arr,
 * y_arr, z_arr (device; 0..n-1 for the integer grid) by the reference's
 * three-point non-uniform difference with its boundary copy
 * (fastqslpy/FastQSL.py:120-163, curl_of_B_grid): float32 arithmetic in the
 * reference's order, float64 outputs.  Needs at least 3 nodes per axis. */
int qsl_curl_grid(const float *Bx, const float *By, const float *Bz, int nx, int ny, int nz, const float *x_arr,
                  const float *y_arr, const float *z_arr, double *curl_x, double *curl_y, double *curl_z,
                  qsl_stream_t stream);

/* ------------------------------------------------------------------------
 * Field-line polylines — fastqslpy/MagTool.py (trilerp :3-18, Bnorm :20-22,
 * RK4_bline :24-34, TraceBline :36-45)
 * ------------------------------------------------------------------------ */

/* RK4_bline for n seeds at once (seeds: device float64, n x 3): from each
 * seed, fixed steps of dr along the unit field (float64 arithmetic in that
 * function's order), storing the point reached before each step as float32
 * at out_*[s * out_len + idx] for idx = start, start + stride, ... (Python
 * range(start, stop, stride)), until a coordinate leaves [0, nx].  Entries
 * not visited are left as they are (TraceBline's arrays start as NaN; it
 * runs range(maxstep/2, maxstep, 1) with dr = 0.25, then
 * range(maxstep/2, 0, -1) with dr = -0.25).  Every visited index must lie in
 * [0, out_len). */
int qsl_trace_path(const float *Bx, const float *By, const float *Bz, int nx, int ny, int nz, const double *seeds,
                   int64_t n, int64_t start, int64_t stop, int64_t stride, double dr, float *out_x, float *out_y,
                   float *out_z, int64_t out_len, qsl_stream_t stream);

/* trilerp (normalize = 0) or Bnorm (normalize = 1) at n points (device
 * float64, n x 3) with MagTool's clamping; out: device float64, n x 3. */
int qsl_sample_points(const float *Bx, const float *By, const float *Bz, int nx, int ny, int nz, const double *pts,
                      int64_t n, int normalize, double *out, qsl_stream_t stream);

/* ------------------------------------------------------------------------
 * Hybrid finite-difference + Scott Q — demo/Q_RKF45MixCuPyDiffScott.ipynb cell 9
 * ------------------------------------------------------------------------ */

/* Lists the seeds of the interior pixels of nplanes stacked (n0, n1) planes
 * whose finite-difference Q (Q, shape nplanes x (n0-2) x (n1-2), from
 * qsl_qcalc_plane) is unusable: B_flag set at the seed, or Q NaN.  seeds
 * (device, capacity nplanes*(n0-2)*(n1-2)) receives their seed indices in no
 * particular order, *count_dev (device) their number; nothing is read back to
 * the host.  Feed them to qsl_trace_scott as its order map with count_dev as
 * the line count, then call qsl_hybrid_merge. */
int qsl_hybrid_select(const int *B_flag, const double *Q, int n0, int n1, int64_t nplanes, unsigned *seeds,
                      unsigned long long *count_dev, qsl_stream_t stream);

/* Q of every interior pixel selected as above becomes q_perp at its seed
 * (float, seed-indexed, the Scott tracer's output). */
int qsl_hybrid_merge(const int *B_flag, const float *q_perp, int n0, int n1, int64_t nplanes, double *Q,
                     qsl_stream_t stream);

/* Reference settings of the Scott tracer (TraceBlineScott.cu:10-14): absolute
 * tolerance 1e-3*tol_coef (its tolerance variable is never initialised,
 * :352,378), length limit 2*(nx+ny+nz), 10000 steps over both directions. */
void qsl_params_reference_scott(qsl_trace_params *p_h);

/* Replaces TraceAllBlineScott (fastqslpy/cu/TraceBlineScott.cu:521-528),
 * compiled at run time by the reference's Scott notebooks: same 30 arguments
 * in order, plus capacity (the length of the per-seed arrays; required) and
 * the stream.  Exact arithmetic, central-difference gradient. */
int qsl_trace_all_bline_scott(const float *Bx, const float *By, const float *Bz, const int *BshapeN,
                              const float *curB_x, const float *curB_y, const float *curB_z, double *twist,
                              const bool *curB_flag, const float *inp_x, const float *inp_y, const float *inp_z,
                              const float *inp_cross_dir, float *start_x, float *start_y, float *start_z,
                              int *flag_start, float *end_x, float *end_y, float *end_z, int *flag_end,
                              float *B_this_x, float *B_this_y, float *B_this_z, float *q_0_arr, float *q_perp_arr,
                              const float *s_len, const unsigned long long *N, double *LineLen,
                              const float *tol_coef, int64_t capacity, qsl_stream_t stream);

/* Native Scott entry: any store, exact (SoA + QSL_GRAD_FD only) or fast
 * arithmetic, either gradient.  sched_h: order / samples are used (the
 * schedule is one line per thread). */
int qsl_trace_scott(const qsl_field_t *field, const qsl_trace_params *params_h, const qsl_scott_io *io_h,
                    int64_t n, const unsigned long long *n_dev, float s_len, float tol_coef, const float *curBx,
                    const float *curBy, const float *curBz, int grad_mode, const qsl_sched *sched_h,
                    qsl_stream_t stream);

/* ------------------------------------------------------------------------
 * Q assembly.
 * ------------------------------------------------------------------------ */

/* Replaces fastqslpy/FastQSL.py:65-117 (QCalcPlane).  Inputs are nplanes
 * stacked (n0, n1) row-major planes; Q is (nplanes, n0-2, n1-2).
 * jac_scale = (1/(2*stride_step))^4.  Give exactly one of Q32 (the
 * reference's FP32 rounding) or Q64 (FP64).  Bz_in / Bz_out are Bz at the
 * start / end footpoints (the reference uses the z component whatever the
 * exit face, FastQSL.py:112-113). */
int qsl_qcalc_plane(const float *x_end, const float *y_end, const float *z_end, const int *flag_end,
                    const float *x_start, const float *y_start, const float *z_start, const int *flag_start,
                    const float *Bz_in, const float *Bz_out, const float *Bx_0, const float *By_0,
                    const float *Bz_0, int n0, int n1, int64_t nplanes, double jac_scale,
                    const float *cross_dir_h, float *Q32, double *Q64, qsl_stream_t stream);

/* Replaces the seed construction of fastqslpy/FastQSL.py:4-57
 * (CookPseudoLine): for every pixel with B_flag == 1 (row-major order; only
 * interior pixels of each (n0, n1) plane when interior_only), four seeds
 * around its start footpoint, +-stride along the start face's two axes in
 * the order (+u, +v, -u, -v).  Outputs must hold 4n seeds and n pixels;
 * count_dev[0] receives the pixel count and count_dev[1] the seed count
 * (4 per pixel, usable as the n_dev of qsl_trace).  workspace: device scratch of
 * qsl_cook_workspace_bytes(n) bytes. */
int64_t qsl_cook_workspace_bytes(int64_t n);
int qsl_cook_pseudo_line(const int *B_flag, const float *x_start, const float *y_start, const float *z_start,
                         const int *flag_start, const float *Bz_in, const float *Bz_out, int64_t n, int n0, int n1,
                         int interior_only, float stride, float *cut_x, float *cut_y, float *cut_z,
                         float *Bz0_start, float *Bz0_end, int64_t *pix, unsigned long long *count_dev,
                         void *workspace, int64_t workspace_bytes, qsl_stream_t stream);

/* qsl_cook_pseudo_line without a workspace argument.  This entry has no
 * counterpart in the reference.  It is for callers that cannot allocate
 * device memory: a host application whose allocator has reserved the GPU's
 * memory for its own pool (nothing is left to cudaMalloc, and the pool is not
 * exposed to plug-ins), and language bindings that only receive borrowed
 * device pointers from their host runtime and have no device allocator of
 * their own.  The compaction scratch (12 bytes per 1024 pixels) is a fixed
 * array of QSL_NOALLOC_SCRATCH_BYTES inside this library, present on every
 * GPU that loads the library until the process exits; n is limited to
 * qsl_cook_noalloc_max_pixels() (about 358 million pixels) and larger
 * requests return QSL_ERR_TOO_LARGE.  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress) with that device current;
 * make that first call before any stream capture.  A call that finds a
 * different current context on the device (after cudaDeviceReset) looks the
 * address up again, so make the first call after a reset outside a capture
 * too.  All calls on a device
 * share the one array: calls whose work overlaps on the GPU (other streams,
 * other host threads) race and must be serialised by the caller.  The
 * entry allocates nothing: no cudaMalloc, cudaFree or allocating library
 * routine.  Outputs and count_dev are as for qsl_cook_pseudo_line. */
#define QSL_NOALLOC_SCRATCH_BYTES (4LL << 20)
int64_t qsl_cook_noalloc_max_pixels(void);
int qsl_cook_pseudo_line_noalloc(const int *B_flag, const float *x_start, const float *y_start, const float *z_start,
                                 const int *flag_start, const float *Bz_in, const float *Bz_out, int64_t n, int n0,
                                 int n1, int interior_only, float stride, float *cut_x, float *cut_y, float *cut_z,
                                 float *Bz0_start, float *Bz0_end, int64_t *pix, unsigned long long *count_dev,
                                 qsl_stream_t stream);

/* Replaces demo/Q_RKF45CuPy.ipynb cell 10: Q of each pseudo-line pixel from
 * its 4 traced pseudo-lines; jac_scale = (1/(2*stride))^4.  The pixel count
 * is `count`, or *count_dev when set (then max_count bounds the launch). */
int qsl_qcut(const float *start_x, const float *start_y, const float *start_z, const int *flag_start,
             const float *end_x, const float *end_y, const float *end_z, const int *flag_end,
             const float *Bz0_start, const float *Bz0_end, int64_t count, const unsigned long long *count_dev,
             int64_t max_count, double jac_scale, float *Qcut32, double *Qcut64, qsl_stream_t stream);

/* Replaces demo/Q_RKF45CuPy.ipynb cell 11: Qfinal (nplanes, n0-2, n1-2) gets
 * Qcut at every compacted interior pixel `pix`. */
int qsl_qmerge(const int64_t *pix, const float *Qcut32, const double *Qcut64, int64_t count,
               const unsigned long long *count_dev, int64_t max_count, int n0, int n1, float *Qfinal32,
               double *Qfinal64, qsl_stream_t stream);

/* Seed grid of nplanes stacked (n0, n1) planes (no reference counterpart:
 * the notebooks build their seed planes with cupy.linspace / meshgrid on the
 * host side of the kernel call, demo/Q_RKF45CuPy.ipynb cell 7).  Seed
 * q = (k * n0 + i) * n1 + j, written as float32 to xs, ys, zs, is
 *   ((center + (k s) normal) + ((i - (n0-1)/2) s) v) + ((j - (n1-1)/2) s) u
 * with s = spacing, each product and sum rounded in double on its own, then
 * rounded to float (the same values as that expression evaluated one
 * array operation at a time in double).  center, normal, u, v: 3 doubles on
 * the HOST.  One launch on `stream`. */
int qsl_plane_seeds(const double *center_h, const double *normal_h, const double *u_h, const double *v_h,
                    double spacing, int n0, int n1, int nplanes, float *xs, float *ys, float *zs,
                    qsl_stream_t stream);

/* ------------------------------------------------------------------------
 * Native Q-map batches (no reference counterpart: the reference's notebooks
 * run one Q map at a time, demo/Q_RKF45CuPy.ipynb cells 7-11, with the
 * RKF45 kernel TraceBlineAdaptive.cu:429-510 and FastQSL.py:4-117).  The
 * whole plane Q pipeline of many jobs laid out in one caller-provided
 * workspace and queued from the host library: per job its seed grid
 * (qsl_plane_seeds) and tile order (qsl_tile_order), one batched main trace
 * (or windows of it), then per job Q (qsl_qcalc_plane, FP64) and the
 * pseudo-line compaction (qsl_cook_pseudo_line), one batched pseudo-line
 * trace, per job pseudo Q and merge (qsl_qcut, qsl_qmerge).  The Q maps
 * equal a batch of the same jobs built from those entries one by one, bit
 * for bit.  No device allocation, no synchronisation; a serving loop builds
 * a batch of small requests in a few launches per request.
 * ------------------------------------------------------------------------ */
typedef struct qsl_qmap_job {
    const qsl_field_t *field;
    qsl_trace_params params;   /* arith must be QSL_ARITH_FAST */
    double center[3];          /* plane k at center + k spacing normal */
    double normal[3];          /* unit normal: the plane step and the Q cross direction */
    double u[3], v[3];         /* in-plane unit axes: columns along u, rows along v */
    double spacing;            /* seed spacing within and between planes (the Q stride) */
    int32_t n0, n1, nplanes;   /* rows, columns (>= 3 each), planes (>= 1); at most 2^32 seeds */
    int32_t tile_y, tile_x;    /* seed tile of the trace order (0: seed order) */
    float s_len, tol_coef;
} qsl_qmap_job;
typedef struct qsl_qmap_batch qsl_qmap_batch_t;

/* Bytes a batch of these jobs needs: device workspace (its arrays and job
 * tables) and pinned host staging (the job tables on their way to the
 * device). */
int qsl_qmap_batch_size(const qsl_qmap_job *jobs, int njobs, int64_t *device_bytes, int64_t *host_bytes);
/* Lays the batch out in `workspace` (device, 256-byte aligned, at least
 * device_bytes) and queues on `stream` the seed grids, the tile orders and
 * the host-to-device copy of the job tables from `host_staging` (host, at
 * least host_bytes, pinned for an asynchronous copy; it must stay untouched
 * until the stream has passed the copy).  *out: a host handle. */
int qsl_qmap_batch_create(const qsl_qmap_job *jobs, int njobs, void *workspace, int64_t workspace_bytes,
                          void *host_staging, int64_t host_bytes, qsl_stream_t stream, qsl_qmap_batch_t **out);
/* End of the batched main trace's line space (for windows). */
int64_t qsl_qmap_batch_lines(const qsl_qmap_batch_t *batch);
/* The batched main trace over lines [line_lo, line_hi) (line_hi < 0: to the
 * end), max_blocks / occupancy as in qsl_batch_run_window. */
int qsl_qmap_batch_run_main(const qsl_qmap_batch_t *batch, int64_t line_lo, int64_t line_hi, int max_blocks,
                            int occupancy, qsl_stream_t stream);
/* Everything after the main trace: Q, pseudo-lines and merge of every job
 * (the Q assembly, compaction, pseudo Q and merge as one launch each for
 * the whole batch, the pseudo-line trace as one batched trace). */
int qsl_qmap_batch_run_post(const qsl_qmap_batch_t *batch, int max_blocks, int occupancy, qsl_stream_t stream);
/* Device address of job k's Q, float64 (nplanes, n0 - 2, n1 - 2) inside the workspace. */
double *qsl_qmap_batch_q(const qsl_qmap_batch_t *batch, int job);
/* Frees the host handle (the workspace belongs to the caller). */
int qsl_qmap_batch_destroy(qsl_qmap_batch_t *batch);

/* Tile visiting order of nplanes stacked (n0, n1) seed planes (seed index
 * (p * n0 + y) * n1 + x), the `order` map of qsl_sched / qsl_batch_job:
 * order[k] = the seed visited k-th when the seeds are sorted by (plane
 * group, y / ty, x / tx, plane within the group, y % ty, x % tx); groups of
 * plane_group consecutive planes (<= 0 or >= nplanes: one group of all
 * planes).  Tiles at the far edges are smaller.  nplanes * n0 * n1 <= 2^32.
 * One launch on `stream`. */
int qsl_tile_order(int nplanes, int n0, int n1, int ty, int tx, int plane_group, uint32_t *order,
                   qsl_stream_t stream);

/* Measurement helper with no reference counterpart: the L1 ceiling of the
 * tracers' 16-byte field gathers.  Launches `blocks` blocks of 128 threads;
 * each thread issues 8 * iters 16-byte read-only loads from `buf`
 * (buf_bytes: a power of two from 4 KiB, small enough to stay in L1; the
 * caller zeroes it), each warp request spread over `spread` 128-byte lines
 * (1, 2, 4 = coalesced 512 bytes, 8, 16 or 32).  The caller times the launch
 * on `stream`; bytes loaded = blocks * 128 * 8 * iters * 16.  `sink`: one
 * device word the kernel may write. */
int qsl_l1_probe(const void *buf, int64_t buf_bytes, int spread, int blocks, int iters, unsigned *sink,
                 qsl_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif
