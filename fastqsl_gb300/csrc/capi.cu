// C ABI of fastqsl_gb300 (declarations and contracts in
// include/fastqsl_gb300.h).
#include <climits>
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <mutex>
#include <new>
#include <vector>

#include "../../include/fastqsl_gb300.h"
#include "qassembly.h"
#include "qsl_internal.h"

using namespace qsl;

static thread_local char g_err[512];

static int fail(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

static int cuda_fail(cudaError_t e, const char* what) {
    return fail(e == cudaErrorMemoryAllocation ? QSL_ERR_NOMEM : QSL_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define QSL_CHECK_CUDA(expr, what)                  \
    do {                                            \
        cudaError_t e_ = (expr);                    \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

namespace qsl {

// Lets other translation units of the library report an error through
// qsl_last_error().
int set_error(int code, const char* msg) { return fail(code, "%s", msg); }

int persistent_grid(const void* kernel, int block, size_t smem) {
    int dev = 0, sms = 0, per = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, block, smem) != cudaSuccess) return -1;
    if (per < 1) per = 1;
    return sms * per;
}

}  // namespace qsl

extern "C" {

const char* qsl_last_error(void) { return g_err; }

const char* qsl_version(void) { return "fastqsl_gb300 0.1 (sm_103a)"; }

void qsl_params_reference_rk4(qsl_trace_params* p) {
    p->integrator = QSL_RK4;
    p->tol_law = QSL_TOL_REFERENCE;
    p->tol = 1e-3;
    p->h_min = 0.1;
    p->h_max = 100.0;
    p->reject_factor = 0.618;
    p->len_ratio = 2.0;
    p->max_steps = 100000;
    p->boundary_twist = 1;
    p->arith = QSL_ARITH_EXACT;
    p->max_rejects = 0;
}

void qsl_params_reference_rkf45(qsl_trace_params* p) {
    p->integrator = QSL_RKF45;
    p->tol_law = QSL_TOL_REFERENCE;
    p->tol = 1e-3;
    p->h_min = 0.1;
    p->h_max = 100.0;
    p->reject_factor = 0.618;
    p->len_ratio = 3.0;
    p->max_steps = 500000;
    p->boundary_twist = 0;
    p->arith = QSL_ARITH_EXACT;
    p->max_rejects = 0;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Field stores
// ---------------------------------------------------------------------------
struct qsl_field {
    int layout;
    Dims d;
    const float *bx, *by, *bz;  // SOA only: the caller's arrays (borrowed)
    float4* f4;
    uint4* bricks;
    float* scale;
    uint4* cells;  // H8C records
    int nbx, nby, nbz;
    int64_t bytes;
    int device;
};

static int64_t layout_bytes(int nx, int ny, int nz, int layout, int* nbx, int* nby, int* nbz) {
    const int bx = (nx - 1 + BRICK_CELLS - 1) / BRICK_CELLS, by = (ny - 1 + BRICK_CELLS - 1) / BRICK_CELLS,
              bz = (nz - 1 + BRICK_CELLS - 1) / BRICK_CELLS;
    if (nbx) *nbx = bx;
    if (nby) *nby = by;
    if (nbz) *nbz = bz;
    const int64_t nodes = (int64_t)nx * ny * nz;
    switch (layout) {
        case LAYOUT_SOA: return 0;
        case LAYOUT_F4: return nodes * (int64_t)sizeof(float4);
        case LAYOUT_H4B: {
            const int64_t nb = (int64_t)bx * by * bz;
            return nb * BRICK_U4 * (int64_t)sizeof(uint4) + nb * (int64_t)sizeof(float);
        }
        case LAYOUT_H8C: return (int64_t)bx * by * bz * 512 * CELL_RECORD_U4 * (int64_t)sizeof(uint4);
        default: return -1;
    }
}

static bool dims_ok(int nx, int ny, int nz) {
    if (nx < 2 || ny < 2 || nz < 2) return false;
    // 32-bit cell coordinates and brick indices; 2^40 nodes is far beyond HBM.
    return (double)nx * ny * nz < 1.1e12;
}

extern "C" {

int64_t qsl_field_store_bytes(int nx, int ny, int nz, int layout) {
    if (!dims_ok(nx, ny, nz)) return fail(QSL_ERR_INVALID, "bad field shape %d x %d x %d", nx, ny, nz);
    const int64_t b = layout_bytes(nx, ny, nz, layout, nullptr, nullptr, nullptr);
    if (b < 0) return fail(QSL_ERR_INVALID, "unknown layout %d", layout);
    return b;
}

int qsl_field_create(const float* Bx, const float* By, const float* Bz, int nx, int ny, int nz, int layout,
                     qsl_stream_t stream, qsl_field_t** out) {
    if (!out) return fail(QSL_ERR_INVALID, "out is null");
    *out = nullptr;
    if (!Bx || !By || !Bz) return fail(QSL_ERR_INVALID, "null field array");
    if (!dims_ok(nx, ny, nz)) return fail(QSL_ERR_INVALID, "bad field shape %d x %d x %d", nx, ny, nz);
    int nbx, nby, nbz;
    const int64_t bytes = layout_bytes(nx, ny, nz, layout, &nbx, &nby, &nbz);
    if (bytes < 0) return fail(QSL_ERR_INVALID, "unknown layout %d", layout);
    if (layout == LAYOUT_H4B) {
        // the brick sampler forms a record index within a z-slab of bricks
        // in 32 bits (FieldH4B::ky, kz)
        const unsigned long long slab = (unsigned long long)BRICK_U4 * nbx * nby + 640ull * nbx + 64ull * nby +
                                        576ull * nbz;
        if (slab >= (1ull << 32))
            return fail(QSL_ERR_TOO_LARGE, "field too wide for fp16 bricks (%d x %d nodes per z-slab)", nx, ny);
    }
    qsl_field* f = new (std::nothrow) qsl_field();
    if (!f) return fail(QSL_ERR_NOMEM, "host allocation failed");
    f->layout = layout;
    f->d = Dims{nx, ny, nz};
    f->bytes = bytes;
    f->nbx = nbx;
    f->nby = nby;
    f->nbz = nbz;
    cudaGetDevice(&f->device);
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaSuccess;
    if (layout == LAYOUT_SOA) {
        f->bx = Bx;
        f->by = By;
        f->bz = Bz;
    } else if (layout == LAYOUT_F4) {
        e = cudaMalloc(&f->f4, (size_t)bytes);
        if (e == cudaSuccess) e = launch_pack_f4(Bx, By, Bz, f->d, f->f4, st);
    } else if (layout == LAYOUT_H4B) {
        const int64_t nb = (int64_t)nbx * nby * nbz;
        e = cudaMalloc(&f->bricks, (size_t)(nb * BRICK_U4 * sizeof(uint4)));
        if (e == cudaSuccess) e = cudaMalloc(&f->scale, (size_t)(nb * sizeof(float)));
        if (e == cudaSuccess) e = launch_pack_h4b(Bx, By, Bz, f->d, nbx, nby, nbz, f->bricks, f->scale, st);
    } else {
        e = cudaMalloc(&f->cells, (size_t)bytes);
        if (e == cudaSuccess) e = launch_pack_h8c(Bx, By, Bz, f->d, nbx, nby, nbz, f->cells, st);
    }
    if (e != cudaSuccess) {
        cudaFree(f->f4);
        cudaFree(f->bricks);
        cudaFree(f->scale);
        cudaFree(f->cells);
        delete f;
        return cuda_fail(e, "qsl_field_create");
    }
    *out = f;
    return QSL_OK;
}

int qsl_field_destroy(qsl_field_t* f) {
    if (!f) return QSL_OK;
    cudaFree(f->f4);
    cudaFree(f->bricks);
    cudaFree(f->scale);
    cudaFree(f->cells);
    delete f;
    return QSL_OK;
}

int64_t qsl_field_bytes(const qsl_field_t* f) { return f ? f->bytes : 0; }

int qsl_field_update(qsl_field_t* f, const float* Bx, const float* By, const float* Bz, qsl_stream_t stream) {
    if (!f || !Bx || !By || !Bz) return fail(QSL_ERR_INVALID, "null argument");
    cudaStream_t st = (cudaStream_t)stream;
    if (f->layout == LAYOUT_SOA) {
        f->bx = Bx;
        f->by = By;
        f->bz = Bz;
        return QSL_OK;
    }
    cudaError_t e = f->layout == LAYOUT_F4    ? launch_pack_f4(Bx, By, Bz, f->d, f->f4, st)
                    : f->layout == LAYOUT_H4B ? launch_pack_h4b(Bx, By, Bz, f->d, f->nbx, f->nby, f->nbz, f->bricks,
                                                                f->scale, st)
                                              : launch_pack_h8c(Bx, By, Bz, f->d, f->nbx, f->nby, f->nbz, f->cells, st);
    if (e != cudaSuccess) return cuda_fail(e, "qsl_field_update");
    return QSL_OK;
}

}  // extern "C"

// device views of a store
static FieldSoA soa_of(const qsl_field* f) { return FieldSoA{f->bx, f->by, f->bz, f->d}; }
static FieldF4 f4_of(const qsl_field* f) { return FieldF4{f->f4, f->d}; }
static FieldH4B h4b_of(const qsl_field* f) {
    return FieldH4B{f->bricks, f->scale, f->d, f->nbx, f->nby, (unsigned)(BRICK_U4 * f->nbx - 64),
                    (unsigned)((unsigned long long)BRICK_U4 * f->nbx * f->nby - 576)};
}
static FieldH4BW h4bw_of(const qsl_field* f) { return FieldH4BW{h4b_of(f)}; }
static FieldH8C h8c_of(const qsl_field* f) { return FieldH8C{f->cells, f->d, f->nbx, f->nby}; }

// The per-launch constants of a packed stretched store, formed on the host
// from the host coordinates in the arithmetic store_prepare uses on the
// device for the drop-in (so both give the same bits): first and last node
// coordinates, the clamp bounds 1e-6 inside them (double, narrowed), the
// uniform-formula spacing (hi - lo) / n and the search-table bins per unit
// coordinate.
template <int M>
static void stretch_constants_host(FieldStretchT<M>& f, const float* ax, const float* ay, const float* az) {
    const int n[3] = {f.d.nx, f.d.ny, f.d.nz};
    const float* a[3] = {ax, ay, az};
    float lo[3], hi[3], clo[3], chi[3], us[3], binv[3];
    for (int k = 0; k < 3; ++k) {
        lo[k] = a[k][0];
        hi[k] = a[k][n[k] - 1];
        clo[k] = (float)((double)lo[k] + 1e-6);
        chi[k] = (float)((double)hi[k] - 1e-6);
        us[k] = (hi[k] - lo[k]) / (float)n[k];
        // tables: bins per unit coordinate; uniform formula: 1 / us (as
        // store_prepare forms them on the device)
        binv[k] = (M == 2 || M == 4) ? 1.0f / us[k] : (float)(STRETCH_BINS_PER_CELL * (n[k] - 1)) / (hi[k] - lo[k]);
    }
    f.lo = make_float3(lo[0], lo[1], lo[2]);
    f.hi = make_float3(hi[0], hi[1], hi[2]);
    f.clo = make_float3(clo[0], clo[1], clo[2]);
    f.chi = make_float3(chi[0], chi[1], chi[2]);
    f.us = make_float3(us[0], us[1], us[2]);
    f.sbinv = make_float3(binv[0], binv[1], binv[2]);
}
// the summed coordinate extents, as len_scale forms them on the device
template <int M>
static double stretch_len_scale_host(const FieldStretchT<M>& f) {
    return (double)(((f.hi.x + f.hi.y) + f.hi.z) - ((f.lo.x + f.lo.y) + f.lo.z));
}

// ---------------------------------------------------------------------------
// Tracing
// ---------------------------------------------------------------------------
static TraceOut make_out(const qsl_trace_io* io) {
    TraceOut o;
    o.start_x = io->start_x; o.start_y = io->start_y; o.start_z = io->start_z; o.flag_start = io->flag_start;
    o.end_x = io->end_x; o.end_y = io->end_y; o.end_z = io->end_z; o.flag_end = io->flag_end;
    o.bthis_x = io->B_this_x; o.bthis_y = io->B_this_y; o.bthis_z = io->B_this_z; o.b_flag = io->B_flag;
    o.bstart_x = io->B_start_x; o.bstart_y = io->B_start_y; o.bstart_z = io->B_start_z;
    o.bend_x = io->B_end_x; o.bend_y = io->B_end_y; o.bend_z = io->B_end_z;
    o.line_len = io->LineLen;
    o.twist = io->twist;
    o.status_start = io->status_start;
    o.status_end = io->status_end;
    return o;
}

static bool io_ok(const qsl_trace_io* io) {
    return io && io->inp_x && io->inp_y && io->inp_z && io->start_x && io->start_y && io->start_z &&
           io->flag_start && io->end_x && io->end_y && io->end_z && io->flag_end && io->B_this_x && io->B_this_y &&
           io->B_this_z && io->B_flag && io->B_start_x && io->B_start_y && io->B_start_z && io->B_end_x &&
           io->B_end_y && io->B_end_z && io->LineLen;
}

static bool params_ok(const qsl_trace_params* p) {
    return p && (p->integrator == QSL_RK4 || p->integrator == QSL_RKF45) &&
           (p->tol_law == QSL_TOL_REFERENCE || p->tol_law == QSL_TOL_ABSOLUTE) &&
           (p->arith == QSL_ARITH_EXACT || p->arith == QSL_ARITH_FAST || p->arith == QSL_ARITH_FAST_W16) &&
           p->max_steps >= 0 && p->max_rejects >= 0 &&
           p->max_steps <= 0x7fffffff && p->reject_factor > 0.0 && p->reject_factor < 1.0 && p->len_ratio >= 0.0;
}

template <class F>
static int run_trace(TraceJob<F>& J, int arith, bool twist, int schedule, long long n_host,
                     unsigned long long* queue_dev, cudaStream_t st) {
    unsigned long long* q = nullptr;
    bool own = false;
    if (schedule == QSL_SCHED_QUEUE) {
        q = queue_dev;
        if (!q) {
            QSL_CHECK_CUDA(cudaMallocAsync((void**)&q, sizeof(unsigned long long), st), "queue allocation");
            own = true;
        }
        cudaError_t e = cudaMemsetAsync(q, 0, sizeof(unsigned long long), st);
        if (e != cudaSuccess) {
            if (own) cudaFreeAsync(q, st);
            return cuda_fail(e, "queue reset");
        }
    }
    J.queue = q;
    const Schedule sched = schedule == QSL_SCHED_QUEUE ? SCHED_QUEUE : SCHED_STATIC;
    cudaError_t e;
    if constexpr (std::is_same<F, FieldSoA>::value) {
        e = arith == QSL_ARITH_EXACT ? launch_trace_exact(J, twist, sched, n_host, st)
                                     : launch_trace_fast_soa(J, twist, sched, n_host, st);
    } else if constexpr (std::is_same<F, FieldF4>::value) {
        e = launch_trace_fast_f4(J, twist, sched, n_host, st);
    } else if constexpr (std::is_same<F, FieldH4B>::value) {
        e = launch_trace_fast_h4b(J, twist, sched, n_host, st);
    } else if constexpr (std::is_same<F, FieldH4BW>::value) {
        e = launch_trace_fast_h4bw(J, twist, sched, n_host, st);
    } else if constexpr (std::is_same<F, FieldStretchP>::value) {
        e = launch_trace_fast_stretch_packed(J, twist, sched, n_host, st);
    } else if constexpr (std::is_same<F, FieldStretchPU>::value) {
        e = launch_trace_fast_stretch_packed_uni(J, twist, sched, n_host, st);
    } else if constexpr (std::is_same<F, FieldStretch>::value) {
        e = arith == QSL_ARITH_EXACT ? launch_trace_exact_stretch(J, twist, sched, n_host, st)
                                     : launch_trace_fast_stretch(J, twist, sched, n_host, st);
    } else if constexpr (std::is_same<F, FieldStretchU>::value) {
        e = arith == QSL_ARITH_EXACT ? launch_trace_exact_stretch_uni(J, twist, sched, n_host, st)
                                     : launch_trace_fast_stretch_uni(J, twist, sched, n_host, st);
    } else {
        e = launch_trace_fast_h8c(J, twist, sched, n_host, st);
    }
    if (own) cudaFreeAsync(q, st);
    if (e != cudaSuccess) return cuda_fail(e, "trace launch");
    return QSL_OK;
}

template <class F>
static void fill_common(TraceJob<F>& J, const qsl_trace_io* io, const qsl_trace_params* prm,
                        unsigned long long* samples_dev) {
    J.shape_dev = nullptr;
    J.cur = FieldSoA{nullptr, nullptr, nullptr, J.f.d};
    J.inp_x = io->inp_x;
    J.inp_y = io->inp_y;
    J.inp_z = io->inp_z;
    J.o = make_out(io);
    J.prm = *prm;
    J.lim.h_min = (float)prm->h_min;
    J.lim.h_max = (float)prm->h_max;
    J.lim.reject = (float)prm->reject_factor;
    J.lim.max_steps = prm->max_steps > INT_MAX ? INT_MAX : (prm->max_steps < 0 ? 0 : (int)prm->max_steps);
    // the kernels' own product, (float)(len_ratio * (double)(nx + ny + nz))
    J.lim.len_lim = (float)(prm->len_ratio * (double)(J.f.d.nx + J.f.d.ny + J.f.d.nz));
    J.queue = nullptr;
    J.samples = samples_dev;
    J.order = nullptr;
    J.chunk = 0;
    J.occupancy = 0;
    J.cur_packed = 0;
    J.cur_store = J.f;
    memset(&J.s, 0, sizeof(J.s));
    J.s.n_cap = -1;
}

extern "C" {

extern "C++" {
static void store_view(const qsl_field_t* f, FieldSoA& s) { s = soa_of(f); }
static void store_view(const qsl_field_t* f, FieldF4& s) { s = f4_of(f); }
static void store_view(const qsl_field_t* f, FieldH4B& s) { s = h4b_of(f); }
static void store_view(const qsl_field_t* f, FieldH4BW& s) { s = h4bw_of(f); }
static void store_view(const qsl_field_t* f, FieldH8C& s) { s = h8c_of(f); }
}

// qsl_trace and qsl_trace_cur: the current density comes from the caller's
// arrays (curBx/y/z) or from a store of the field's layout (cur_field).
static int trace_impl(const qsl_field_t* field, const qsl_field_t* cur_field, const qsl_trace_params* prm,
                      const qsl_trace_io* io, int64_t n, const unsigned long long* n_dev, float s_len,
                      float tol_coef, const float* cross_dir_h, const float* curBx, const float* curBy,
                      const float* curBz, const qsl_sched* sched_h, qsl_stream_t stream) {
    qsl_sched sc{QSL_SCHED_QUEUE, 0, nullptr, nullptr, nullptr, 0};
    if (sched_h) sc = *sched_h;
    const int schedule = sc.schedule;
    unsigned long long* samples_dev = sc.samples;
    unsigned long long* queue_dev = sc.queue;
    if (sc.chunk < 0 || sc.chunk > (1 << 20)) return fail(QSL_ERR_INVALID, "chunk out of range");
    if (sc.occupancy != 0 && (sc.occupancy < 6 || sc.occupancy > 10))
        return fail(QSL_ERR_INVALID, "occupancy must be 0, 6, 7, 8, 9 or 10");
    if (sc.order && n > 0xffffffffLL) return fail(QSL_ERR_TOO_LARGE, "order map limits n to 2^32-1");
    if (!field) return fail(QSL_ERR_INVALID, "field is null");
    if (!params_ok(prm)) return fail(QSL_ERR_INVALID, "bad trace params");
    if (n < 0) return fail(QSL_ERR_INVALID, "negative seed count");
    if (n == 0) return QSL_OK;  // also bounds a device count: nothing to write
    if (!io_ok(io)) return fail(QSL_ERR_INVALID, "null pointer in trace io");
    if (schedule != QSL_SCHED_QUEUE && schedule != QSL_SCHED_STATIC)
        return fail(QSL_ERR_INVALID, "bad schedule %d", schedule);
    const bool twist = curBx != nullptr || cur_field != nullptr;
    if (curBx && (!curBy || !curBz || !io->twist)) return fail(QSL_ERR_INVALID, "twist needs curB_x/y/z and twist");
    if (cur_field) {
        if (!io->twist) return fail(QSL_ERR_INVALID, "twist needs the twist output");
        if (cur_field->layout != field->layout || cur_field->d.nx != field->d.nx || cur_field->d.ny != field->d.ny ||
            cur_field->d.nz != field->d.nz)
            return fail(QSL_ERR_INVALID, "the current store must have the field's layout and shape");
    }
    if (field->layout != LAYOUT_SOA && prm->arith == QSL_ARITH_EXACT)
        return fail(QSL_ERR_INVALID, "exact arithmetic needs the SoA layout");
    if (field->layout != LAYOUT_H4B && prm->arith == QSL_ARITH_FAST_W16)
        return fail(QSL_ERR_INVALID, "fp16 x weights (QSL_ARITH_FAST_W16) need the h4b layout");
    const float cd[3] = {cross_dir_h ? cross_dir_h[0] : 0.f, cross_dir_h ? cross_dir_h[1] : 0.f,
                         cross_dir_h ? cross_dir_h[2] : 1.f};
    cudaStream_t st = (cudaStream_t)stream;
    auto scal = [&](TraceScalars& s) {
        s.s_len = s_len;
        s.tol_coef = tol_coef;
        s.n = n;
        s.n_dev = n_dev;
        s.n_cap = n_dev ? n : -1;  // a device count never exceeds the outputs' length n
        s.cross[0] = cd[0]; s.cross[1] = cd[1]; s.cross[2] = cd[2];
        s.twist_on = twist ? 1 : 0;
    };
    const FieldSoA cur{curBx, curBy, curBz, field->d};
    auto go = [&](auto store) {
        TraceJob<decltype(store)> J;
        J.f = store;
        fill_common(J, io, prm, samples_dev);
        J.cur = cur;
        if (cur_field) {
            store_view(cur_field, J.cur_store);
            J.cur_packed = 1;
        }
        J.order = sc.order;
        J.chunk = sc.chunk;
        J.occupancy = sc.occupancy;
        scal(J.s);
        return run_trace(J, prm->arith, twist, schedule, n, queue_dev, st);
    };
    switch (field->layout) {
        case LAYOUT_SOA: return go(soa_of(field));
        case LAYOUT_F4: return go(f4_of(field));
        case LAYOUT_H4B: return prm->arith == QSL_ARITH_FAST_W16 ? go(h4bw_of(field)) : go(h4b_of(field));
        default: return go(h8c_of(field));
    }
}

int qsl_trace(const qsl_field_t* field, const qsl_trace_params* prm, const qsl_trace_io* io, int64_t n,
              const unsigned long long* n_dev, float s_len, float tol_coef, const float* cross_dir_h,
              const float* curBx, const float* curBy, const float* curBz, const qsl_sched* sched_h,
              qsl_stream_t stream) {
    return trace_impl(field, nullptr, prm, io, n, n_dev, s_len, tol_coef, cross_dir_h, curBx, curBy, curBz, sched_h,
                      stream);
}

int qsl_trace_cur(const qsl_field_t* field, const qsl_field_t* cur, const qsl_trace_params* prm,
                  const qsl_trace_io* io, int64_t n, const unsigned long long* n_dev, float s_len, float tol_coef,
                  const float* cross_dir_h, const qsl_sched* sched_h, qsl_stream_t stream) {
    if (!cur) return fail(QSL_ERR_INVALID, "current store is null");
    return trace_impl(field, cur, prm, io, n, n_dev, s_len, tol_coef, cross_dir_h, nullptr, nullptr, nullptr, sched_h,
                      stream);
}

// Drop-in entry: the reference kernel's argument list (TraceBlineAdaptive.cu:
// 429-437), scalars by device pointer.  The field is read in place (SoA).
int qsl_trace_all_bline(int integrator, int arith, const float* Bx, const float* By, const float* Bz,
                        const int* BshapeN, const float* curB_x, const float* curB_y, const float* curB_z,
                        double* twist, const bool* curB_flag, const float* inp_x, const float* inp_y,
                        const float* inp_z, const float* inp_cross_dir, float* start_x, float* start_y,
                        float* start_z, int* flag_start, float* end_x, float* end_y, float* end_z, int* flag_end,
                        float* B_this_x, float* B_this_y, float* B_this_z, int* B_flag, float* B_start_x,
                        float* B_start_y, float* B_start_z, float* B_end_x, float* B_end_y, float* B_end_z,
                        const float* s_len, const unsigned long long* N, double* LineLen, const float* tol_coef,
                        int64_t capacity, qsl_stream_t stream) {
    if (capacity == 0) return QSL_OK;  // nothing can be written
    if (!Bx || !By || !Bz || !BshapeN || !inp_cross_dir || !s_len || !N)
        return fail(QSL_ERR_INVALID, "null required pointer");
    if (integrator == QSL_RKF45 && !tol_coef) return fail(QSL_ERR_INVALID, "RKF45 needs tol_coef");
    if (arith != QSL_ARITH_EXACT && arith != QSL_ARITH_FAST) return fail(QSL_ERR_INVALID, "bad arith %d", arith);
    qsl_trace_params prm;
    if (integrator == QSL_RK4) qsl_params_reference_rk4(&prm);
    else if (integrator == QSL_RKF45) qsl_params_reference_rkf45(&prm);
    else return fail(QSL_ERR_INVALID, "bad integrator %d", integrator);
    prm.arith = arith;
    qsl_trace_io io{inp_x, inp_y, inp_z, start_x, start_y, start_z, flag_start, end_x, end_y, end_z, flag_end,
                    B_this_x, B_this_y, B_this_z, B_flag, B_start_x, B_start_y, B_start_z, B_end_x, B_end_y,
                    B_end_z, LineLen, twist};
    if (!io_ok(&io)) return fail(QSL_ERR_INVALID, "null pointer in outputs");
    // the twist code runs only when *curB_flag is true on the device
    const bool twist_possible = curB_flag && curB_x && curB_y && curB_z && twist;
    TraceJob<FieldSoA> J;
    J.f = FieldSoA{Bx, By, Bz, Dims{2, 2, 2}};
    fill_common(J, &io, &prm, nullptr);
    J.shape_dev = BshapeN;
    J.cur = FieldSoA{curB_x, curB_y, curB_z, Dims{2, 2, 2}};
    J.s.s_len_dev = s_len;
    J.s.tol_coef_dev = integrator == QSL_RKF45 ? tol_coef : nullptr;
    J.s.tol_coef = 1.f;
    J.s.n_dev = N;
    J.s.cross_dev = inp_cross_dir;
    J.s.twist_flag_dev = twist_possible ? curB_flag : nullptr;
    J.s.twist_on = 0;
    J.s.n_cap = capacity < 0 ? -1 : capacity;
    return run_trace(J, arith, twist_possible, QSL_SCHED_QUEUE, 0, nullptr, (cudaStream_t)stream);
}

// Stretched grid, native form: field arrays (x fastest) of shape nx x ny x nz
// on the increasing node coordinates x_arr_h, y_arr_h, z_arr_h (host), host
// scalars and settings.
int qsl_trace_stretch(const float* Bx, const float* By, const float* Bz, int nx, int ny, int nz,
                      const float* x_arr_h, const float* y_arr_h, const float* z_arr_h, int uni,
                      const qsl_trace_params* prm, const qsl_trace_io* io, int64_t n, float s_len, float tol_coef,
                      const float* cross_dir_h, const float* curBx, const float* curBy, const float* curBz,
                      const qsl_sched* sched_h, qsl_stream_t stream) {
    if (!Bx || !By || !Bz || !x_arr_h || !y_arr_h || !z_arr_h) return fail(QSL_ERR_INVALID, "null field or coordinates");
    if (!dims_ok(nx, ny, nz)) return fail(QSL_ERR_INVALID, "bad field shape %d x %d x %d", nx, ny, nz);
    if (!params_ok(prm)) return fail(QSL_ERR_INVALID, "bad trace params");
    if (prm->arith == QSL_ARITH_FAST_W16)
        return fail(QSL_ERR_INVALID, "fp16 x weights (QSL_ARITH_FAST_W16) are a qsl_trace option of the h4b layout");
    if (n < 0) return fail(QSL_ERR_INVALID, "negative seed count");
    if (n == 0) return QSL_OK;
    if (!io_ok(io)) return fail(QSL_ERR_INVALID, "null pointer in trace io");
    const float* ah[3] = {x_arr_h, y_arr_h, z_arr_h};
    const int na[3] = {nx, ny, nz};
    for (int k = 0; k < 3; ++k)
        for (int i = 0; i + 1 < na[k]; ++i)
            if (!(ah[k][i] < ah[k][i + 1])) return fail(QSL_ERR_INVALID, "coordinates of axis %d not increasing", k);
    qsl_sched sc{QSL_SCHED_STATIC, 0, nullptr, nullptr, nullptr, 0};
    if (sched_h) sc = *sched_h;
    if (sc.schedule != QSL_SCHED_QUEUE && sc.schedule != QSL_SCHED_STATIC)
        return fail(QSL_ERR_INVALID, "bad schedule %d", sc.schedule);
    if (sc.occupancy != 0 && (sc.occupancy < 4 || sc.occupancy > 10))
        return fail(QSL_ERR_INVALID, "occupancy must be 0 or 4 to 10");
    if (sc.order && n > 0xffffffffLL) return fail(QSL_ERR_TOO_LARGE, "order map limits n to 2^32-1");
    const bool twist = curBx != nullptr;
    if (twist && (!curBy || !curBz || !io->twist)) return fail(QSL_ERR_INVALID, "twist needs curB_x/y/z and twist");
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t cells = (int64_t)(nx - 1) + (ny - 1) + (nz - 1);
    const int64_t nodes = (int64_t)nx * ny * nz;
    // (the packed sampler indexes records in 32 bits)
    const bool packed_path = prm->arith == QSL_ARITH_FAST && cells * (1 + STRETCH_BINS_PER_CELL) < (1LL << 31) &&
                             nodes < (1LL << 31);
    // one stream-ordered buffer for the launch: the coordinates, then (fast
    // arithmetic) the x-pair node records and the search tables
    const int64_t tcells = (packed_path && !uni) ? cells : 0;
    const int64_t srec_len = (tcells + 1) & ~(int64_t)1;  // even: sbin starts on a 32-byte boundary
    const int64_t ncoord = (int64_t)nx + ny + nz;
    const size_t coord_bytes = ((size_t)ncoord * sizeof(float) + 255) / 256 * 256;
    const size_t bytes = coord_bytes + (packed_path ? (size_t)(2 * nodes + srec_len) * sizeof(float4) +
                                                          (size_t)tcells * STRETCH_BINS_PER_CELL * 2 * sizeof(float4)
                                                    : 0);
    char* buf = nullptr;
    QSL_CHECK_CUDA(cudaMallocAsync((void**)&buf, bytes, st), "launch buffer allocation");
    float* coord = reinterpret_cast<float*>(buf);
    cudaError_t e = cudaSuccess;
    for (int k = 0, off = 0; k < 3 && e == cudaSuccess; off += na[k], ++k)
        e = cudaMemcpyAsync(coord + off, ah[k], (size_t)na[k] * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) {
        cudaFreeAsync(buf, st);
        return cuda_fail(e, "coordinate upload");
    }
    const float *x_arr = coord, *y_arr = coord + nx, *z_arr = coord + nx + ny;
    auto go = [&](auto store) {
        TraceJob<decltype(store)> J;
        J.f = store;
        fill_common(J, io, prm, sc.samples);
        J.cur = FieldSoA{curBx, curBy, curBz, J.f.d};
        J.order = sc.order;
        J.chunk = sc.chunk;
        J.occupancy = sc.occupancy;
        J.s.s_len = s_len;
        J.s.tol_coef = tol_coef;
        J.s.n = n;
        J.s.cross[0] = cross_dir_h ? cross_dir_h[0] : 0.f;
        J.s.cross[1] = cross_dir_h ? cross_dir_h[1] : 0.f;
        J.s.cross[2] = cross_dir_h ? cross_dir_h[2] : 1.f;
        J.s.twist_on = twist ? 1 : 0;
        if constexpr (std::is_same<decltype(store), FieldStretchP>::value ||
                      std::is_same<decltype(store), FieldStretchPU>::value)
            J.lim.len_lim = (float)(prm->len_ratio * stretch_len_scale_host(J.f));
        return run_trace(J, prm->arith, twist, sc.schedule, n, sc.queue, st);
    };
    int rc;
    if (!packed_path) {
        // the caller's arrays with the one search the host knows applies
        auto arrays = [&](auto fa) {
            fa.bx = Bx;
            fa.by = By;
            fa.bz = Bz;
            fa.d = Dims{nx, ny, nz};
            fa.ax = x_arr;
            fa.ay = y_arr;
            fa.az = z_arr;
            fa.uni_dev = nullptr;
            return go(fa);
        };
        rc = uni ? arrays(FieldStretchU{}) : arrays(FieldStretch{});
        cudaFreeAsync(buf, st);
        return rc;
    }
    // fast arithmetic: the nodes interleaved into x-pair records for the
    // launch (node o and o + 1 as two float4: one 32-byte load per corner
    // pair; the same values), followed, for the search, by its tables (a
    // 16-byte record per cell, padded to an even count, then two 16-byte
    // records per bin, read as one 32-byte load); the uniform formula needs
    // none
    float4* b4 = reinterpret_cast<float4*>(buf + coord_bytes);
    float4* srec = uni ? nullptr : b4 + 2 * nodes;
    float4* sbin = uni ? nullptr : srec + srec_len;
    e = launch_pack_f4x2(Bx, By, Bz, Dims{nx, ny, nz}, b4, st);
    if (e == cudaSuccess && !uni) e = launch_stretch_tables(x_arr, y_arr, z_arr, Dims{nx, ny, nz}, srec, sbin, st);
    if (e != cudaSuccess) {
        cudaFreeAsync(buf, st);
        return cuda_fail(e, "node copy");
    }
    auto packed = [&](auto fp) {
        fp.bx = Bx;
        fp.by = By;
        fp.bz = Bz;
        fp.d = Dims{nx, ny, nz};
        fp.ax = x_arr;
        fp.ay = y_arr;
        fp.az = z_arr;
        fp.uni_dev = nullptr;
        stretch_constants_host(fp, x_arr_h, y_arr_h, z_arr_h);
        fp.b4 = b4;
        fp.srec = srec;
        fp.sbin = sbin;
        return go(fp);
    };
    rc = uni ? packed(FieldStretchPU{}) : packed(FieldStretchP{});
    cudaFreeAsync(buf, st);
    return rc;
}

// Drop-in entry for the stretched-grid kernel: the argument list of
// TraceAllBline in TraceBlineAdaptiveStretch.cu:422-433, scalars by device
// pointer, the field read in place.
int qsl_trace_all_bline_stretch(int arith, const float* Bx, const float* By, const float* Bz, const int* BshapeN,
                                const float* x_arr, const float* y_arr, const float* z_arr, const bool* flag_uni,
                                const float* curB_x, const float* curB_y, const float* curB_z, double* twist,
                                const bool* curB_flag, const float* inp_x, const float* inp_y, const float* inp_z,
                                const float* inp_cross_dir, float* start_x, float* start_y, float* start_z,
                                int* flag_start, float* end_x, float* end_y, float* end_z, int* flag_end,
                                float* B_this_x, float* B_this_y, float* B_this_z, int* B_flag, float* B_start_x,
                                float* B_start_y, float* B_start_z, float* B_end_x, float* B_end_y, float* B_end_z,
                                const float* s_len, const unsigned long long* N, double* LineLen,
                                const float* tol_coef, int64_t capacity, qsl_stream_t stream) {
    if (capacity == 0) return QSL_OK;
    if (!Bx || !By || !Bz || !BshapeN || !x_arr || !y_arr || !z_arr || !flag_uni || !inp_cross_dir || !s_len || !N ||
        !tol_coef)
        return fail(QSL_ERR_INVALID, "null required pointer");
    if (arith != QSL_ARITH_EXACT && arith != QSL_ARITH_FAST) return fail(QSL_ERR_INVALID, "bad arith %d", arith);
    qsl_trace_params prm;
    qsl_params_reference_stretch(&prm);
    prm.arith = arith;
    qsl_trace_io io{inp_x, inp_y, inp_z, start_x, start_y, start_z, flag_start, end_x, end_y, end_z, flag_end,
                    B_this_x, B_this_y, B_this_z, B_flag, B_start_x, B_start_y, B_start_z, B_end_x, B_end_y,
                    B_end_z, LineLen, twist};
    if (!io_ok(&io)) return fail(QSL_ERR_INVALID, "null pointer in outputs");
    const bool twist_possible = curB_flag && curB_x && curB_y && curB_z && twist;
    // the search and the uniform formula compiled apart: both kernels are
    // launched, and each returns at once unless *flag_uni is its own form
    // (the flag lives on the device; reading it here would synchronise)
    auto form = [&](auto f) {
        TraceJob<decltype(f)> J;
        f.bx = Bx;
        f.by = By;
        f.bz = Bz;
        f.d = Dims{2, 2, 2};
        f.ax = x_arr;
        f.ay = y_arr;
        f.az = z_arr;
        f.uni_dev = flag_uni;
        J.f = f;
        fill_common(J, &io, &prm, nullptr);
        J.shape_dev = BshapeN;
        J.cur = FieldSoA{curB_x, curB_y, curB_z, Dims{2, 2, 2}};
        J.s.s_len_dev = s_len;
        J.s.tol_coef_dev = tol_coef;
        J.s.tol_coef = 1.f;
        J.s.n_dev = N;
        J.s.cross_dev = inp_cross_dir;
        J.s.twist_flag_dev = twist_possible ? curB_flag : nullptr;
        J.s.twist_on = 0;
        J.s.n_cap = capacity < 0 ? -1 : capacity;
        return run_trace(J, arith, twist_possible, QSL_SCHED_QUEUE, 0, nullptr, (cudaStream_t)stream);
    };
    const int rc = form(FieldStretch{});
    return rc != QSL_OK ? rc : form(FieldStretchU{});
}

int qsl_trace_all_bline_rkf45(const float* Bx, const float* By, const float* Bz, const int* BshapeN,
                              const float* curB_x, const float* curB_y, const float* curB_z, double* twist,
                              const bool* curB_flag, const float* inp_x, const float* inp_y, const float* inp_z,
                              const float* inp_cross_dir, float* start_x, float* start_y, float* start_z,
                              int* flag_start, float* end_x, float* end_y, float* end_z, int* flag_end,
                              float* B_this_x, float* B_this_y, float* B_this_z, int* B_flag, float* B_start_x,
                              float* B_start_y, float* B_start_z, float* B_end_x, float* B_end_y, float* B_end_z,
                              const float* s_len, const unsigned long long* N, double* LineLen,
                              const float* tol_coef, qsl_stream_t stream) {
    return qsl_trace_all_bline(QSL_RKF45, QSL_ARITH_EXACT, Bx, By, Bz, BshapeN, curB_x, curB_y, curB_z, twist,
                               curB_flag, inp_x, inp_y, inp_z, inp_cross_dir, start_x, start_y, start_z, flag_start,
                               end_x, end_y, end_z, flag_end, B_this_x, B_this_y, B_this_z, B_flag, B_start_x,
                               B_start_y, B_start_z, B_end_x, B_end_y, B_end_z, s_len, N, LineLen, tol_coef, -1, stream);
}

int qsl_trace_all_bline_rk4(const float* Bx, const float* By, const float* Bz, const int* BshapeN,
                            const float* curB_x, const float* curB_y, const float* curB_z, double* twist,
                            const bool* curB_flag, const float* inp_x, const float* inp_y, const float* inp_z,
                            const float* inp_cross_dir, float* start_x, float* start_y, float* start_z,
                            int* flag_start, float* end_x, float* end_y, float* end_z, int* flag_end,
                            float* B_this_x, float* B_this_y, float* B_this_z, int* B_flag, float* B_start_x,
                            float* B_start_y, float* B_start_z, float* B_end_x, float* B_end_y, float* B_end_z,
                            const float* s_len, const unsigned long long* N, double* LineLen, qsl_stream_t stream) {
    return qsl_trace_all_bline(QSL_RK4, QSL_ARITH_EXACT, Bx, By, Bz, BshapeN, curB_x, curB_y, curB_z, twist,
                               curB_flag, inp_x, inp_y, inp_z, inp_cross_dir, start_x, start_y, start_z, flag_start,
                               end_x, end_y, end_z, flag_end, B_this_x, B_this_y, B_this_z, B_flag, B_start_x,
                               B_start_y, B_start_z, B_end_x, B_end_y, B_end_z, s_len, N, LineLen, nullptr, -1, stream);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batched trace plans
// ---------------------------------------------------------------------------
// Jobs are grouped by store type (slot = the layout code); each slot is one
// launch over its job table.
struct qsl_batch {
    int device;
    // per store type: job table and warp-aligned line offsets in device memory
    void* jobs[kStoreTypes];
    long long* begin[kStoreTypes];
    int njobs[kStoreTypes];
    long long total[kStoreTypes];
    bool twist[kStoreTypes];
    int64_t lines;
};

template <class F>
static TraceJob<F> batch_job_of(const qsl_batch_job& b, const F& f) {
    TraceJob<F> J;
    J.f = f;
    fill_common(J, &b.io, &b.params, nullptr);
    J.cur = FieldSoA{b.curB[0], b.curB[1], b.curB[2], f.d};
    J.order = b.order;
    J.s.s_len = b.s_len;
    J.s.tol_coef = b.tol_coef;
    J.s.n = b.n;
    J.s.n_dev = b.n_dev;
    J.s.cross[0] = b.cross_dir[0]; J.s.cross[1] = b.cross_dir[1]; J.s.cross[2] = b.cross_dir[2];
    J.s.twist_on = b.curB[0] ? 1 : 0;
    return J;
}

static int64_t align256(int64_t x) { return (x + 255) / 256 * 256; }

// Per store type: the job list (TraceJob<F> of that store, as bytes) and the
// line offsets.
struct BatchLists {
    std::vector<char> j[kStoreTypes];
    size_t jsz[kStoreTypes] = {sizeof(TraceJob<FieldSoA>), sizeof(TraceJob<FieldF4>), sizeof(TraceJob<FieldH4B>),
                               sizeof(TraceJob<FieldH8C>)};
    std::vector<long long> b[kStoreTypes];
    bool tw[kStoreTypes] = {false, false, false, false};
    int64_t lines = 0;
    size_t count(int k) const { return j[k].size() / jsz[k]; }
};

template <class F>
static void push_job(std::vector<char>& v, const TraceJob<F>& J) {
    const char* p = reinterpret_cast<const char*>(&J);
    v.insert(v.end(), p, p + sizeof(J));
}

static int batch_lists(const qsl_batch_job* jobs_h, int njobs, BatchLists& L) {
    if (njobs < 0 || (njobs > 0 && !jobs_h)) return fail(QSL_ERR_INVALID, "bad job list");
    for (int k = 0; k < kStoreTypes; ++k) L.b[k] = std::vector<long long>{0};
    for (int k = 0; k < njobs; ++k) {
        const qsl_batch_job& b = jobs_h[k];
        if (!b.field) return fail(QSL_ERR_INVALID, "job %d: null field", k);
        if (!params_ok(&b.params) || b.params.arith != QSL_ARITH_FAST)
            return fail(QSL_ERR_INVALID, "job %d: bad params (batched jobs use fast arithmetic)", k);
        if (b.n < 0) return fail(QSL_ERR_INVALID, "job %d: negative n", k);
        if (b.n > 0 && !io_ok(&b.io)) return fail(QSL_ERR_INVALID, "job %d: null pointer in io", k);
        if (b.curB[0] && (!b.curB[1] || !b.curB[2] || !b.io.twist))
            return fail(QSL_ERR_INVALID, "job %d: twist needs curB_x/y/z and twist", k);
        if (b.order && b.n > 0xffffffffLL) return fail(QSL_ERR_TOO_LARGE, "job %d: order map limits n", k);
        const qsl_field* f = b.field;
        const long long padded = (b.n + 31) / 32 * 32;
        L.lines += b.n;
        const int slot = f->layout;
        switch (slot) {
            case LAYOUT_SOA: push_job(L.j[slot], batch_job_of(b, soa_of(f))); break;
            case LAYOUT_F4: push_job(L.j[slot], batch_job_of(b, f4_of(f))); break;
            case LAYOUT_H4B: push_job(L.j[slot], batch_job_of(b, h4b_of(f))); break;
            default: push_job(L.j[slot], batch_job_of(b, h8c_of(f))); break;
        }
        L.b[slot].push_back(L.b[slot].back() + padded);
        L.tw[slot] = L.tw[slot] || b.curB[0];
    }
    return QSL_OK;
}

// Serialised batch table: per store type a TraceJob<F> array and its line
// offsets, each at a 256-byte aligned offset of one buffer.
static void batch_layout(const BatchLists& L, qsl_batch_info* info) {
    int64_t off = 0;
    for (int k = 0; k < kStoreTypes; ++k) {
        info->jobs_offset[k] = off;
        off = align256(off + (int64_t)L.j[k].size());
        info->begin_offset[k] = off;
        off = align256(off + (int64_t)(L.b[k].size() * sizeof(long long)));
        info->njobs[k] = (int32_t)L.count(k);
        info->twist[k] = L.tw[k] ? 1 : 0;
        info->total[k] = L.b[k].back();
    }
    info->table_bytes = off;
    info->lines = L.lines;
}

// One launch per store type with jobs (a type without jobs launches nothing).
static cudaError_t launch_slots(void* const jobs[], long long* const begin[], const int njobs[],
                                const long long total[], const bool twist[], unsigned long long* samples,
                                int max_blocks, long long lo, long long hi, int occ, cudaStream_t st) {
    cudaError_t e = launch_trace_batch_soa((const TraceJob<FieldSoA>*)jobs[0], begin[0], njobs[0], total[0], twist[0],
                                           samples, max_blocks, lo, hi, occ, st);
    if (e == cudaSuccess)
        e = launch_trace_batch_f4((const TraceJob<FieldF4>*)jobs[1], begin[1], njobs[1], total[1], twist[1], samples,
                                  max_blocks, lo, hi, occ, st);
    if (e == cudaSuccess)
        e = launch_trace_batch_h4b((const TraceJob<FieldH4B>*)jobs[2], begin[2], njobs[2], total[2], twist[2],
                                   samples, max_blocks, lo, hi, occ, st);
    if (e == cudaSuccess)
        e = launch_trace_batch_h8c((const TraceJob<FieldH8C>*)jobs[3], begin[3], njobs[3], total[3], twist[3],
                                   samples, max_blocks, lo, hi, occ, st);
    return e;
}

extern "C" {

int qsl_batch_pack(const qsl_batch_job* jobs_h, int njobs, void* table_h, int64_t table_bytes,
                   qsl_batch_info* info_h) {
    if (!info_h) return fail(QSL_ERR_INVALID, "info is null");
    BatchLists L;
    int rc = batch_lists(jobs_h, njobs, L);
    if (rc != QSL_OK) return rc;
    batch_layout(L, info_h);
    if (!table_h) return QSL_OK;  // size query
    if (table_bytes < info_h->table_bytes) return fail(QSL_ERR_INVALID, "table buffer too small");
    char* t = (char*)table_h;
    for (int k = 0; k < kStoreTypes; ++k) {
        if (!L.j[k].empty()) memcpy(t + info_h->jobs_offset[k], L.j[k].data(), L.j[k].size());
        memcpy(t + info_h->begin_offset[k], L.b[k].data(), L.b[k].size() * sizeof(long long));
    }
    return QSL_OK;
}

int qsl_batch_run_window(const void* table_dev, const qsl_batch_info* info_h, unsigned long long* samples_dev,
                         int64_t line_lo, int64_t line_hi, int max_blocks, int occupancy, qsl_stream_t stream) {
    if (!table_dev || !info_h) return fail(QSL_ERR_INVALID, "null table or info");
    if (max_blocks < 0) return fail(QSL_ERR_INVALID, "max_blocks must be >= 0");
    if (occupancy != 0 && (occupancy < 6 || occupancy > 10))
        return fail(QSL_ERR_INVALID, "occupancy must be 0, 6, 7, 8, 9 or 10");
    char* t = (char*)table_dev;
    const qsl_batch_info& I = *info_h;
    void* jobs[kStoreTypes];
    long long* begin[kStoreTypes];
    int nj[kStoreTypes];
    long long total[kStoreTypes];
    bool tw[kStoreTypes];
    for (int k = 0; k < kStoreTypes; ++k) {
        jobs[k] = t + I.jobs_offset[k];
        begin[k] = (long long*)(t + I.begin_offset[k]);
        nj[k] = I.njobs[k];
        total[k] = I.total[k];
        tw[k] = I.twist[k] != 0;
    }
    QSL_CHECK_CUDA(launch_slots(jobs, begin, nj, total, tw, samples_dev, max_blocks, line_lo, line_hi, occupancy,
                                (cudaStream_t)stream),
                   "batch run");
    return QSL_OK;
}

int qsl_batch_run(const void* table_dev, const qsl_batch_info* info_h, unsigned long long* samples_dev,
                  qsl_stream_t stream) {
    return qsl_batch_run_window(table_dev, info_h, samples_dev, 0, -1, 0, 0, stream);
}

int qsl_batch_create(const qsl_batch_job* jobs_h, int njobs, qsl_stream_t stream, qsl_batch_t** out) {
    if (!out) return fail(QSL_ERR_INVALID, "out is null");
    *out = nullptr;
    BatchLists L;
    int rc = batch_lists(jobs_h, njobs, L);
    if (rc != QSL_OK) return rc;
    qsl_batch* B = new (std::nothrow) qsl_batch();
    if (!B) return fail(QSL_ERR_NOMEM, "host allocation failed");
    cudaGetDevice(&B->device);
    B->lines = L.lines;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < kStoreTypes && e == cudaSuccess; ++k) {
        B->njobs[k] = (int)L.count(k);
        B->total[k] = L.b[k].back();
        B->twist[k] = L.tw[k];
        if (L.j[k].empty()) continue;
        e = cudaMalloc(&B->jobs[k], L.j[k].size());
        if (e == cudaSuccess) e = cudaMalloc((void**)&B->begin[k], L.b[k].size() * sizeof(long long));
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(B->jobs[k], L.j[k].data(), L.j[k].size(), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(B->begin[k], L.b[k].data(), L.b[k].size() * sizeof(long long),
                                cudaMemcpyHostToDevice, st);
    }
    // the host lists die on return: make sure the copies have read them
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        qsl_batch_destroy(B);
        return cuda_fail(e, "batch upload");
    }
    *out = B;
    return QSL_OK;
}

int qsl_batch_launch(const qsl_batch_t* B, unsigned long long* samples_dev, qsl_stream_t stream) {
    if (!B) return fail(QSL_ERR_INVALID, "batch is null");
    QSL_CHECK_CUDA(launch_slots(B->jobs, B->begin, B->njobs, B->total, B->twist, samples_dev, 0, 0, -1, 0,
                                (cudaStream_t)stream),
                   "batch launch");
    return QSL_OK;
}

int64_t qsl_batch_lines(const qsl_batch_t* B) { return B ? B->lines : 0; }

int qsl_batch_destroy(qsl_batch_t* B) {
    if (!B) return QSL_OK;
    for (int k = 0; k < kStoreTypes; ++k) {
        cudaFree(B->jobs[k]);
        cudaFree(B->begin[k]);
    }
    delete B;
    return QSL_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Scott deviation-vector tracer
// ---------------------------------------------------------------------------
static bool scott_io_ok(const qsl_scott_io* io) {
    return io && io->inp_x && io->inp_y && io->inp_z && io->start_x && io->start_y && io->start_z &&
           io->flag_start && io->end_x && io->end_y && io->end_z && io->flag_end && io->B_this_x && io->B_this_y &&
           io->B_this_z && io->q_0 && io->q_perp && io->LineLen;
}

template <class F>
static void scott_fill(ScottJob<F>& J, const qsl_scott_io* io, const qsl_trace_params* prm) {
    J.shape_dev = nullptr;
    J.inp_x = io->inp_x; J.inp_y = io->inp_y; J.inp_z = io->inp_z;
    ScottOut& o = J.o;
    o.start_x = io->start_x; o.start_y = io->start_y; o.start_z = io->start_z; o.flag_start = io->flag_start;
    o.end_x = io->end_x; o.end_y = io->end_y; o.end_z = io->end_z; o.flag_end = io->flag_end;
    o.bthis_x = io->B_this_x; o.bthis_y = io->B_this_y; o.bthis_z = io->B_this_z;
    o.q0 = io->q_0; o.qperp = io->q_perp; o.line_len = io->LineLen; o.twist = io->twist;
    J.prm = *prm;
    J.order = nullptr;
    J.samples = nullptr;
    memset(&J.s, 0, sizeof(J.s));
    J.s.n_cap = -1;
}

extern "C" {

int qsl_trace_scott(const qsl_field_t* field, const qsl_trace_params* prm, const qsl_scott_io* io, int64_t n,
                    const unsigned long long* n_dev, float s_len, float tol_coef, const float* curBx,
                    const float* curBy, const float* curBz, int grad_mode, const qsl_sched* sched_h,
                    qsl_stream_t stream) {
    if (!field) return fail(QSL_ERR_INVALID, "field is null");
    if (!params_ok(prm) || prm->integrator != QSL_RKF45)
        return fail(QSL_ERR_INVALID, "bad trace params (the Scott tracer is RKF45)");
    if (prm->arith == QSL_ARITH_FAST_W16)
        return fail(QSL_ERR_INVALID, "fp16 x weights (QSL_ARITH_FAST_W16) are a qsl_trace option of the h4b layout");
    if (grad_mode != QSL_GRAD_FD && grad_mode != QSL_GRAD_ANALYTIC) return fail(QSL_ERR_INVALID, "bad grad_mode");
    if (prm->arith == QSL_ARITH_EXACT && (grad_mode != QSL_GRAD_FD || field->layout != LAYOUT_SOA))
        return fail(QSL_ERR_INVALID, "exact arithmetic needs the SoA layout and QSL_GRAD_FD");
    if (n < 0) return fail(QSL_ERR_INVALID, "negative seed count");
    if (n == 0) return QSL_OK;
    if (!scott_io_ok(io)) return fail(QSL_ERR_INVALID, "null pointer in scott io");
    const bool twist = curBx != nullptr;
    if (twist && (!curBy || !curBz || !io->twist)) return fail(QSL_ERR_INVALID, "twist needs curB_x/y/z and twist");
    qsl_sched sc{QSL_SCHED_STATIC, 0, nullptr, nullptr, nullptr, 0};
    if (sched_h) sc = *sched_h;
    if (sc.order && n > 0xffffffffLL) return fail(QSL_ERR_TOO_LARGE, "order map limits n to 2^32-1");
    cudaStream_t st = (cudaStream_t)stream;
    const FieldSoA cur{curBx, curBy, curBz, field->d};
    cudaError_t e;
    auto common = [&](auto& J) {
        scott_fill(J, io, prm);
        J.cur = cur;
        J.order = sc.order;
        J.samples = sc.samples;
        J.s.s_len = s_len;
        J.s.tol_coef = tol_coef;
        J.s.n = n;
        J.s.n_dev = n_dev;
        J.s.n_cap = n_dev ? n : -1;
        J.s.twist_on = twist ? 1 : 0;
    };
    if (field->layout == LAYOUT_SOA) {
        ScottJob<FieldSoA> J;
        J.f = soa_of(field);
        common(J);
        e = prm->arith == QSL_ARITH_EXACT ? launch_scott_exact(J, twist, n, st)
                                          : launch_scott_fast_soa(J, grad_mode, twist, n, st);
    } else if (field->layout == LAYOUT_F4) {
        ScottJob<FieldF4> J;
        J.f = f4_of(field);
        common(J);
        e = launch_scott_fast_f4(J, grad_mode, twist, n, st);
    } else if (field->layout == LAYOUT_H4B) {
        ScottJob<FieldH4B> J;
        J.f = h4b_of(field);
        common(J);
        e = launch_scott_fast_h4b(J, grad_mode, twist, n, st);
    } else {
        ScottJob<FieldH8C> J;
        J.f = h8c_of(field);
        common(J);
        e = launch_scott_fast_h8c(J, grad_mode, twist, n, st);
    }
    if (e != cudaSuccess) return cuda_fail(e, "scott launch");
    return QSL_OK;
}

int qsl_trace_all_bline_scott(const float* Bx, const float* By, const float* Bz, const int* BshapeN,
                              const float* curB_x, const float* curB_y, const float* curB_z, double* twist,
                              const bool* curB_flag, const float* inp_x, const float* inp_y, const float* inp_z,
                              const float* inp_cross_dir, float* start_x, float* start_y, float* start_z,
                              int* flag_start, float* end_x, float* end_y, float* end_z, int* flag_end,
                              float* B_this_x, float* B_this_y, float* B_this_z, float* q_0_arr, float* q_perp_arr,
                              const float* s_len, const unsigned long long* N, double* LineLen,
                              const float* tol_coef, int64_t capacity, qsl_stream_t stream) {
    (void)inp_cross_dir;  // read by the reference kernel but unused by its Scott tracer
    if (capacity == 0) return QSL_OK;
    if (!Bx || !By || !Bz || !BshapeN || !s_len || !N || !tol_coef)
        return fail(QSL_ERR_INVALID, "null required pointer");
    if (capacity < 0) return fail(QSL_ERR_INVALID, "capacity (the per-seed array length) is required");
    qsl_scott_io io{inp_x, inp_y, inp_z, start_x, start_y, start_z, flag_start, end_x, end_y, end_z, flag_end,
                    B_this_x, B_this_y, B_this_z, q_0_arr, q_perp_arr, LineLen, twist};
    if (!scott_io_ok(&io)) return fail(QSL_ERR_INVALID, "null pointer in outputs");
    qsl_trace_params prm;
    qsl_params_reference_scott(&prm);
    const bool twist_possible = curB_flag && curB_x && curB_y && curB_z && twist;
    ScottJob<FieldSoA> J;
    J.f = FieldSoA{Bx, By, Bz, Dims{2, 2, 2}};
    scott_fill(J, &io, &prm);
    J.shape_dev = BshapeN;
    J.cur = FieldSoA{curB_x, curB_y, curB_z, Dims{2, 2, 2}};
    J.s.s_len_dev = s_len;
    J.s.tol_coef_dev = tol_coef;
    J.s.n_dev = N;
    J.s.n_cap = capacity;
    J.s.twist_flag_dev = twist_possible ? curB_flag : nullptr;
    const cudaError_t e = launch_scott_exact(J, twist_possible, capacity, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "scott launch");
    return QSL_OK;
}

void qsl_params_reference_stretch(qsl_trace_params* p) {
    qsl_params_reference_rkf45(p);
    p->len_ratio = 2.0;         // x the summed coordinate extents
    p->max_steps = 0x7fffffff;  // the reference has no step limit
    p->boundary_twist = 1;
}

void qsl_params_reference_scott(qsl_trace_params* p) {
    qsl_params_reference_rkf45(p);
    p->tol_law = QSL_TOL_ABSOLUTE;
    p->len_ratio = 2.0;
    p->max_steps = 10000;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Q assembly
// ---------------------------------------------------------------------------
extern "C" {
int qsl_qcalc_plane(const float* x_end, const float* y_end, const float* z_end, const int* flag_end,
                    const float* x_start, const float* y_start, const float* z_start, const int* flag_start,
                    const float* Bz_in, const float* Bz_out, const float* Bx_0, const float* By_0,
                    const float* Bz_0, int n0, int n1, int64_t nplanes, double jac_scale,
                    const float* cross_dir_h, float* Q32, double* Q64, qsl_stream_t stream) {
    if (!x_end || !y_end || !z_end || !flag_end || !x_start || !y_start || !z_start || !flag_start || !Bz_in ||
        !Bz_out || !Bx_0 || !By_0 || !Bz_0 || !cross_dir_h)
        return fail(QSL_ERR_INVALID, "null input");
    if ((Q32 == nullptr) == (Q64 == nullptr)) return fail(QSL_ERR_INVALID, "exactly one of Q32 / Q64");
    if (n0 < 3 || n1 < 3 || nplanes < 0) return fail(QSL_ERR_INVALID, "plane must be at least 3 x 3");
    QPlaneArgs a;
    a.xe = x_end; a.ye = y_end; a.ze = z_end; a.fe = flag_end;
    a.xs = x_start; a.ys = y_start; a.zs = z_start; a.fs = flag_start;
    a.bz_in = Bz_in; a.bz_out = Bz_out; a.bx0 = Bx_0; a.by0 = By_0; a.bz0 = Bz_0;
    a.cx = cross_dir_h[0]; a.cy = cross_dir_h[1]; a.cz = cross_dir_h[2];
    a.n0 = n0; a.n1 = n1; a.nplanes = nplanes;
    a.k32 = (float)jac_scale;
    a.k64 = jac_scale;
    a.q32 = Q32;
    a.q64 = Q64;
    QSL_CHECK_CUDA(launch_qcalc_plane(a, Q64 != nullptr, (cudaStream_t)stream), "qcalc_plane");
    return QSL_OK;
}

int64_t qsl_cook_workspace_bytes(int64_t n) {
    const long long t = cook_tiles(n);
    return (int64_t)(t * (sizeof(int) + sizeof(long long)) + 64);
}

int qsl_cook_pseudo_line(const int* B_flag, const float* x_start, const float* y_start, const float* z_start,
                         const int* flag_start, const float* Bz_in, const float* Bz_out, int64_t n, int n0, int n1,
                         int interior_only, float stride, float* cut_x, float* cut_y, float* cut_z,
                         float* Bz0_start, float* Bz0_end, int64_t* pix, unsigned long long* count_dev,
                         void* workspace, int64_t workspace_bytes, qsl_stream_t stream) {
    if (!B_flag || !x_start || !y_start || !z_start || !flag_start || !Bz_in || !Bz_out || !cut_x || !cut_y ||
        !cut_z || !Bz0_start || !Bz0_end || !count_dev || !workspace)
        return fail(QSL_ERR_INVALID, "null pointer");
    if (n < 0) return fail(QSL_ERR_INVALID, "negative n");
    if (interior_only && (n0 < 1 || n1 < 1 || n % ((int64_t)n0 * n1) != 0))
        return fail(QSL_ERR_INVALID, "interior_only needs n a multiple of n0*n1");
    if (workspace_bytes < qsl_cook_workspace_bytes(n)) return fail(QSL_ERR_INVALID, "workspace too small");
    const long long tiles = cook_tiles(n);
    long long* tile_off = (long long*)workspace;
    int* tile_count = (int*)(tile_off + tiles);
    CookArgs a;
    a.bflag = B_flag; a.xs = x_start; a.ys = y_start; a.zs = z_start; a.fs = flag_start;
    a.bz_in = Bz_in; a.bz_out = Bz_out; a.n = n; a.n0 = n0; a.n1 = n1; a.interior_only = interior_only;
    a.stride = stride; a.tile_off = tile_off;
    a.cx = cut_x; a.cy = cut_y; a.cz = cut_z; a.bz0s = Bz0_start; a.bz0e = Bz0_end; a.pix = (long long*)pix;
    QSL_CHECK_CUDA(launch_cook(a, tile_count, tile_off, count_dev, (cudaStream_t)stream), "cook_pseudo_line");
    return QSL_OK;
}

int qsl_qcut(const float* start_x, const float* start_y, const float* start_z, const int* flag_start,
             const float* end_x, const float* end_y, const float* end_z, const int* flag_end,
             const float* Bz0_start, const float* Bz0_end, int64_t count, const unsigned long long* count_dev,
             int64_t max_count, double jac_scale, float* Qcut32, double* Qcut64, qsl_stream_t stream) {
    if (!start_x || !start_y || !start_z || !flag_start || !end_x || !end_y || !end_z || !flag_end ||
        !Bz0_start || !Bz0_end)
        return fail(QSL_ERR_INVALID, "null input");
    if ((Qcut32 == nullptr) == (Qcut64 == nullptr)) return fail(QSL_ERR_INVALID, "exactly one of Qcut32 / Qcut64");
    QcutArgs a;
    a.xs = start_x; a.ys = start_y; a.zs = start_z; a.fs = flag_start;
    a.xe = end_x; a.ye = end_y; a.ze = end_z; a.fe = flag_end;
    a.bz0s = Bz0_start; a.bz0e = Bz0_end;
    a.count_dev = count_dev; a.count = count;
    a.k32 = (float)jac_scale; a.k64 = jac_scale;
    a.q32 = Qcut32; a.q64 = Qcut64;
    const long long mc = count_dev ? max_count : count;
    QSL_CHECK_CUDA(launch_qcut(a, Qcut64 != nullptr, mc, (cudaStream_t)stream), "qcut");
    return QSL_OK;
}

int qsl_qmerge(const int64_t* pix, const float* Qcut32, const double* Qcut64, int64_t count,
               const unsigned long long* count_dev, int64_t max_count, int n0, int n1, float* Qfinal32,
               double* Qfinal64, qsl_stream_t stream) {
    if (!pix) return fail(QSL_ERR_INVALID, "null pix");
    const long long mc = count_dev ? max_count : count;
    if (Qcut32 && Qfinal32) {
        QSL_CHECK_CUDA(launch_qmerge_f32((const long long*)pix, Qcut32, count_dev, count, mc, n0, n1, Qfinal32,
                                         (cudaStream_t)stream), "qmerge");
    } else if (Qcut64 && Qfinal64) {
        QSL_CHECK_CUDA(launch_qmerge_f64((const long long*)pix, Qcut64, count_dev, count, mc, n0, n1, Qfinal64,
                                         (cudaStream_t)stream), "qmerge");
    } else {
        return fail(QSL_ERR_INVALID, "Qcut and Qfinal must both be float or both double");
    }
    return QSL_OK;
}

int qsl_curl_grid(const float* Bx, const float* By, const float* Bz, int nx, int ny, int nz, const float* x_arr,
                  const float* y_arr, const float* z_arr, double* curl_x, double* curl_y, double* curl_z,
                  qsl_stream_t stream) {
    if (!Bx || !By || !Bz || !x_arr || !y_arr || !z_arr || !curl_x || !curl_y || !curl_z)
        return fail(QSL_ERR_INVALID, "null argument");
    if (nx < 3 || ny < 3 || nz < 3 || !dims_ok(nx, ny, nz))
        return fail(QSL_ERR_INVALID, "curl needs at least 3 nodes per axis (%d x %d x %d)", nx, ny, nz);
    QSL_CHECK_CUDA(launch_curl(Bx, By, Bz, x_arr, y_arr, z_arr, nx, ny, nz, curl_x, curl_y, curl_z,
                               (cudaStream_t)stream), "curl");
    return QSL_OK;
}

int qsl_trace_path(const float* Bx, const float* By, const float* Bz, int nx, int ny, int nz, const double* seeds,
                   int64_t n, int64_t start, int64_t stop, int64_t stride, double dr, float* out_x, float* out_y,
                   float* out_z, int64_t out_len, qsl_stream_t stream) {
    if (n < 0 || out_len < 0) return fail(QSL_ERR_INVALID, "negative count");
    if (n == 0) return QSL_OK;
    if (!Bx || !By || !Bz || !seeds || !out_x || !out_y || !out_z) return fail(QSL_ERR_INVALID, "null argument");
    if (!dims_ok(nx, ny, nz)) return fail(QSL_ERR_INVALID, "bad field shape %d x %d x %d", nx, ny, nz);
    if (stride == 0) return fail(QSL_ERR_INVALID, "index stride must not be zero");
    if (n > (int64_t)1 << 36) return fail(QSL_ERR_TOO_LARGE, "too many seeds");
    // every index the range visits lies in [0, out_len)
    const bool empty = stride > 0 ? start >= stop : start <= stop;
    if (!empty) {
        const int64_t last = stride > 0 ? start + (stop - 1 - start) / stride * stride
                                        : start - (start - stop - 1) / (-stride) * (-stride);
        const int64_t lo = start < last ? start : last, hi = start < last ? last : start;
        if (lo < 0 || hi >= out_len)
            return fail(QSL_ERR_INVALID, "index range [%lld, %lld] outside the output rows of %lld", (long long)lo,
                        (long long)hi, (long long)out_len);
    }
    if (empty) return QSL_OK;
    QSL_CHECK_CUDA(launch_trace_path(Bx, By, Bz, nx, ny, nz, seeds, n, start, stop, stride, dr, out_x, out_y, out_z,
                                     out_len, (cudaStream_t)stream),
                   "trace path");
    return QSL_OK;
}

int qsl_sample_points(const float* Bx, const float* By, const float* Bz, int nx, int ny, int nz, const double* pts,
                      int64_t n, int normalize, double* out, qsl_stream_t stream) {
    if (n < 0) return fail(QSL_ERR_INVALID, "negative count");
    if (n == 0) return QSL_OK;
    if (!Bx || !By || !Bz || !pts || !out) return fail(QSL_ERR_INVALID, "null argument");
    if (!dims_ok(nx, ny, nz)) return fail(QSL_ERR_INVALID, "bad field shape %d x %d x %d", nx, ny, nz);
    if (n > (int64_t)1 << 37) return fail(QSL_ERR_TOO_LARGE, "too many points");
    QSL_CHECK_CUDA(launch_sample_points(Bx, By, Bz, nx, ny, nz, pts, n, normalize, out, (cudaStream_t)stream),
                   "sample points");
    return QSL_OK;
}

int qsl_hybrid_select(const int* B_flag, const double* Q, int n0, int n1, int64_t nplanes, unsigned* seeds,
                      unsigned long long* count_dev, qsl_stream_t stream) {
    if (!B_flag || !Q || !seeds || !count_dev) return fail(QSL_ERR_INVALID, "null argument");
    if (n0 < 3 || n1 < 3 || nplanes < 0) return fail(QSL_ERR_INVALID, "planes must be at least 3 x 3");
    if ((double)nplanes * n0 * n1 > 4294967295.0) return fail(QSL_ERR_TOO_LARGE, "seed indices exceed 32 bits");
    QSL_CHECK_CUDA(launch_hybrid_select(B_flag, Q, n0, n1, nplanes, seeds, count_dev, (cudaStream_t)stream),
                   "hybrid select");
    return QSL_OK;
}

int qsl_hybrid_merge(const int* B_flag, const float* q_perp, int n0, int n1, int64_t nplanes, double* Q,
                     qsl_stream_t stream) {
    if (!B_flag || !q_perp || !Q) return fail(QSL_ERR_INVALID, "null argument");
    if (n0 < 3 || n1 < 3 || nplanes < 0) return fail(QSL_ERR_INVALID, "planes must be at least 3 x 3");
    QSL_CHECK_CUDA(launch_hybrid_merge(B_flag, q_perp, n0, n1, nplanes, Q, (cudaStream_t)stream), "hybrid merge");
    return QSL_OK;
}

int qsl_device_sm_count(int* sms) {
    int dev = 0;
    QSL_CHECK_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    QSL_CHECK_CUDA(cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, dev), "attribute");
    return QSL_OK;
}

}  // extern "C"
