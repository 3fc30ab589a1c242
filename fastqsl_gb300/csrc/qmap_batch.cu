// Native Q-map batches (qsl_qmap_batch_*): the whole plane Q pipeline of
// many requests laid out in one caller-provided workspace and queued from C++
// (seed grids, tile orders, the batched main trace or a window of it, Q
// assembly, pseudo-line compaction, the batched pseudo-line trace, pseudo Q
// and merge).  The trace kernels are the Python QBatch's; the Q assembly,
// compaction, pseudo Q and merge run as one launch each for the whole batch
// over a job table (QPostJob) with the per-job kernels' arithmetic, so the
// Q maps are the same bit for bit.  The host does two launches per request
// (seed grid, tile order) and one table copy instead of building ~40 arrays
// and job records in Python.  No device allocation and no synchronisation.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <new>
#include <vector>

#include "../../include/fastqsl_gb300.h"
#include "qassembly.h"

namespace qsl {
int set_error(int code, const char* msg);
}

namespace {

constexpr int64_t kAlign = 256;
int64_t up(int64_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

// Offsets of one job's arrays inside the workspace (bytes from the base).
struct JobLayout {
    int64_t xs, ys, zs, order;
    int64_t main[19];  // start_xyz, flag_start, end_xyz, flag_end, B_this_xyz, B_flag, B_start_xyz, B_end_xyz, LineLen
    int64_t sub[19];
    int64_t q, cut[3], bz0s, bz0e, pix, count, work, qcut;
    int64_t work_bytes;
    int64_t n, m;
};

// Trace outputs of n lines: 15 float arrays, 3 int arrays, one double array,
// in qsl_trace_io order (twist and status not written).
void trace_outputs(int64_t n, int64_t& off, int64_t o[19]) {
    // io order: start_x, start_y, start_z, flag_start, end_x, end_y, end_z,
    // flag_end, B_this_x, B_this_y, B_this_z, B_flag, B_start_x..z, B_end_x..z
    for (int k = 0; k < 18; ++k) {
        o[k] = off;
        off = up(off + n * 4);
    }
    o[18] = off;
    off = up(off + n * 8);
}

int64_t layout(const qsl_qmap_job& j, int64_t off, JobLayout& L) {
    const int64_t n = (int64_t)j.n0 * j.n1 * j.nplanes;
    const int64_t m = (int64_t)j.nplanes * (j.n0 - 2) * (j.n1 - 2);
    L.n = n;
    L.m = m;
    L.xs = off; off = up(off + n * 4);
    L.ys = off; off = up(off + n * 4);
    L.zs = off; off = up(off + n * 4);
    L.order = -1;
    if (j.tile_y > 0 && j.tile_x > 0) {
        L.order = off;
        off = up(off + n * 4);
    }
    trace_outputs(n, off, L.main);
    trace_outputs(4 * m, off, L.sub);
    L.q = off; off = up(off + m * 8);
    for (int k = 0; k < 3; ++k) {
        L.cut[k] = off;
        off = up(off + 4 * m * 4);
    }
    L.bz0s = off; off = up(off + m * 4);
    L.bz0e = off; off = up(off + m * 4);
    L.pix = off; off = up(off + m * 8);
    L.count = off; off = up(off + 16);
    L.work_bytes = qsl_cook_workspace_bytes(n);
    L.work = off; off = up(off + L.work_bytes);
    L.qcut = off; off = up(off + m * 8);
    return off;
}

qsl_trace_io io_of(char* base, const JobLayout& L, const int64_t o[19], int64_t seeds_x, int64_t seeds_y,
                   int64_t seeds_z) {
    qsl_trace_io io;
    memset(&io, 0, sizeof(io));
    io.inp_x = (const float*)(base + seeds_x);
    io.inp_y = (const float*)(base + seeds_y);
    io.inp_z = (const float*)(base + seeds_z);
    float** f[15] = {&io.start_x, &io.start_y, &io.start_z, &io.end_x, &io.end_y, &io.end_z, &io.B_this_x,
                     &io.B_this_y, &io.B_this_z, &io.B_start_x, &io.B_start_y, &io.B_start_z, &io.B_end_x,
                     &io.B_end_y, &io.B_end_z};
    const int fk[15] = {0, 1, 2, 4, 5, 6, 8, 9, 10, 12, 13, 14, 15, 16, 17};
    for (int k = 0; k < 15; ++k) *f[k] = (float*)(base + o[fk[k]]);
    io.flag_start = (int*)(base + o[3]);
    io.flag_end = (int*)(base + o[7]);
    io.B_flag = (int*)(base + o[11]);
    io.LineLen = (double*)(base + o[18]);
    (void)L;
    return io;
}

bool job_ok(const qsl_qmap_job& j) {
    return j.field && j.n0 >= 3 && j.n1 >= 3 && j.nplanes >= 1 && j.spacing > 0.0 && isfinite(j.spacing) &&
           (double)j.n0 * j.n1 * j.nplanes <= 4294967295.0;
}

}  // namespace

struct qsl_qmap_batch {
    int njobs;
    std::vector<qsl_qmap_job> jobs;
    std::vector<JobLayout> lay;
    char* ws;
    int64_t main_table, sub_table;  // workspace offsets of the two trace job tables
    int64_t post_table;             // and of the Q-assembly table (QPostJob[njobs], then the begin columns)
    qsl_batch_info main_info, sub_info;
    long long post_grid[qsl::kPostGrids];
};

namespace {

// The two batch job lists (main trace, pseudo-line trace) of a laid-out batch.
void job_lists(const qsl_qmap_batch& B, std::vector<qsl_batch_job>& mj, std::vector<qsl_batch_job>& sj) {
    mj.resize(B.njobs);
    sj.resize(B.njobs);
    for (int k = 0; k < B.njobs; ++k) {
        const qsl_qmap_job& j = B.jobs[k];
        const JobLayout& L = B.lay[k];
        qsl_batch_job a;
        memset(&a, 0, sizeof(a));
        a.field = j.field;
        a.params = j.params;
        a.s_len = j.s_len;
        a.tol_coef = j.tol_coef;
        for (int c = 0; c < 3; ++c) a.cross_dir[c] = (float)j.normal[c];
        qsl_batch_job s = a;
        a.io = io_of(B.ws, L, L.main, L.xs, L.ys, L.zs);
        a.n = L.n;
        a.order = L.order >= 0 ? (const uint32_t*)(B.ws + L.order) : nullptr;
        s.io = io_of(B.ws, L, L.sub, L.cut[0], L.cut[1], L.cut[2]);
        s.n = 4 * L.m;
        s.n_dev = (const unsigned long long*)(B.ws + L.count) + 1;
        mj[k] = a;
        sj[k] = s;
    }
}

// Bytes of the Q-assembly table of njobs jobs.
int64_t post_bytes(int njobs) {
    return up((int64_t)njobs * (int64_t)sizeof(qsl::QPostJob) + qsl::kPostGrids * (int64_t)(njobs + 1) * 8);
}

// The Q-assembly table of a laid-out batch, written to dst (post_bytes), and
// the three grid sizes.  Each job's arguments are those the per-job entries
// (qsl_qcalc_plane, qsl_cook_pseudo_line, qsl_qcut, qsl_qmerge) build from
// the same arrays.
int post_table(const qsl_qmap_batch& B, char* dst, long long grid[qsl::kPostGrids]) {
    using qsl::QPostJob;
    const int nj = B.njobs;
    QPostJob* T = reinterpret_cast<QPostJob*>(dst);
    long long* begin = reinterpret_cast<long long*>(dst + (size_t)nj * sizeof(QPostJob));
    for (int g = 0; g < qsl::kPostGrids; ++g) grid[g] = 0;
    char* w = B.ws;
    for (int k = 0; k < nj; ++k) {
        const qsl_qmap_job& j = B.jobs[k];
        const JobLayout& L = B.lay[k];
        const double jac = pow(1.0 / (2.0 * j.spacing), 4.0);
        auto F = [&](const int64_t* o, int i) { return (const float*)(w + o[i]); };
        auto I = [&](const int64_t* o, int i) { return (const int*)(w + o[i]); };
        QPostJob P;
        memset(&P, 0, sizeof(P));
        // qsl_qcalc_plane(end xyz flag, start xyz flag, B_start z, B_end z, B_this xyz, ..., Q64)
        qsl::QPlaneArgs& q = P.q;
        q.xe = F(L.main, 4); q.ye = F(L.main, 5); q.ze = F(L.main, 6); q.fe = I(L.main, 7);
        q.xs = F(L.main, 0); q.ys = F(L.main, 1); q.zs = F(L.main, 2); q.fs = I(L.main, 3);
        q.bz_in = F(L.main, 14); q.bz_out = F(L.main, 17);
        q.bx0 = F(L.main, 8); q.by0 = F(L.main, 9); q.bz0 = F(L.main, 10);
        q.cx = (float)j.normal[0]; q.cy = (float)j.normal[1]; q.cz = (float)j.normal[2];
        q.n0 = j.n0; q.n1 = j.n1; q.nplanes = j.nplanes;
        q.k32 = (float)jac; q.k64 = jac;
        q.q32 = nullptr; q.q64 = (double*)(w + L.q);
        // qsl_cook_pseudo_line(B_flag, start xyz flag, B_start z, B_end z, n, n0, n1, interior_only = 1, ...)
        P.tile_off = (long long*)(w + L.work);
        P.tile_count = (int*)(P.tile_off + qsl::cook_tiles(L.n));
        P.total = (unsigned long long*)(w + L.count);
        qsl::CookArgs& c = P.c;
        c.bflag = I(L.main, 11);
        c.xs = F(L.main, 0); c.ys = F(L.main, 1); c.zs = F(L.main, 2); c.fs = I(L.main, 3);
        c.bz_in = F(L.main, 14); c.bz_out = F(L.main, 17);
        c.n = L.n; c.n0 = j.n0; c.n1 = j.n1; c.interior_only = 1;
        c.stride = (float)j.spacing;
        c.tile_off = P.tile_off;
        c.cx = (float*)(w + L.cut[0]); c.cy = (float*)(w + L.cut[1]); c.cz = (float*)(w + L.cut[2]);
        c.bz0s = (float*)(w + L.bz0s); c.bz0e = (float*)(w + L.bz0e);
        c.pix = (long long*)(w + L.pix);
        // qsl_qcut(pseudo-line start xyz flag, end xyz flag, Bz0 start / end, count on the device, ...)
        qsl::QcutArgs& kc = P.k;
        kc.xs = F(L.sub, 0); kc.ys = F(L.sub, 1); kc.zs = F(L.sub, 2); kc.fs = I(L.sub, 3);
        kc.xe = F(L.sub, 4); kc.ye = F(L.sub, 5); kc.ze = F(L.sub, 6); kc.fe = I(L.sub, 7);
        kc.bz0s = c.bz0s; kc.bz0e = c.bz0e;
        kc.count_dev = P.total; kc.count = 0;
        kc.k32 = (float)jac; kc.k64 = jac;
        kc.q32 = nullptr; kc.q64 = (double*)(w + L.qcut);
        P.qblocks = qsl::qcalc_blocks(L.m);
        P.cblocks = qsl::qcalc_blocks(L.m);
        const long long sizes[qsl::kPostGrids] = {P.qblocks, qsl::cook_tiles(L.n), P.cblocks};
        for (int g = 0; g < qsl::kPostGrids; ++g) {
            begin[g * (nj + 1) + k] = grid[g];
            grid[g] += sizes[g];
        }
        memcpy(T + k, &P, sizeof(P));
    }
    for (int g = 0; g < qsl::kPostGrids; ++g) {
        begin[g * (nj + 1) + nj] = grid[g];
        if (grid[g] > 0x7fffffffLL) return qsl::set_error(QSL_ERR_TOO_LARGE, "batch too large for one Q-assembly grid");
    }
    return QSL_OK;
}

int sizes(const qsl_qmap_job* jobs, int njobs, std::vector<JobLayout>* lay, int64_t* arrays_bytes,
          int64_t* main_table, int64_t* sub_table, qsl_batch_info* mi, qsl_batch_info* si) {
    if (!jobs || njobs < 1) return qsl::set_error(QSL_ERR_INVALID, "a batch needs at least one job");
    std::vector<JobLayout> L(njobs);
    int64_t off = 0;
    for (int k = 0; k < njobs; ++k) {
        if (!job_ok(jobs[k]))
            return qsl::set_error(QSL_ERR_INVALID,
                                  "a job needs a field, n0, n1 >= 3, nplanes >= 1, a positive spacing and at most "
                                  "2^32 seeds");
        off = layout(jobs[k], off, L[k]);
    }
    // table sizes from a dry run of the job lists (addresses from a stand-in
    // base: the sizes do not depend on them, the checks want them non-null)
    qsl_qmap_batch B;
    B.njobs = njobs;
    B.jobs.assign(jobs, jobs + njobs);
    B.lay = L;
    B.ws = reinterpret_cast<char*>((uintptr_t)kAlign);
    std::vector<qsl_batch_job> mj, sj;
    job_lists(B, mj, sj);
    int rc = qsl_batch_pack(mj.data(), njobs, nullptr, 0, mi);
    if (rc != QSL_OK) return rc;
    rc = qsl_batch_pack(sj.data(), njobs, nullptr, 0, si);
    if (rc != QSL_OK) return rc;
    *arrays_bytes = off;
    *main_table = up(mi->table_bytes);
    *sub_table = up(si->table_bytes);
    if (lay) *lay = L;
    return QSL_OK;
}

int cuda_err(cudaError_t e) { return qsl::set_error(QSL_ERR_CUDA, cudaGetErrorString(e)); }

}  // namespace

extern "C" {

int qsl_qmap_batch_size(const qsl_qmap_job* jobs, int njobs, int64_t* device_bytes, int64_t* host_bytes) {
    if (!device_bytes || !host_bytes) return qsl::set_error(QSL_ERR_INVALID, "null output");
    int64_t arrays, mt, st;
    qsl_batch_info mi, si;
    const int rc = sizes(jobs, njobs, nullptr, &arrays, &mt, &st, &mi, &si);
    if (rc != QSL_OK) return rc;
    *device_bytes = arrays + mt + st + post_bytes(njobs);
    *host_bytes = mt + st + post_bytes(njobs);
    return QSL_OK;
}

int qsl_qmap_batch_create(const qsl_qmap_job* jobs, int njobs, void* workspace, int64_t workspace_bytes,
                          void* host_staging, int64_t host_bytes, qsl_stream_t stream, qsl_qmap_batch_t** out) {
    if (!out) return qsl::set_error(QSL_ERR_INVALID, "out is null");
    *out = nullptr;
    if (!workspace || !host_staging) return qsl::set_error(QSL_ERR_INVALID, "null workspace or staging buffer");
    if (((uintptr_t)workspace) % kAlign != 0) return qsl::set_error(QSL_ERR_INVALID, "workspace not 256-byte aligned");
    std::vector<JobLayout> lay;
    int64_t arrays, mt, st;
    qsl_batch_info mi, si;
    int rc = sizes(jobs, njobs, &lay, &arrays, &mt, &st, &mi, &si);
    if (rc != QSL_OK) return rc;
    const int64_t pt = post_bytes(njobs);
    if (workspace_bytes < arrays + mt + st + pt) return qsl::set_error(QSL_ERR_INVALID, "workspace too small");
    if (host_bytes < mt + st + pt) return qsl::set_error(QSL_ERR_INVALID, "host staging buffer too small");
    qsl_qmap_batch* B = new (std::nothrow) qsl_qmap_batch();
    if (!B) return qsl::set_error(QSL_ERR_NOMEM, "host allocation failed");
    B->njobs = njobs;
    B->jobs.assign(jobs, jobs + njobs);
    B->lay = lay;
    B->ws = (char*)workspace;
    B->main_table = arrays;
    B->sub_table = arrays + mt;
    B->post_table = arrays + mt + st;
    cudaStream_t s = (cudaStream_t)stream;
    // seed grids and tile orders, one launch each per job
    for (int k = 0; k < njobs && rc == QSL_OK; ++k) {
        const qsl_qmap_job& j = jobs[k];
        const JobLayout& L = lay[k];
        rc = qsl_plane_seeds(j.center, j.normal, j.u, j.v, j.spacing, j.n0, j.n1, j.nplanes, (float*)(B->ws + L.xs),
                             (float*)(B->ws + L.ys), (float*)(B->ws + L.zs), stream);
        if (rc == QSL_OK && L.order >= 0)
            rc = qsl_tile_order(j.nplanes, j.n0, j.n1, j.tile_y, j.tile_x, j.nplanes, (uint32_t*)(B->ws + L.order),
                                stream);
    }
    // the three job tables, serialised into the staging buffer and copied
    std::vector<qsl_batch_job> mj, sj;
    if (rc == QSL_OK) {
        job_lists(*B, mj, sj);
        rc = qsl_batch_pack(mj.data(), njobs, host_staging, mt, &B->main_info);
    }
    if (rc == QSL_OK) rc = qsl_batch_pack(sj.data(), njobs, (char*)host_staging + mt, st, &B->sub_info);
    if (rc == QSL_OK) rc = post_table(*B, (char*)host_staging + mt + st, B->post_grid);
    if (rc == QSL_OK) {
        const cudaError_t e = cudaMemcpyAsync(B->ws + B->main_table, host_staging, (size_t)(mt + st + pt),
                                              cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) rc = cuda_err(e);
    }
    if (rc != QSL_OK) {
        delete B;
        return rc;
    }
    *out = B;
    return QSL_OK;
}

int64_t qsl_qmap_batch_lines(const qsl_qmap_batch_t* B) {
    if (!B) return 0;
    int64_t t = 0;
    for (int k = 0; k < 4; ++k) t = B->main_info.total[k] > t ? B->main_info.total[k] : t;
    return t;
}

int qsl_qmap_batch_run_main(const qsl_qmap_batch_t* B, int64_t line_lo, int64_t line_hi, int max_blocks,
                            int occupancy, qsl_stream_t stream) {
    if (!B) return qsl::set_error(QSL_ERR_INVALID, "null batch");
    return qsl_batch_run_window(B->ws + B->main_table, &B->main_info, nullptr, line_lo, line_hi, max_blocks,
                                occupancy, stream);
}

int qsl_qmap_batch_run_post(const qsl_qmap_batch_t* B, int max_blocks, int occupancy, qsl_stream_t stream) {
    if (!B) return qsl::set_error(QSL_ERR_INVALID, "null batch");
    cudaStream_t s = (cudaStream_t)stream;
    const qsl::QPostJob* T = (const qsl::QPostJob*)(B->ws + B->post_table);
    const long long* begin = (const long long*)(B->ws + B->post_table + (int64_t)B->njobs * sizeof(qsl::QPostJob));
    // Q of every job, then the compaction of its flagged pixels into
    // pseudo-line seeds
    cudaError_t e = qsl::launch_qpost_assemble(T, begin, B->njobs, B->post_grid, s);
    if (e != cudaSuccess) return cuda_err(e);
    const int rc = qsl_batch_run_window(B->ws + B->sub_table, &B->sub_info, nullptr, 0, -1, max_blocks, occupancy,
                                        stream);
    if (rc != QSL_OK) return rc;
    // Q of the pseudo-lines, merged into each map
    e = qsl::launch_qpost_pseudo(T, begin, B->njobs, B->post_grid, s);
    return e == cudaSuccess ? QSL_OK : cuda_err(e);
}

double* qsl_qmap_batch_q(const qsl_qmap_batch_t* B, int job) {
    if (!B || job < 0 || job >= B->njobs) return nullptr;
    return (double*)(B->ws + B->lay[job].q);
}

int qsl_qmap_batch_destroy(qsl_qmap_batch_t* B) {
    delete B;
    return QSL_OK;
}

}  // extern "C"
