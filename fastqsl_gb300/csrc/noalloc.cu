// qsl_cook_pseudo_line_noalloc: the pseudo-line compaction of
// qsl_cook_pseudo_line with its scratch memory in a fixed device array of
// this library instead of a caller-supplied workspace, for callers that have
// no way to allocate device memory (see include/fastqsl_gb300.h).
//
// The scratch (per-tile pixel counts and their prefix offsets, 12 bytes per
// 1024 pixels) lives in g_cook_scratch below: every GPU that loads the
// library holds it until the process exits, and every call on that GPU uses
// the same bytes.
#include <cuda_runtime.h>
#include <stdio.h>

#include <mutex>

#include "../../include/fastqsl_gb300.h"
#include "qassembly.h"

namespace qsl {
int set_error(int code, const char* msg);
}

namespace {

constexpr long long kScratchBytes = QSL_NOALLOC_SCRATCH_BYTES;

__device__ __align__(256) unsigned char g_cook_scratch[kScratchBytes];

// Host code cannot use g_cook_scratch's name as a device address; its
// address on each device is looked up once, with that device current, and
// again whenever the device's current context is a different one (after
// cudaDeviceReset the module is loaded anew and the array may move).  The
// context handle comes from the driver's cuCtxGetCurrent, reached through the
// runtime's entry-point query so the library needs no link to libcuda.
constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_addr[kMaxDevices];
void* g_scratch_ctx[kMaxDevices];
bool g_scratch_ready[kMaxDevices];

typedef int (*ctx_get_current_t)(void**);

void* current_context() {
    static ctx_get_current_t fn = nullptr;
    static bool looked = false;
    if (!looked) {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (ctx_get_current_t)f;
        looked = true;
    }
    void* ctx = nullptr;
    if (fn && fn(&ctx) != 0) ctx = nullptr;
    return ctx;
}

int scratch_on_current_device(void** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return qsl::set_error(QSL_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return qsl::set_error(QSL_ERR_INVALID, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_ready[dev] || g_scratch_ctx[dev] != current_context()) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_cook_scratch);
        if (e != cudaSuccess || p == nullptr) {
            char msg[256];
            snprintf(msg, sizeof(msg), "cudaGetSymbolAddress(g_cook_scratch): %s", cudaGetErrorString(e));
            return qsl::set_error(QSL_ERR_CUDA, msg);
        }
        g_scratch_addr[dev] = p;
        // taken after the lookup, which makes the device's primary context
        // current if no context was
        g_scratch_ctx[dev] = current_context();
        g_scratch_ready[dev] = true;
    }
    *out = g_scratch_addr[dev];
    return QSL_OK;
}

}  // namespace

extern "C" {

int64_t qsl_cook_noalloc_max_pixels(void) {
    // tiles * (8 + 4) bytes of scratch, kTile = 1024 pixels per tile
    const long long tiles = (kScratchBytes - 64) / (long long)(sizeof(long long) + sizeof(int));
    return (int64_t)(tiles * 1024);
}

int qsl_cook_pseudo_line_noalloc(const int* B_flag, const float* x_start, const float* y_start,
                                 const float* z_start, const int* flag_start, const float* Bz_in, const float* Bz_out,
                                 int64_t n, int n0, int n1, int interior_only, float stride, float* cut_x,
                                 float* cut_y, float* cut_z, float* Bz0_start, float* Bz0_end, int64_t* pix,
                                 unsigned long long* count_dev, qsl_stream_t stream) {
    if (!B_flag || !x_start || !y_start || !z_start || !flag_start || !Bz_in || !Bz_out || !cut_x || !cut_y ||
        !cut_z || !Bz0_start || !Bz0_end || !count_dev)
        return qsl::set_error(QSL_ERR_INVALID, "null pointer");
    if (n < 0) return qsl::set_error(QSL_ERR_INVALID, "negative n");
    if (interior_only && (n0 < 1 || n1 < 1 || n % ((int64_t)n0 * n1) != 0))
        return qsl::set_error(QSL_ERR_INVALID, "interior_only needs n a multiple of n0*n1");
    if (n > qsl_cook_noalloc_max_pixels()) {
        char msg[256];
        snprintf(msg, sizeof(msg),
                 "qsl_cook_pseudo_line_noalloc: %lld pixels exceed the fixed scratch (%lld bytes, at most %lld "
                 "pixels); use qsl_cook_pseudo_line with a workspace",
                 (long long)n, kScratchBytes, (long long)qsl_cook_noalloc_max_pixels());
        return qsl::set_error(QSL_ERR_TOO_LARGE, msg);
    }
    void* scratch = nullptr;
    const int rc = scratch_on_current_device(&scratch);
    if (rc != QSL_OK) return rc;
    // Every value the kernels read from the scratch is written earlier in
    // the same call (tile counts, then their prefix offsets), so nothing
    // needs clearing between calls.
    const long long tiles = qsl::cook_tiles(n);
    long long* tile_off = (long long*)scratch;
    int* tile_count = (int*)(tile_off + tiles);
    qsl::CookArgs a;
    a.bflag = B_flag; a.xs = x_start; a.ys = y_start; a.zs = z_start; a.fs = flag_start;
    a.bz_in = Bz_in; a.bz_out = Bz_out; a.n = n; a.n0 = n0; a.n1 = n1; a.interior_only = interior_only;
    a.stride = stride; a.tile_off = tile_off;
    a.cx = cut_x; a.cy = cut_y; a.cz = cut_z; a.bz0s = Bz0_start; a.bz0e = Bz0_end; a.pix = (long long*)pix;
    const cudaError_t e = qsl::launch_cook(a, tile_count, tile_off, count_dev, (cudaStream_t)stream);
    if (e != cudaSuccess) return qsl::set_error(QSL_ERR_CUDA, cudaGetErrorString(e));
    return QSL_OK;
}

}  // extern "C"
