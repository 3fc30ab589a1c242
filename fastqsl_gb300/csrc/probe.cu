// L1 load-bandwidth probe: the ceiling of the tracers' 16-byte field gathers.
//
// Every warp request loads one 16-byte word per lane (ld.global.nc.v4, the
// tracers' load) from a buffer small enough to stay in each SM's L1, with
// its 32 lanes spread over `spread` 128-byte lines (4 = a coalesced 512-byte
// request; more lines per request = a scattered gather).  Eight independent
// loads per iteration keep the load pipe busy; the results are folded into
// one word so that no load is dead.
#include "qsl_internal.h"

namespace qsl {

__global__ void __launch_bounds__(kTraceBlock) k_l1_probe(const uint4* __restrict__ buf, unsigned mask_u4,
                                                          int spread, int iters, unsigned* __restrict__ sink) {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned s = (unsigned)spread;
    // lane -> (line, slot): lanes l, l + s, l + 2s, ... share line l % s
    const unsigned off = (lane % s) * 8u + (lane / s) % 8u;
    unsigned base = (blockIdx.x * 97u + (threadIdx.x >> 5) * 31u) * 8u * s;
    unsigned acc = 0;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const uint4 v = __ldg(buf + ((base + (unsigned)u * 8u * s + off) & mask_u4));
            acc ^= v.x ^ v.w;
        }
        base += 64u * s;
    }
    if (acc == 0x9e3779b9u) sink[0] = acc;  // never true for the zeroed buffer the probe is given
}

}  // namespace qsl

extern "C" int qsl_l1_probe(const void* buf, int64_t buf_bytes, int spread, int blocks, int iters,
                            unsigned* sink, qsl_stream_t stream) {
    using namespace qsl;
    if (!buf || !sink || blocks <= 0 || iters <= 0) return QSL_ERR_INVALID;
    if (spread != 1 && spread != 2 && spread != 4 && spread != 8 && spread != 16 && spread != 32)
        return QSL_ERR_INVALID;
    // a power-of-two number of 16-byte words, at least one window of 32 lines
    if (buf_bytes < 4096 || (buf_bytes & (buf_bytes - 1)) != 0 || buf_bytes > (1LL << 30)) return QSL_ERR_INVALID;
    if ((reinterpret_cast<uintptr_t>(buf) & 15) != 0) return QSL_ERR_INVALID;
    const unsigned mask = (unsigned)(buf_bytes / 16 - 1);
    k_l1_probe<<<blocks, kTraceBlock, 0, (cudaStream_t)stream>>>(reinterpret_cast<const uint4*>(buf), mask, spread,
                                                                  iters, sink);
    return cudaGetLastError() == cudaSuccess ? QSL_OK : QSL_ERR_CUDA;
}
