// Seed geometry on the device: the seed grid of stacked planes and the tile
// visiting order of a stack, one launch each.  Both replace sequences of
// framework tensor operations (a dozen element-wise launches, a sort) whose
// host cost dominated small Q-map requests.
#include "qsl_internal.h"

namespace qsl {

int set_error(int code, const char* msg);

// Seed q = (k * n0 + i) * n1 + j of nplanes stacked (n0, n1) planes:
//   ((c + (k s) N) + (di s) V) + (dj s) U,  di = i - (n0 - 1) / 2, dj = j - (n1 - 1) / 2,
// every product and sum rounded in double on its own (no contraction), then
// rounded to float.
__global__ void k_plane_seeds(double3 c, double3 nn, double3 u, double3 v, double s, int n0, int n1,
                              long long total, float* __restrict__ xs, float* __restrict__ ys,
                              float* __restrict__ zs) {
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(q % n1);
        const long long r = q / n1;
        const int i = (int)(r % n0);
        const long long k = r / n0;
        const double kk = __dmul_rn((double)k, s);
        const double ii = __dmul_rn((double)i - (double)(n0 - 1) / 2.0, s);
        const double jj = __dmul_rn((double)j - (double)(n1 - 1) / 2.0, s);
        const double x = __dadd_rn(__dadd_rn(__dadd_rn(c.x, __dmul_rn(kk, nn.x)), __dmul_rn(ii, v.x)), __dmul_rn(jj, u.x));
        const double y = __dadd_rn(__dadd_rn(__dadd_rn(c.y, __dmul_rn(kk, nn.y)), __dmul_rn(ii, v.y)), __dmul_rn(jj, u.y));
        const double z = __dadd_rn(__dadd_rn(__dadd_rn(c.z, __dmul_rn(kk, nn.z)), __dmul_rn(ii, v.z)), __dmul_rn(jj, u.z));
        xs[q] = __double2float_rn(x);
        ys[q] = __double2float_rn(y);
        zs[q] = __double2float_rn(z);
    }
}

// Tile order: seeds sorted by (plane group, tile row, tile column, plane in
// the group, row in the tile, column in the tile).  Each seed's rank is
// the number of seeds before it in that order, in closed form:
//   full plane groups before + full tile rows before (G planes each) + tiles
//   before in this tile row (height h) + planes before in this tile (h x w
//   seeds) + rows before in this plane of the tile (w) + columns before,
// G = planes in this group, h x w this tile's size (smaller at the far
// edges); order[rank] = the seed's index.
__global__ void k_tile_order(int nplanes, int n0, int n1, int ty, int tx, int g, long long total,
                             unsigned* __restrict__ order) {
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(q % n1);
        const long long r = q / n1;
        const int y = (int)(r % n0);
        const int p = (int)(r / n0);
        const int pg = p / g, pp = p % g;
        const int ti = y / ty, tj = x / tx;
        const long long G = min(g, nplanes - pg * g);
        const long long h = min(ty, n0 - ti * ty);
        const long long w = min(tx, n1 - tj * tx);
        const long long rank = (long long)pg * g * n0 * n1 + G * ((long long)ti * ty) * n1 +
                               G * h * ((long long)tj * tx) + (long long)pp * h * w + (long long)(y % ty) * w +
                               (x % tx);
        order[rank] = (unsigned)q;
    }
}

static int grid_for(long long total) {
    const long long b = (total + 255) / 256;
    return (int)(b < 65535LL * 16 ? (b > 0 ? b : 1) : 65535LL * 16);
}

}  // namespace qsl

extern "C" int qsl_plane_seeds(const double* center_h, const double* normal_h, const double* u_h, const double* v_h,
                               double spacing, int n0, int n1, int nplanes, float* xs, float* ys, float* zs,
                               qsl_stream_t stream) {
    using namespace qsl;
    if (!center_h || !normal_h || !u_h || !v_h || !xs || !ys || !zs) return set_error(QSL_ERR_INVALID, "null pointer");
    if (n0 < 1 || n1 < 1 || nplanes < 1) return set_error(QSL_ERR_INVALID, "n0, n1 and nplanes must be positive");
    const long long total = (long long)n0 * n1 * nplanes;
    const double3 c = make_double3(center_h[0], center_h[1], center_h[2]);
    const double3 nn = make_double3(normal_h[0], normal_h[1], normal_h[2]);
    const double3 u = make_double3(u_h[0], u_h[1], u_h[2]);
    const double3 v = make_double3(v_h[0], v_h[1], v_h[2]);
    k_plane_seeds<<<grid_for(total), 256, 0, (cudaStream_t)stream>>>(c, nn, u, v, spacing, n0, n1, total, xs, ys, zs);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? QSL_OK : set_error(QSL_ERR_CUDA, cudaGetErrorString(e));
}

extern "C" int qsl_tile_order(int nplanes, int n0, int n1, int ty, int tx, int plane_group, uint32_t* order,
                              qsl_stream_t stream) {
    using namespace qsl;
    if (!order) return set_error(QSL_ERR_INVALID, "null pointer");
    if (n0 < 1 || n1 < 1 || nplanes < 1 || ty < 1 || tx < 1)
        return set_error(QSL_ERR_INVALID, "sizes and tile edges must be positive");
    const long long total = (long long)n0 * n1 * nplanes;
    if (total > 0xffffffffLL) return set_error(QSL_ERR_TOO_LARGE, "an order map indexes at most 2^32 seeds");
    const int g = plane_group > 0 && plane_group < nplanes ? plane_group : nplanes;
    k_tile_order<<<grid_for(total), 256, 0, (cudaStream_t)stream>>>(nplanes, n0, n1, ty, tx, g, total, order);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? QSL_OK : set_error(QSL_ERR_CUDA, cudaGetErrorString(e));
}
