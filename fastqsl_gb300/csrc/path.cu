// Field-line polylines for plotting: the fixed-step RK4 tracer of
// fastqslpy/MagTool.py (trilerp :3-18, Bnorm :20-22, RK4_bline :24-34,
// TraceBline :36-45), which records every point of a line instead of its
// footpoints.  That module computes in float64 (its weights come from
// float32 positions minus int64 indices, so every product and sum after the
// corner gather is float64) and stores the points as float32; each thread
// here follows one line in the same operation order with IEEE float64 adds,
// multiplies, divides and square roots (this translation unit is compiled
// with -fmad=false), so the stored points agree bit for bit.
//
// Behaviour kept from that module:
//  * a position is clamped per axis before sampling: below 0 -> 1e-8, above
//    n -> n - 1e-8; corner indices past the last node repeat the last node
//    (its slices come back shorter and broadcast);
//  * the 8 corner products are summed as a contiguous (2, 2, 2) float64
//    array: ((p000+p001)+(p010+p011)) + ((p100+p101)+(p110+p111)), index
//    order [x][y][z]; |B|^2 is summed x, y, z in sequence;
//  * the loop stops when any coordinate is below 0 or above nx (the first
//    axis length bounds all three); the current point is clamped in place at
//    the first sample of each step, and that clamped point is stored and
//    advanced.
// Where that module raises (a zero field sample gives NaN, a point exactly
// on the far face slices past the array), a line here stops at the NaN and
// clamps the index to the last node.
#include "qsl_internal.h"

namespace qsl {

struct PathField {
    const float *bx, *by, *bz;
    int n[3];
};

__device__ __forceinline__ double clamp_ref(double v, int n) {
    if (v < 0.0) return 1e-8;
    if (v > (double)n) return __dsub_rn((double)n, 1e-8);
    return v;
}

// trilerp (MagTool.py:3-18) at the clamped point c
__device__ void trilerp_ref(const PathField& F, const double c[3], double b[3]) {
    long long i0[3], i1[3];
    double w[3][2];
    for (int d = 0; d < 3; ++d) {
        long long i = (long long)c[d];  // truncation; c >= 0 after the clamp (NaN converts to 0)
        i = i < 0 ? 0 : (i > F.n[d] - 1 ? F.n[d] - 1 : i);
        i0[d] = i;
        i1[d] = i + 1 > F.n[d] - 1 ? F.n[d] - 1 : i + 1;
        const double f = __dsub_rn(c[d], (double)i);
        w[d][0] = __dsub_rn(1.0, f);
        w[d][1] = f;
    }
    const long long sx = 1, sy = F.n[0], sz = (long long)F.n[0] * F.n[1];
    const float* comp[3] = {F.bx, F.by, F.bz};
    for (int q = 0; q < 3; ++q) {
        double p[8];
        for (int i = 0; i < 2; ++i)
            for (int j = 0; j < 2; ++j)
                for (int k = 0; k < 2; ++k) {
                    const long long o = (i ? i1[0] : i0[0]) * sx + (j ? i1[1] : i0[1]) * sy + (k ? i1[2] : i0[2]) * sz;
                    const double wt = __dmul_rn(__dmul_rn(w[0][i], w[1][j]), w[2][k]);
                    p[i * 4 + j * 2 + k] = __dmul_rn((double)__ldg(comp[q] + o), wt);
                }
        b[q] = __dadd_rn(__dadd_rn(__dadd_rn(p[0], p[1]), __dadd_rn(p[2], p[3])),
                         __dadd_rn(__dadd_rn(p[4], p[5]), __dadd_rn(p[6], p[7])));
    }
}

// Bnorm (MagTool.py:20-22) at v (clamped on a copy)
__device__ void bnorm_ref(const PathField& F, const double v[3], double u[3]) {
    double c[3], b[3];
    for (int d = 0; d < 3; ++d) c[d] = clamp_ref(v[d], F.n[d]);
    trilerp_ref(F, c, b);
    const double s = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(b[0], b[0]), __dmul_rn(b[1], b[1])), __dmul_rn(b[2], b[2])));
    for (int d = 0; d < 3; ++d) u[d] = __ddiv_rn(b[d], s);
}

struct PathArgs {
    PathField F;
    const double* seeds;  // n x 3
    long long n;
    long long start, stop, stride;  // Python range(start, stop, stride) of output indices
    double dr;
    float *ox, *oy, *oz;  // n x out_len
    long long out_len;
};

// RK4_bline (MagTool.py:24-34) for one seed per thread
__global__ void __launch_bounds__(64) k_trace_path(const PathArgs A) {
    const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= A.n) return;
    double P[3] = {A.seeds[3 * s], A.seeds[3 * s + 1], A.seeds[3 * s + 2]};
    const double bound = (double)A.F.n[0];
    float* ox = A.ox + s * A.out_len;
    float* oy = A.oy + s * A.out_len;
    float* oz = A.oz + s * A.out_len;
    const double dr = A.dr;
    for (long long idx = A.start; A.stride > 0 ? idx < A.stop : idx > A.stop; idx += A.stride) {
        if (P[0] < 0.0 || P[1] < 0.0 || P[2] < 0.0 || P[0] > bound || P[1] > bound || P[2] > bound) break;
        if (isnan(P[0]) || isnan(P[1]) || isnan(P[2])) break;
        for (int d = 0; d < 3; ++d) P[d] = clamp_ref(P[d], A.F.n[d]);
        double f1[3], f2[3], f3[3], f4[3], t[3];
        bnorm_ref(A.F, P, f1);
        for (int d = 0; d < 3; ++d) t[d] = __dadd_rn(P[d], __dmul_rn(dr, f1[d]) * 0.5);
        bnorm_ref(A.F, t, f2);
        for (int d = 0; d < 3; ++d) t[d] = __dadd_rn(P[d], __dmul_rn(dr, f2[d]) * 0.5);
        bnorm_ref(A.F, t, f3);
        for (int d = 0; d < 3; ++d) t[d] = __dadd_rn(P[d], __dmul_rn(dr, f3[d]));
        bnorm_ref(A.F, t, f4);
        ox[idx] = (float)P[0];
        oy[idx] = (float)P[1];
        oz[idx] = (float)P[2];
        for (int d = 0; d < 3; ++d) {
            const double k = __dadd_rn(__dadd_rn(__dadd_rn(f1[d], 2.0 * f2[d]), 2.0 * f3[d]), f4[d]);
            P[d] = __dadd_rn(P[d], __ddiv_rn(__dmul_rn(dr, k), 6.0));
        }
    }
}

struct SampleArgs {
    PathField F;
    const double* pts;  // n x 3
    long long n;
    int normalize;
    double* out;  // n x 3
};

__global__ void __launch_bounds__(128) k_sample_points(const SampleArgs A) {
    const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= A.n) return;
    const double v[3] = {A.pts[3 * s], A.pts[3 * s + 1], A.pts[3 * s + 2]};
    double r[3];
    if (A.normalize) {
        bnorm_ref(A.F, v, r);
    } else {
        double c[3];
        for (int d = 0; d < 3; ++d) c[d] = clamp_ref(v[d], A.F.n[d]);
        trilerp_ref(A.F, c, r);
    }
    for (int d = 0; d < 3; ++d) A.out[3 * s + d] = r[d];
}

cudaError_t launch_trace_path(const float* bx, const float* by, const float* bz, int nx, int ny, int nz,
                              const double* seeds, long long n, long long start, long long stop, long long stride,
                              double dr, float* ox, float* oy, float* oz, long long out_len, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const PathArgs A{{bx, by, bz, {nx, ny, nz}}, seeds, n, start, stop, stride, dr, ox, oy, oz, out_len};
    k_trace_path<<<(unsigned)((n + 63) / 64), 64, 0, st>>>(A);
    return cudaGetLastError();
}

cudaError_t launch_sample_points(const float* bx, const float* by, const float* bz, int nx, int ny, int nz,
                                 const double* pts, long long n, int normalize, double* out, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const SampleArgs A{{bx, by, bz, {nx, ny, nz}}, pts, n, normalize, out};
    k_sample_points<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(A);
    return cudaGetLastError();
}

}  // namespace qsl
