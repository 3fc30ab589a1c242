// Field stores and trilinear sampling for the GB300 tracer.
//
// Three layouts of the same (nx, ny, nz) node grid:
//   FieldSoA  — the caller's three float32 arrays, x fastest (the reference
//               layout, fastqslpy/cu/TraceBlineAdaptive.cu:36-39); one corner
//               costs three 4-byte gathers.
//   FieldF4   — interleaved float4 (Bx, By, Bz, 0) per node; one corner is one
//               16-byte load.
//   FieldH4B  — 8x8x8-cell bricks with a one-node apron on the + side (9^3
//               nodes), each node four fp16 (Bx, By, Bz, 0) scaled by a
//               per-brick float, stored as x-pair records (node i and i+1
//               in 16 bytes); one x-pair of corners is one 16-byte load and
//               a whole trilinear stencil never leaves its brick.
//   FieldH8C  — fp16 cell records: each cell holds the 8 corner vectors it
//               interpolates (64 bytes, power-of-two scale per cell), so a
//               trilinear sample is one 32-byte and one 16-byte load, each a
//               single L1 sector, instead of eight node loads spread over
//               several sectors.  Nodes are stored up to 8 times over (about
//               64 B per cell against 11 B for FieldH4B).
//   FieldStretch — the caller's SoA arrays on a stretched (rectilinear)
//               grid: node coordinates per axis, cells found by the
//               reference's search (fastqslpy/cu/TraceBlineAdaptiveStretch.cu).
//
// Sampling comes in two arithmetics:
//   exact — the reference's rounding sequence (weights formed in double and
//           narrowed, IEEE divide and sqrt).  Only instantiated in translation
//           units compiled with -fmad=false, so no multiply-add is fused.
//   fast  — float weights, fused multiply-add, rsqrt normalisation.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace qsl {

// ---------------------------------------------------------------------------
// small vector helpers (own code; semantics of plain per-component float ops)
// ---------------------------------------------------------------------------
__device__ __forceinline__ float3 v3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return v3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float3 operator/(float3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float norm(float3 a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }
// |a| with the hardware square-root approximation (sqrt.approx.ftz.f32,
// relative error ~2^-22): the fast stepper's error norm and step length, where the
// IEEE square root's range checks and fix-up cost more than they are worth
__device__ __forceinline__ float norm_fast(float3 a) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(fmaf(a.x, a.x, fmaf(a.y, a.y, a.z * a.z))));
    return r;
}
// 1/sqrt(x) by the hardware approximation with subnormal inputs flushed to
// zero (rsqrt.approx.ftz.f32): the fast samplers' normalisation, where |B|^2
// is far above the subnormal range whenever B/|B| is defined
__device__ __forceinline__ float rsqrt_fast(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
// x / y as x times the hardware reciprocal approximation (rcp.approx.ftz.f32,
// relative error ~2^-23; y is a cell width, far from the subnormal range),
// the product rounded on its own (__fmul_rn is never merged into a fused
// multiply-add), so that every kernel that inlines it gets the same bits
__device__ __forceinline__ float div_fast(float x, float y) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(y));
    return __fmul_rn(x, r);
}
__device__ __forceinline__ float comp(float3 a, int d) { return d == 0 ? a.x : (d == 1 ? a.y : a.z); }

struct Dims {
    int nx, ny, nz;
    __device__ __forceinline__ int n(int d) const { return d == 0 ? nx : (d == 1 ? ny : nz); }
};

// ---------------------------------------------------------------------------
// Field stores.  corners() returns the 8 node vectors of cell (ix, iy, iz) in
// corner order q = (dx<<2)|(dy<<1)|dz, and the multiplier that turns them into
// field units (1 except for fp16 bricks).
// ---------------------------------------------------------------------------
struct FieldSoA {
    const float* bx;
    const float* by;
    const float* bz;
    Dims d;
    __device__ __forceinline__ float corners(int ix, int iy, int iz, float3 c[8]) const {
        const int64_t sx = 1, sy = d.nx, sz = (int64_t)d.nx * d.ny;
        const int64_t base = ix + sy * iy + sz * iz;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int64_t o = base + ((q >> 2) & 1) * sx + ((q >> 1) & 1) * sy + (q & 1) * sz;
            c[q] = v3(__ldg(bx + o), __ldg(by + o), __ldg(bz + o));
        }
        return 1.0f;
    }
    __device__ __forceinline__ float scalar(int m, int64_t o) const {
        return __ldg((m == 0 ? bx : (m == 1 ? by : bz)) + o);
    }
};

struct FieldF4 {
    const float4* b;
    Dims d;
    __device__ __forceinline__ float corners(int ix, int iy, int iz, float3 c[8]) const {
        const int64_t sy = d.nx, sz = (int64_t)d.nx * d.ny;
        const int64_t base = ix + sy * iy + sz * iz;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int64_t o = base + ((q >> 2) & 1) + ((q >> 1) & 1) * sy + (q & 1) * sz;
            const float4 v = __ldg(b + o);
            c[q] = v3(v.x, v.y, v.z);
        }
        return 1.0f;
    }
};

// fp16 brick store: brick (bi, bj, bk) holds nodes [8bi, 8bi+8] x [8bj, 8bj+8]
// x [8bk, 8bk+8] (clamped at the far faces) as x-pair records: record a of
// row (b, c) is the 16-byte pair {node (a, b, c), node (a + 1, b, c)}, each
// node four fp16 (Bx, By, Bz, 0), a = 0..7; a row is 8 records = 128 B, a
// brick 81 rows = BRICK_U4 uint4 (10368 B).  A trilinear stencil is then 4
// 16-byte loads (rows (b, c), (b+1, c), (b, c+1), (b+1, c+1) at record a)
// instead of 8 node loads: the L1 data path costs about one cycle per
// distinct 128-byte line a warp request touches, at any load width up to
// 16 bytes, so halving the requests halves that cost; nodes are stored
// twice over (10368 against 5832 B per brick).
constexpr int BRICK_CELLS = 8;
constexpr int BRICK_NODES = 9;
constexpr int BRICK_U4 = 648;  // 81 rows x 8 records
struct FieldH4B {
    const uint4* bricks;
    const float* scale;  // per brick
    Dims d;
    int nbx, nby;        // bricks along x and y
    // record index of cell (ix, iy, iz) = h4b_record(): brick * BRICK_U4 +
    // (ix & 7) + 8 (iy & 7) + 72 (iz & 7) regrouped per axis as
    // ix + 640 (ix >> 3) + 8 iy + ky (iy >> 3) + 72 iz + kz (iz >> 3)
    unsigned ky, kz;     // BRICK_U4 nbx - 64, BRICK_U4 nbx nby - 576
    __device__ __forceinline__ float corners(int ix, int iy, int iz, float3 c[8]) const {
        const int bi = ix >> 3, bj = iy >> 3, bk = iz >> 3;
        const int64_t brick = bi + (int64_t)nbx * (bj + (int64_t)nby * bk);
        const uint4* bp = bricks + brick * BRICK_U4 + (ix & 7) + 8 * ((iy & 7) + BRICK_NODES * (iz & 7));
#pragma unroll
        for (int q = 0; q < 4; ++q) {  // q = (dy << 1) | dz
            const uint4 r = __ldg(bp + ((q >> 1) & 1) * 8 + (q & 1) * (8 * BRICK_NODES));
            const unsigned lo[2] = {r.x, r.y}, hi[2] = {r.z, r.w};
#pragma unroll
            for (int dx = 0; dx < 2; ++dx) {
                const unsigned* u = dx ? hi : lo;
                const float2 xy = __half22float2(*reinterpret_cast<const __half2*>(&u[0]));
                const float z = __half2float(__ushort_as_half((unsigned short)(u[1] & 0xffffu)));
                c[(dx << 2) | q] = v3(xy.x, xy.y, z);
            }
        }
        return __ldg(scale + brick);
    }
};
// The same brick store sampled with fp16 x weights (QSL_ARITH_FAST_W16, an
// opt-in of qsl_trace): a distinct type so that its kernels are compiled
// apart and the default sampler keeps FP32 weights.
struct FieldH4BW : FieldH4B {};

// fp16 cell records.  Record (64 bytes, 32-byte aligned) as 16 32-bit words:
// w[0..3] Bx, w[4..7] By, w[8..11] Bz, where word k of a component is the
// fp16 pair (low half: corner dx = 0, high half: corner dx = 1) of corner
// column k = (dy << 1) | dz; w[12] the cell's scale (a power of two, so the
// fp16 value of a node is the same in every cell that holds it); w[13..15]
// zero.  Cells are grouped in 8^3 bricks; cell (a, b, c) of brick
// (bi, bj, bk) is record 512 * (bi + nbx (bj + nby bk)) + a + 8 (b + 8 c).
constexpr int CELL_RECORD_U4 = 4;  // uint4 per record
struct FieldH8C {
    const uint4* cells;
    Dims d;
    int nbx, nby;  // bricks along x and y
    __device__ __forceinline__ unsigned long long record_index(int ix, int iy, int iz) const {
        // brick indices fit 32 bits (field stores hold < 1.1e12 nodes)
        const unsigned brick =
            (unsigned)(ix >> 3) + (unsigned)nbx * ((unsigned)(iy >> 3) + (unsigned)nby * (unsigned)(iz >> 3));
        const unsigned local = (unsigned)((ix & 7) + 8 * ((iy & 7) + 8 * (iz & 7)));
        return ((unsigned long long)brick << 9) + local;
    }
    __device__ __forceinline__ const uint4* record(int ix, int iy, int iz) const {
        return cells + record_index(ix, iy, iz) * CELL_RECORD_U4;
    }
    __device__ __forceinline__ float corners(int ix, int iy, int iz, float3 c[8]) const {
        const uint4* r = record(ix, iy, iz);
        const uint4 wx = __ldg(r), wy = __ldg(r + 1), wz = __ldg(r + 2);
        const unsigned ux[4] = {wx.x, wx.y, wx.z, wx.w}, uy[4] = {wy.x, wy.y, wy.z, wy.w},
                       uz[4] = {wz.x, wz.y, wz.z, wz.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float2 x = __half22float2(*reinterpret_cast<const __half2*>(&ux[k]));
            const float2 y = __half22float2(*reinterpret_cast<const __half2*>(&uy[k]));
            const float2 z = __half22float2(*reinterpret_cast<const __half2*>(&uz[k]));
            c[k] = v3(x.x, y.x, z.x);      // dx = 0
            c[4 + k] = v3(x.y, y.y, z.y);  // dx = 1
        }
        return __ldg(reinterpret_cast<const float*>(r + 3));
    }
};

// Stretched grid: the SoA arrays plus increasing node coordinates ax[nx],
// ay[ny], az[nz].  uni selects the reference's uniform-spacing index formula
// instead of its search; lo/hi are the first and last coordinates (set at
// kernel start from the coordinate arrays).
// M (mode) fixes the cell search at compile time, so each inlined sample
// carries one search only (the loop body is instruction-fetch bound):
// 1 and 2 = packed: the node values come from an interleaved float4 copy
// (b4: one 16-byte load per corner instead of three 4-byte gathers; the same
// float values, so the same results); 1 = per-axis tables (srec, sbin; built
// by launch_stretch_tables) that give the reference search's own cell for
// every coordinate in one or two dependent loads instead of ~log2(n); 2 = the
// uniform-spacing formula.  3, 4 and 5 read the caller's arrays: 3 with the
// tables (the twist current density of a packed search launch), 4 with the
// formula (the drop-in's uniform form and the current density of a packed
// uniform launch), 5 with the reference's bisection (the drop-in's search
// form).  The drop-in, whose choice (flag_uni) lives on the device, launches
// the 4 and 5 kernels and each returns at once unless the flag is its own.
template <int M>
struct FieldStretchT {
    const float* bx;
    const float* by;
    const float* bz;
    Dims d;
    const float* ax;
    const float* ay;
    const float* az;
    const bool* uni_dev;  // drop-in: the kernel runs only if *uni_dev matches its mode
    float3 lo, hi;        // first and last node coordinates (read at kernel start)
    float3 clo, chi;      // lo + 1e-6 and hi - 1e-6, formed in double and narrowed
    float3 us;            // uniform-formula spacing (hi - lo) / n
    const float4* b4;     // packed: x-pair records {node o, node o + 1}, two float4 (Bx, By, Bz, 0) each,
                          // o = ix + nx (iy + ny iz) (one 32-byte load per x corner pair)
    // search tables (M = 1), axes x, y, z one after another (axis k starts at
    // cell offset stretch_cell_offset(k)):
    //   srec[j]  the cell the reference's search gives for any coordinate in
    //            (a[j], a[j+1]] and its first coordinate and width:
    //            {a[i], a[i+1] - a[i], i as int bits, 0}
    //   sbin[2b], sbin[2b+1]  STRETCH_BINS_PER_CELL * (n - 1) uniform bins
    //            over [a[0], a[n-1]] per axis, each covering the cells a
    //            coordinate of the bin (widened by 1 % of a bin plus 4e-7 nb
    //            bins, the float rounding of the bin index) can lie in: for
    //            one or two cells their srec records and the node between
    //            them, else the range (k_stretch_tables)
    const float4* srec;
    const float4* sbin;
    float3 sbinv;         // search tables (M = 1, 3): bins per unit coordinate; uniform formula
                          // (M = 2, 4): 1 / us, the fast arithmetic's reciprocal (set at kernel start)
    __device__ __forceinline__ float corners(int ix, int iy, int iz, float3 c[8]) const {
        if constexpr (M == 1 || M == 2) {
#pragma unroll
            for (int q = 0; q < 4; ++q) {  // q = (dy << 1) | dz
                const float4* r = b4 + 2 * record(ix, iy + (q >> 1), iz + (q & 1));
                const float4 a = __ldg(r), b = __ldg(r + 1);
                c[q] = v3(a.x, a.y, a.z);
                c[4 | q] = v3(b.x, b.y, b.z);
            }
            return 1.0f;
        } else {
            const FieldSoA s{bx, by, bz, d};
            return s.corners(ix, iy, iz, c);
        }
    }
    __device__ __forceinline__ const float* axis(int k) const { return k == 0 ? ax : (k == 1 ? ay : az); }
    // record index of node (ix, iy, iz) in the packed copy (the copy holds
    // fewer than 2^31 nodes)
    __device__ __forceinline__ unsigned record(int ix, int iy, int iz) const {
        return (unsigned)ix + (unsigned)d.nx * ((unsigned)iy + (unsigned)d.ny * (unsigned)iz);
    }
    // one node's (Bx, By, Bz)
    __device__ __forceinline__ float3 node(int ix, int iy, int iz) const {
        if constexpr (M == 1 || M == 2) {
            const float4 v = __ldg(b4 + 2 * (size_t)record(ix, iy, iz));
            return v3(v.x, v.y, v.z);
        } else {
            const int64_t o = ix + (int64_t)d.nx * (iy + (int64_t)d.ny * iz);
            return v3(__ldg(bx + o), __ldg(by + o), __ldg(bz + o));
        }
    }
};
using FieldStretch = FieldStretchT<5>;    // caller's arrays, the reference's search
using FieldStretchU = FieldStretchT<4>;   // caller's arrays, the uniform-spacing formula
using FieldStretchP = FieldStretchT<1>;
using FieldStretchPU = FieldStretchT<2>;
// the search a mode runs: 1 tables, 2 formula, 3 the reference's bisection
template <int M>
constexpr int stretch_search_mode() { return M == 3 ? 1 : (M == 4 ? 2 : (M == 5 ? 3 : M)); }

constexpr int STRETCH_BINS_PER_CELL = 4;
// first table cell of axis k (0, 1, 2) for node counts d
__host__ __device__ __forceinline__ int stretch_cell_offset(const Dims& d, int k) {
    return k == 0 ? 0 : (k == 1 ? d.nx - 1 : d.nx + d.ny - 2);
}

// ---------------------------------------------------------------------------
// Cell location with the reference's face pinning (Interp3dxyzn,
// TraceBlineAdaptive.cu:112-131): a coordinate <= 0 uses cell 0 with fraction
// 0, >= n-1 uses cell n-2 with fraction 1; NaN indexes cell 0.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void locate(float c, int n, int& i, float& r) {
    r = c - floorf(c);
    i = __float2int_rd(c);
    if (c <= 0.f) { r = 0.f; i = 0; }
    if (c >= (float)(n - 1)) { r = 1.f; i = n - 2; }
}

// Fast form of locate(): clamp into [0, top] with top the largest float
// below n-1, so that the truncation is at most n-2 and the fraction the
// remainder (5 instructions per axis instead of 8).  A point on the far face
// samples cell n-2 at a fraction 1 - 2^-24 (n-1) below 1 rather than at 1;
// elsewhere it is locate().  A NaN coordinate lands on cell 0 with fraction 0
// (the line's position is NaN anyway and leaves with flag 42 at the boundary
// test).
__device__ __forceinline__ void locate_fast(float c, int n, int& i, float& r) {
    const float top = __int_as_float(__float_as_int((float)(n - 1)) - 1);
    const float cc = fminf(fmaxf(c, 0.f), top);
    i = __float2int_rz(cc);
    r = cc - (float)i;
}

// exact: reference rounding of the corner weights (double products narrowed
// to float; the bare-fraction products rx*ry are float products).
__device__ __forceinline__ void weights_exact(float rx, float ry, float rz, float w[8]) {
    const double ox = 1.0 - (double)rx, oy = 1.0 - (double)ry, oz = 1.0 - (double)rz;
    w[0] = (float)(ox * oy * oz);
    w[1] = (float)(ox * oy * (double)rz);
    w[2] = (float)(ox * (double)ry * oz);
    w[3] = (float)(ox * (double)ry * (double)rz);
    w[4] = (float)((double)rx * oy * oz);
    w[5] = (float)((double)rx * oy * (double)rz);
    const float rxy = rx * ry;
    w[6] = (float)((double)rxy * oz);
    w[7] = rxy * rz;
}

__device__ __forceinline__ void weights_fast(float rx, float ry, float rz, float w[8]) {
    const float ox = 1.f - rx, oy = 1.f - ry, oz = 1.f - rz;
    const float a0 = ox * oy, a1 = ox * ry, a2 = rx * oy, a3 = rx * ry;
    w[0] = a0 * oz; w[1] = a0 * rz; w[2] = a1 * oz; w[3] = a1 * rz;
    w[4] = a2 * oz; w[5] = a2 * rz; w[6] = a3 * oz; w[7] = a3 * rz;
}

template <bool EXACT>
__device__ __forceinline__ float3 blend(const float3 c[8], const float w[8]) {
    float x = c[0].x * w[0], y = c[0].y * w[0], z = c[0].z * w[0];
#pragma unroll
    for (int q = 1; q < 8; ++q) {
        if (EXACT) {
            x = x + c[q].x * w[q];
            y = y + c[q].y * w[q];
            z = z + c[q].z * w[q];
        } else {
            x = fmaf(c[q].x, w[q], x);
            y = fmaf(c[q].y, w[q], y);
            z = fmaf(c[q].z, w[q], z);
        }
    }
    return v3(x, y, z);
}

// Trilinear B at p; unit = true returns B/|B|.  Reference: Interp3dxyzn,
// TraceBlineAdaptive.cu:95-201.
template <bool EXACT, class F>
__device__ __forceinline__ float3 sample(const F& f, float3 p, bool unit) {
    int ix, iy, iz;
    float rx, ry, rz;
    if (EXACT) {
        locate(p.x, f.d.nx, ix, rx);
        locate(p.y, f.d.ny, iy, ry);
        locate(p.z, f.d.nz, iz, rz);
    } else {
        locate_fast(p.x, f.d.nx, ix, rx);
        locate_fast(p.y, f.d.ny, iy, ry);
        locate_fast(p.z, f.d.nz, iz, rz);
    }
    float w[8];
    if (EXACT) weights_exact(rx, ry, rz, w);
    else weights_fast(rx, ry, rz, w);
    float3 c[8];
    const float s = f.corners(ix, iy, iz, c);
    float3 r = blend<EXACT>(c, w);
    if (unit) {
        if (EXACT) {
            const float nb = sqrtf(r.x * r.x + r.y * r.y + r.z * r.z);
            r = v3(r.x / nb, r.y / nb, r.z / nb);
        } else {
            const float inv = rsqrt_fast(fmaf(r.x, r.x, fmaf(r.y, r.y, r.z * r.z)));
            r = v3(r.x * inv, r.y * inv, r.z * inv);
        }
    } else if (s != 1.0f) {
        r = v3(r.x * s, r.y * s, r.z * s);
    }
    return r;
}

// Fast arithmetic: B/|B| and B at p from one interpolation (the twist kernels
// need both at each step's start point), normalised and scaled as
// sample<false> does with unit = true / false.  Stores without a one-pass
// form take two samples.
template <class F>
__device__ __forceinline__ float3 sample_unit_raw(const F& f, float3 p, float3& raw) {
    raw = sample<false>(f, p, false);
    return sample<false>(f, p, true);
}

template <class F>
__device__ __forceinline__ float3 sample_unit_raw_generic(const F& f, float3 p, float3& raw) {
    int ix, iy, iz;
    float rx, ry, rz;
    locate_fast(p.x, f.d.nx, ix, rx);
    locate_fast(p.y, f.d.ny, iy, ry);
    locate_fast(p.z, f.d.nz, iz, rz);
    float w[8];
    weights_fast(rx, ry, rz, w);
    float3 c[8];
    const float s = f.corners(ix, iy, iz, c);
    const float3 r = blend<false>(c, w);
    raw = s != 1.0f ? v3(r.x * s, r.y * s, r.z * s) : r;
    const float inv = rsqrt_fast(fmaf(r.x, r.x, fmaf(r.y, r.y, r.z * r.z)));
    return v3(r.x * inv, r.y * inv, r.z * inv);
}
template <>
__device__ __forceinline__ float3 sample_unit_raw<FieldSoA>(const FieldSoA& f, float3 p, float3& raw) {
    return sample_unit_raw_generic(f, p, raw);
}
template <>
__device__ __forceinline__ float3 sample_unit_raw<FieldF4>(const FieldF4& f, float3 p, float3& raw) {
    return sample_unit_raw_generic(f, p, raw);
}

// ---------------------------------------------------------------------------
// Fast sampling of the fp16 stores: FP32 interpolation of fp16 node values.
//
// The x-lerp of a corner pair (a, b) is a + r (b - a) in FP32 with the FP32
// fraction r: a widened exactly and b - a rounded once to f32, both by the
// mixed-precision multiply-add (fma.rn.f32.f16 with an f16 one: the product
// is exact, the sum rounded once; it issues on the FMA pipe, where
// cvt.f32.f16 and sub.rn.f32.f16 go to the narrower fp16 pipe, measured
// 0.5 % slower), then one f32 multiply-add, the (Bx, By) pair on the packed
// f32x2 pipe.  The y and z lerps run on packed f32 pairs as well.  Every
// weight and every operation is FP32; only the stored node values are fp16.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void xdiff_h4(uint2 lo, uint2 hi, float2& axy, float& az, float2& dxy, float& dz) {
    // the widening and the difference as mixed-precision multiply-adds by
    // an f16 one (a x 1 + 0 = a exactly; b x 1 - a rounded once = b - a)
    asm("{\n\t"
        ".reg .f16 a0, a1, a2, a3, b0, b1, b2, b3, one;\n\t"
        ".reg .f32 n0, n1, n2;\n\t"
        "mov.b16 one, 0x3C00;\n\t"
        "mov.b32 {a0, a1}, %6;\n\t"
        "mov.b32 {a2, a3}, %7;\n\t"
        "mov.b32 {b0, b1}, %8;\n\t"
        "mov.b32 {b2, b3}, %9;\n\t"
        "fma.rn.f32.f16 %0, a0, one, 0f00000000;\n\t"
        "fma.rn.f32.f16 %1, a1, one, 0f00000000;\n\t"
        "fma.rn.f32.f16 %2, a2, one, 0f00000000;\n\t"
        "neg.f32 n0, %0;\n\t"
        "neg.f32 n1, %1;\n\t"
        "neg.f32 n2, %2;\n\t"
        "fma.rn.f32.f16 %3, b0, one, n0;\n\t"
        "fma.rn.f32.f16 %4, b1, one, n1;\n\t"
        "fma.rn.f32.f16 %5, b2, one, n2;\n\t"
        "}"
        : "=f"(axy.x), "=f"(axy.y), "=f"(az), "=f"(dxy.x), "=f"(dxy.y), "=f"(dz)
        : "r"(lo.x), "r"(lo.y), "r"(hi.x), "r"(hi.y));
}

// a + r (b - a) of one fp16 pair (low half a, high half b) in FP32.
__device__ __forceinline__ float xmix_f32(unsigned pair, float r) {
    float a, d;
    asm("{\n\t"
        ".reg .f16 l, h, one;\n\t"
        ".reg .f32 n;\n\t"
        "mov.b16 one, 0x3C00;\n\t"
        "mov.b32 {l, h}, %2;\n\t"
        "fma.rn.f32.f16 %0, l, one, 0f00000000;\n\t"
        "neg.f32 n, %0;\n\t"
        "fma.rn.f32.f16 %1, h, one, n;\n\t"
        "}"
        : "=f"(a), "=f"(d)
        : "r"(pair));
    return fmaf(d, r, a);
}

// ---------------------------------------------------------------------------
// The fp16-weight sampler of the brick store (opt-in, QSL_ARITH_FAST_W16).
//
// The x-lerp of each corner pair reads the fp16 components directly with the
// mixed-precision multiply-add (fma.rn.f32.f16: the f16 x f16 product is exact
// and the sum is rounded once to f32), with the x weights (1 - r, r) each
// rounded to fp16 (their sum is 1 within 2^-11, which a normalised sample
// does not see): the x fraction is quantised to ~2^-11.  Fewer instructions
// per sample than the FP32 form; its own error figures are stated wherever
// it is measured.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void xlerp_h4(uint2 lo, uint2 hi, unsigned w, float& x, float& y, float& z) {
    asm("{\n\t"
        ".reg .f16 a0, a1, a2, a3, b0, b1, b2, b3, wo, wr;\n\t"
        ".reg .f32 t;\n\t"
        "mov.b32 {a0, a1}, %3;\n\t"
        "mov.b32 {a2, a3}, %4;\n\t"
        "mov.b32 {b0, b1}, %5;\n\t"
        "mov.b32 {b2, b3}, %6;\n\t"
        "mov.b32 {wo, wr}, %7;\n\t"
        "fma.rn.f32.f16 t, a0, wo, 0f00000000;\n\t"
        "fma.rn.f32.f16 %0, b0, wr, t;\n\t"
        "fma.rn.f32.f16 t, a1, wo, 0f00000000;\n\t"
        "fma.rn.f32.f16 %1, b1, wr, t;\n\t"
        "fma.rn.f32.f16 t, a2, wo, 0f00000000;\n\t"
        "fma.rn.f32.f16 %2, b2, wr, t;\n\t"
        "}"
        : "=f"(x), "=f"(y), "=f"(z)
        : "r"(lo.x), "r"(lo.y), "r"(hi.x), "r"(hi.y), "r"(w));
}

// o a + r b (o = 1 - r) for an (x, y) pair on the packed f32 pipe.
__device__ __forceinline__ float2 lerp2(float2 a, float2 b, float o, float r) {
    return __ffma2_rn(b, make_float2(r, r), __fmul2_rn(a, make_float2(o, o)));
}

// The trilinear value at p in brick units (times the brick's scale = B).
// W16 = false: FP32 x-lerps (xdiff_h4); true: fp16 x weights (xlerp_h4).
template <bool W16>
__device__ __forceinline__ float3 h4b_interp(const FieldH4B& f, float3 p, unsigned& brick_out) {
    int ix, iy, iz;
    float rx, ry, rz;
    locate_fast(p.x, f.d.nx, ix, rx);
    locate_fast(p.y, f.d.ny, iy, ry);
    locate_fast(p.z, f.d.nz, iz, rz);
    // the record index, with the z term (the only one that can pass 2^32) in
    // 64 bits
    const unsigned part = (unsigned)ix + 640u * (unsigned)(ix >> 3) + 8u * (unsigned)iy + f.ky * (unsigned)(iy >> 3) +
                          72u * (unsigned)iz;
    const uint4* bp = f.bricks + ((unsigned long long)f.kz * (unsigned)(iz >> 3) + part);
    uint4 u[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) u[q] = __ldg(bp + ((q >> 1) & 1) * 8 + (q & 1) * (8 * BRICK_NODES));
    // e[(dy << 1) | dz]: x-lerped corner pairs
    float2 exy[4];
    float ez[4];
    if constexpr (W16) {
        // the x weights (1 - rx, rx) rounded to fp16 each
        const __half2 wh = __floats2half2_rn(1.f - rx, rx);
        const unsigned w = *reinterpret_cast<const unsigned*>(&wh);
#pragma unroll
        for (int q = 0; q < 4; ++q)
            xlerp_h4(make_uint2(u[q].x, u[q].y), make_uint2(u[q].z, u[q].w), w, exy[q].x, exy[q].y, ez[q]);
    } else {
        float2 az[2], dz[2];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            float2 axy, dxy;
            float a, d;
            xdiff_h4(make_uint2(u[q].x, u[q].y), make_uint2(u[q].z, u[q].w), axy, a, dxy, d);
            exy[q] = __ffma2_rn(dxy, make_float2(rx, rx), axy);
            if (q & 1) { az[q >> 1].y = a; dz[q >> 1].y = d; }
            else { az[q >> 1].x = a; dz[q >> 1].x = d; }
        }
        // the Bz lerps of two corner pairs at a time on the packed pipe
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const float2 e = __ffma2_rn(dz[k], make_float2(rx, rx), az[k]);
            ez[2 * k] = e.x;
            ez[2 * k + 1] = e.y;
        }
    }
    const float oy = 1.f - ry, oz = 1.f - rz;
    const float2 g0 = lerp2(exy[0], exy[2], oy, ry), g1 = lerp2(exy[1], exy[3], oy, ry);
    // the two z-column y-lerps as one packed pair
    const float2 gz = lerp2(make_float2(ez[0], ez[1]), make_float2(ez[2], ez[3]), oy, ry);
    const float2 rxy = lerp2(g0, g1, oz, rz);
    // brick indices fit 32 bits (field stores hold < 1.1e12 nodes, so fewer
    // than 2.2e9 bricks); only the unnormalised samples use it
    brick_out = (unsigned)(ix >> 3) + (unsigned)f.nbx * ((unsigned)(iy >> 3) + (unsigned)f.nby * (unsigned)(iz >> 3));
    return v3(rxy.x, rxy.y, fmaf(gz.y, rz, gz.x * oz));
}

template <bool W16>
__device__ __forceinline__ float3 h4b_sample(const FieldH4B& f, float3 p, bool unit) {
    unsigned brick;
    float3 r = h4b_interp<W16>(f, p, brick);
    if (unit) {
        const float inv = rsqrt_fast(fmaf(r.x, r.x, fmaf(r.y, r.y, r.z * r.z)));
        const float2 xy = __fmul2_rn(make_float2(r.x, r.y), make_float2(inv, inv));
        r = v3(xy.x, xy.y, r.z * inv);
    } else {
        const float s = __ldg(f.scale + brick);
        r = v3(r.x * s, r.y * s, r.z * s);
    }
    return r;
}
template <bool W16>
__device__ __forceinline__ float3 h4b_sample_unit_raw(const FieldH4B& f, float3 p, float3& raw) {
    unsigned brick;
    const float3 r = h4b_interp<W16>(f, p, brick);
    const float s = __ldg(f.scale + brick);
    raw = v3(r.x * s, r.y * s, r.z * s);
    const float inv = rsqrt_fast(fmaf(r.x, r.x, fmaf(r.y, r.y, r.z * r.z)));
    return v3(r.x * inv, r.y * inv, r.z * inv);
}

template <>
__device__ __forceinline__ float3 sample<false, FieldH4B>(const FieldH4B& f, float3 p, bool unit) {
    return h4b_sample<false>(f, p, unit);
}
template <>
__device__ __forceinline__ float3 sample_unit_raw<FieldH4B>(const FieldH4B& f, float3 p, float3& raw) {
    return h4b_sample_unit_raw<false>(f, p, raw);
}
template <>
__device__ __forceinline__ float3 sample<false, FieldH4BW>(const FieldH4BW& f, float3 p, bool unit) {
    return h4b_sample<true>(f, p, unit);
}
template <>
__device__ __forceinline__ float3 sample_unit_raw<FieldH4BW>(const FieldH4BW& f, float3 p, float3& raw) {
    return h4b_sample_unit_raw<true>(f, p, raw);
}

// 32-byte read-only load (one L1 sector); p must be 32-byte aligned.
__device__ __forceinline__ void ldg_v8(const void* p, unsigned (&v)[8]) {
    asm("ld.global.nc.v8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
        : "l"(p));
}

// Fast sample of the cell-record store: the same arithmetic as the fp16
// brick store's fast sample (FP32 x-lerps of the fp16 pairs, packed y/z
// lerps), with Bx/By in one 32-byte load
// (WIDE) or two 16-byte loads, and Bz in one 16-byte load.  The 32-byte load
// is used in code inlined into kernels only: ptxas 13.0 fails (segmentation
// fault) on it inside an out-of-line device function called from several
// kernels of one translation unit.
template <bool WIDE>
__device__ __forceinline__ float3 sample_h8c(const FieldH8C& f, float3 p, bool unit) {
    int ix, iy, iz;
    float rx, ry, rz;
    locate_fast(p.x, f.d.nx, ix, rx);
    locate_fast(p.y, f.d.ny, iy, ry);
    locate_fast(p.z, f.d.nz, iz, rz);
    const uint4* r = f.record(ix, iy, iz);
    uint4 bx, by;
    if (WIDE) {
        unsigned xy[8];
        ldg_v8(r, xy);
        bx = make_uint4(xy[0], xy[1], xy[2], xy[3]);
        by = make_uint4(xy[4], xy[5], xy[6], xy[7]);
    } else {
        bx = __ldg(r);
        by = __ldg(r + 1);
    }
    const uint4 bz = __ldg(r + 2);
    const float2 e0 = make_float2(xmix_f32(bx.x, rx), xmix_f32(by.x, rx)),
                 e1 = make_float2(xmix_f32(bx.y, rx), xmix_f32(by.y, rx)),
                 e2 = make_float2(xmix_f32(bx.z, rx), xmix_f32(by.z, rx)),
                 e3 = make_float2(xmix_f32(bx.w, rx), xmix_f32(by.w, rx));
    const float ez0 = xmix_f32(bz.x, rx), ez1 = xmix_f32(bz.y, rx), ez2 = xmix_f32(bz.z, rx),
                ez3 = xmix_f32(bz.w, rx);
    const float oy = 1.f - ry, oz = 1.f - rz;
    const float2 g0 = lerp2(e0, e2, oy, ry), g1 = lerp2(e1, e3, oy, ry);
    const float gz0 = fmaf(ez2, ry, ez0 * oy), gz1 = fmaf(ez3, ry, ez1 * oy);
    const float2 rxy = lerp2(g0, g1, oz, rz);
    float3 v = v3(rxy.x, rxy.y, fmaf(gz1, rz, gz0 * oz));
    if (unit) {
        const float inv = rsqrt_fast(fmaf(v.x, v.x, fmaf(v.y, v.y, v.z * v.z)));
        v = v3(v.x * inv, v.y * inv, v.z * inv);
    } else {
        const float s = __ldg(reinterpret_cast<const float*>(r + 3));
        v = v3(v.x * s, v.y * s, v.z * s);
    }
    return v;
}

template <>
__device__ __forceinline__ float3 sample<false, FieldH8C>(const FieldH8C& f, float3 p, bool unit) {
    return sample_h8c<true>(f, p, unit);
}

// sample() for out-of-line device functions (see sample_h8c).
template <bool EXACT, class F>
__device__ __forceinline__ float3 sample_outlined(const F& f, float3 p, bool unit) {
    return sample<EXACT>(f, p, unit);
}
template <>
__device__ __forceinline__ float3 sample_outlined<false, FieldH8C>(const FieldH8C& f, float3 p, bool unit) {
    return sample_h8c<false>(f, p, unit);
}

// ---------------------------------------------------------------------------
// Stretched grid (fastqslpy/cu/TraceBlineAdaptiveStretch.cu)
// ---------------------------------------------------------------------------
// The reference's search (GetIndexBiSearch, :42-64): halve [i0, i1] while it
// spans more than 3 nodes, then mid or mid - 1 on one comparison.  For a point
// in the upper part of the last interval this is the cell below the point's
// (the fraction then exceeds 1 and the sample extrapolates); kept as is so the
// results are the reference's.  The result lies in [0, n-2] for n >= 2.
__device__ __forceinline__ int stretch_bisect(float c, int n, const float* __restrict__ a) {
    int i0 = 0, i1 = n - 1, mid = n / 2;
    while (i1 - i0 > 3) {
        if (c > __ldg(a + mid)) i0 = mid;
        else i1 = mid;
        mid = (i0 + i1) / 2;
    }
    int r = (c > __ldg(a + mid)) ? mid : mid - 1;
    r = r > n - 2 ? n - 2 : r;
    return r < 0 ? 0 : r;
}

// The uniform-spacing formula (GetIndexUniStretch, :67-74); its spacing du is
// (a[n-1] - a[0]) / n, the node count, as in the reference (formed once per
// kernel, the same float).
__device__ __forceinline__ int stretch_uni(float c, int n, float a0, float du) {
    int r = __float2int_rd((c - a0) / du);
    r = r < 0 ? 0 : r;
    return r > n - 2 ? n - 2 : r;
}
// Fast form: the quotient as a product with inv = 1 / du (formed once per
// kernel); it can differ from the divide's only where (c - a0) / du lies
// within an ulp or two of an integer, which moves the formula's switch point
// between two cells by that much.
__device__ __forceinline__ int stretch_uni_fast(float c, int n, float a0, float inv) {
    int r = __float2int_rd((c - a0) * inv);
    r = r < 0 ? 0 : r;
    return r > n - 2 ? n - 2 : r;
}

// The reference search's cell for c through the tables of a packed store
// (FieldStretchP): srec[j] is the cell the reference's search returns for
// every coordinate of the interval (a[j], a[j+1]] (its comparisons are all
// of the form c > a[m]), with that cell's first coordinate and width.  The
// bin of c covers the intervals c can lie in: when they are one or two the
// bin holds both records and the node between them (two independent loads,
// c > node picks the upper one), else their range, bisected to the interval
// j with a[j] < c <= a[j+1] (or the range's low end) before srec[j] is
// read.  The same cell, coordinate and width as stretch_bisect followed by
// the two coordinate loads, for c clamped as stretch_locate clamps it.
// WIDE: the bin's two records as one 32-byte load (sbin is 32-byte aligned).
template <int M, bool WIDE>
__device__ __forceinline__ int stretch_table(const FieldStretchT<M>& f, int k, float c, float a0, float binv,
                                             float& ai, float& di) {
    const float* a = f.axis(k);
    const int n = f.d.n(k);
    const int c0 = stretch_cell_offset(f.d, k);
    const int nb = STRETCH_BINS_PER_CELL * (n - 1);
    int b = __float2int_rz((c - a0) * binv);
    b = b < 0 ? 0 : (b > nb - 1 ? nb - 1 : b);
    const float4* sb = f.sbin + 2 * (STRETCH_BINS_PER_CELL * c0 + b);
    float4 A, B;
    if constexpr (WIDE) {
        unsigned w[8];
        ldg_v8(sb, w);
        A = make_float4(__uint_as_float(w[0]), __uint_as_float(w[1]), __uint_as_float(w[2]), __uint_as_float(w[3]));
        B = make_float4(__uint_as_float(w[4]), __uint_as_float(w[5]), __uint_as_float(w[6]), __uint_as_float(w[7]));
    } else {
        A = __ldg(sb);
        B = __ldg(sb + 1);
    }
    if (__float_as_int(B.w) == 0) {
        // one or two intervals: the records of both and the node between
        const bool up = c > A.x;
        ai = up ? B.x : A.y;
        di = up ? B.y : A.z;
        return up ? __float_as_int(B.z) : __float_as_int(A.w);
    }
    int lo = __float_as_int(A.y), hi = __float_as_int(A.z);
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (c > __ldg(a + mid)) lo = mid;
        else hi = mid - 1;
    }
    const float4 rec = __ldg(f.srec + c0 + lo);
    ai = rec.x;
    di = rec.y;
    return __float_as_int(rec.z);
}

// Cell and fraction along one axis: c clamped to (a[0] + 1e-6, a[n-1] - 1e-6)
// (offsets applied in double and narrowed, once per kernel: clo, chi), then
// the index and r = (c - a[i]) / (a[i+1] - a[i])  (Interp3dxyzn, :100-122);
// the fast arithmetic divides with the hardware reciprocal (div_fast).
template <bool EXACT, bool WIDE, int M>
__device__ __forceinline__ void stretch_locate(const FieldStretchT<M>& f, int k, float c, float a0, float an,
                                               float clo, float chi, float du, float binv, int& i, float& r) {
    const float* a = f.axis(k);
    const int n = f.d.n(k);
    c = (c > a0) ? c : clo;
    c = (c < an) ? c : chi;
    float ai, di;
    if constexpr (stretch_search_mode<M>() == 1) {
        i = stretch_table<M, WIDE>(f, k, c, a0, binv, ai, di);
    } else {
        if constexpr (stretch_search_mode<M>() == 2)
            i = EXACT ? stretch_uni(c, n, a0, du) : stretch_uni_fast(c, n, a0, binv);
        else i = stretch_bisect(c, n, a);
        ai = __ldg(a + i);
        di = __ldg(a + i + 1) - ai;
    }
    r = EXACT ? (c - ai) / di : div_fast(__fsub_rn(c, ai), di);
}

// WIDE: the packed stores' 32-byte x-pair records and search bins as one
// 32-byte load each (code inlined into kernels only; see sample_h8c) or two
// 16-byte loads.
template <bool EXACT, int M, bool WIDE = true>
__device__ __forceinline__ float3 sample_stretch(const FieldStretchT<M>& f, float3 p, bool unit) {
    int ix, iy, iz;
    float rx, ry, rz;
    stretch_locate<EXACT, WIDE>(f, 0, p.x, f.lo.x, f.hi.x, f.clo.x, f.chi.x, f.us.x, f.sbinv.x, ix, rx);
    stretch_locate<EXACT, WIDE>(f, 1, p.y, f.lo.y, f.hi.y, f.clo.y, f.chi.y, f.us.y, f.sbinv.y, iy, ry);
    stretch_locate<EXACT, WIDE>(f, 2, p.z, f.lo.z, f.hi.z, f.clo.z, f.chi.z, f.us.z, f.sbinv.z, iz, rz);
    float3 r;
    if constexpr (EXACT) {
        float w[8];
        weights_exact(rx, ry, rz, w);
        float3 c[8];
        f.corners(ix, iy, iz, c);
        r = blend<true>(c, w);
    } else {
        // fast arithmetic: x-lerps of the four corner pairs as each pair is
        // loaded, then y, then z, so that at most a pair of corners is live
        // (the eight corners and weights of a one-shot blend held the
        // kernel's register count near 170); (Bx, By) on the packed pipe
        const float ox = 1.f - rx, oy = 1.f - ry, oz = 1.f - rz;
        float2 exy[4];
        float ez[4];
        // packed stores: the four x-pair records of the stencil, at record
        // indices o, o + nx ny (dz), o + nx (dy), o + nx + nx ny
        const unsigned o0 = (M == 1 || M == 2) ? f.record(ix, iy, iz) : 0u;
        const unsigned sy = (unsigned)f.d.nx, sz = (unsigned)f.d.nx * (unsigned)f.d.ny;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            float3 a, b;
            if constexpr (M == 1 || M == 2) {
                const float4* r = f.b4 + 2 * (size_t)(o0 + ((q >> 1) & 1) * sy + (q & 1) * sz);
                if constexpr (WIDE) {
                    unsigned w[8];
                    ldg_v8(r, w);
                    a = v3(__uint_as_float(w[0]), __uint_as_float(w[1]), __uint_as_float(w[2]));
                    b = v3(__uint_as_float(w[4]), __uint_as_float(w[5]), __uint_as_float(w[6]));
                } else {
                    const float4 ra = __ldg(r), rb = __ldg(r + 1);
                    a = v3(ra.x, ra.y, ra.z);
                    b = v3(rb.x, rb.y, rb.z);
                }
            } else {
                a = f.node(ix, iy + (q >> 1), iz + (q & 1));
                b = f.node(ix + 1, iy + (q >> 1), iz + (q & 1));
            }
            exy[q] = __ffma2_rn(make_float2(b.x, b.y), make_float2(rx, rx),
                                __fmul2_rn(make_float2(a.x, a.y), make_float2(ox, ox)));
            ez[q] = fmaf(b.z, rx, a.z * ox);
        }
        const float2 g0 = __ffma2_rn(exy[2], make_float2(ry, ry), __fmul2_rn(exy[0], make_float2(oy, oy)));
        const float2 g1 = __ffma2_rn(exy[3], make_float2(ry, ry), __fmul2_rn(exy[1], make_float2(oy, oy)));
        const float gz0 = fmaf(ez[2], ry, ez[0] * oy), gz1 = fmaf(ez[3], ry, ez[1] * oy);
        const float2 rxy = __ffma2_rn(g1, make_float2(rz, rz), __fmul2_rn(g0, make_float2(oz, oz)));
        r = v3(rxy.x, rxy.y, fmaf(gz1, rz, gz0 * oz));
    }
    if (unit) {
        if (EXACT) {
            const float nb = sqrtf(r.x * r.x + r.y * r.y + r.z * r.z);
            r = v3(r.x / nb, r.y / nb, r.z / nb);
        } else {
            const float inv = rsqrt_fast(fmaf(r.x, r.x, fmaf(r.y, r.y, r.z * r.z)));
            r = v3(r.x * inv, r.y * inv, r.z * inv);
        }
    }
    return r;
}

template <>
__device__ __forceinline__ float3 sample<true, FieldStretch>(const FieldStretch& f, float3 p, bool unit) {
    return sample_stretch<true>(f, p, unit);
}
template <>
__device__ __forceinline__ float3 sample<true, FieldStretchU>(const FieldStretchU& f, float3 p, bool unit) {
    return sample_stretch<true>(f, p, unit);
}
template <>
__device__ __forceinline__ float3 sample<false, FieldStretch>(const FieldStretch& f, float3 p, bool unit) {
    return sample_stretch<false>(f, p, unit);
}
template <>
__device__ __forceinline__ float3 sample<false, FieldStretchP>(const FieldStretchP& f, float3 p, bool unit) {
    return sample_stretch<false>(f, p, unit);
}
template <>
__device__ __forceinline__ float3 sample<false, FieldStretchPU>(const FieldStretchPU& f, float3 p, bool unit) {
    return sample_stretch<false>(f, p, unit);
}
// out-of-line callers (the boundary RK4 leg) load the records as two
// 16-byte halves
template <>
__device__ __forceinline__ float3 sample_outlined<false, FieldStretchP>(const FieldStretchP& f, float3 p, bool unit) {
    return sample_stretch<false, 1, false>(f, p, unit);
}
template <>
__device__ __forceinline__ float3 sample_outlined<false, FieldStretchPU>(const FieldStretchPU& f, float3 p,
                                                                         bool unit) {
    return sample_stretch<false, 2, false>(f, p, unit);
}
template <>
__device__ __forceinline__ float3 sample<false, FieldStretchT<3>>(const FieldStretchT<3>& f, float3 p, bool unit) {
    return sample_stretch<false>(f, p, unit);
}
template <>
__device__ __forceinline__ float3 sample<false, FieldStretchT<4>>(const FieldStretchT<4>& f, float3 p, bool unit) {
    return sample_stretch<false>(f, p, unit);
}

// Position clamped into [1e-4, n-1-1e-4] as the scalar interpolator of the
// reference does (Interp3d, TraceBlineAdaptive.cu:57-62).
__device__ __forceinline__ float clamp_inside(float c, int n) {
    c = (c > 0.f) ? c : (float)0.0001;
    c = (c < (float)(n - 1)) ? c : (float)((double)((float)n - 1.f) - 0.0001);
    return c;
}

// Exact scalar interpolation of one component (Interp3d, :47-93): each term is
// corner*f1*f2*f3 evaluated left to right, bare float fractions staying float
// products until a double factor appears, summed in double.
__device__ __forceinline__ float sample_scalar_exact(const FieldSoA& f, int m, float x, float y, float z) {
    x = clamp_inside(x, f.d.nx);
    y = clamp_inside(y, f.d.ny);
    z = clamp_inside(z, f.d.nz);
    const float rx = x - floorf(x), ry = y - floorf(y), rz = z - floorf(z);
    const int ix = __float2int_rd(x), iy = __float2int_rd(y), iz = __float2int_rd(z);
    const double ox = 1.0 - (double)rx, oy = 1.0 - (double)ry, oz = 1.0 - (double)rz;
    const int64_t sy = f.d.nx, sz = (int64_t)f.d.nx * f.d.ny;
    const int64_t b = ix + sy * iy + sz * iz;
    float a[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) a[q] = f.scalar(m, b + ((q >> 2) & 1) + ((q >> 1) & 1) * sy + (q & 1) * sz);
    double s = (double)a[0] * ox * oy * oz;
    s = s + (double)a[1] * ox * oy * (double)rz;
    s = s + (double)a[2] * ox * (double)ry * oz;
    s = s + (double)a[3] * ox * (double)ry * (double)rz;
    s = s + (double)(a[4] * rx) * oy * oz;
    s = s + (double)(a[5] * rx) * oy * (double)rz;
    s = s + (double)((a[6] * rx) * ry) * oz;
    s = s + (double)(((a[7] * rx) * ry) * rz);
    return (float)s;
}

// B (all three components) at a clamped position; exact mode evaluates each
// component like the reference's scalar interpolator, fast mode takes one
// vector sample at the clamped point.
template <bool EXACT, class F>
__device__ __forceinline__ float3 sample_endpoint(const F& f, float3 p);

template <>
__device__ __forceinline__ float3 sample_endpoint<true, FieldSoA>(const FieldSoA& f, float3 p) {
    return v3(sample_scalar_exact(f, 0, p.x, p.y, p.z), sample_scalar_exact(f, 1, p.x, p.y, p.z),
              sample_scalar_exact(f, 2, p.x, p.y, p.z));
}

template <bool EXACT, class F>
__device__ __forceinline__ float3 sample_endpoint(const F& f, float3 p) {
    const float3 q = v3(clamp_inside(p.x, f.d.nx), clamp_inside(p.y, f.d.ny), clamp_inside(p.z, f.d.nz));
    return sample<false>(f, q, false);
}

// Stretched grid: the vector interpolator (its clamp included), as the
// reference's stretched kernel samples its endpoints (:466-499).
template <>
__device__ __forceinline__ float3 sample_endpoint<true, FieldStretch>(const FieldStretch& f, float3 p) {
    return sample_stretch<true>(f, p, false);
}
template <>
__device__ __forceinline__ float3 sample_endpoint<false, FieldStretch>(const FieldStretch& f, float3 p) {
    return sample_stretch<false>(f, p, false);
}
template <>
__device__ __forceinline__ float3 sample_endpoint<true, FieldStretchU>(const FieldStretchU& f, float3 p) {
    return sample_stretch<true>(f, p, false);
}
template <>
__device__ __forceinline__ float3 sample_endpoint<false, FieldStretchU>(const FieldStretchU& f, float3 p) {
    return sample_stretch<false>(f, p, false);
}
template <>
__device__ __forceinline__ float3 sample_endpoint<false, FieldStretchP>(const FieldStretchP& f, float3 p) {
    return sample_stretch<false>(f, p, false);
}
template <>
__device__ __forceinline__ float3 sample_endpoint<false, FieldStretchPU>(const FieldStretchPU& f, float3 p) {
    return sample_stretch<false>(f, p, false);
}

}  // namespace qsl
