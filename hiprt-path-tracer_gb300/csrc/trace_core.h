// Traversal core of the 8-wide compressed BVH, shared by the CUDA kernels (trace.cu) and the
// host-compiled test harness that checks the builder and traversal logic on machines without a GPU
// (tests/native/traverse_emu.cpp). Under nvcc it compiles to device code; under a host compiler the
// rounding intrinsics map to plain IEEE float operations (the host build uses -ffp-contract=off).
//
// Replaces hiprtGeomTraversalClosest / hiprtGeomTraversalAnyHit and the filter function of the
// reference (src/Device/includes/Intersect.h:22-69,200-324, src/Device/functions/FilterFunction.h:
// 22-75; GB300 has no RT cores, so traversal is software). Traversal order follows Ylitie et al.
// (HPG 2017): node groups (child base + 8 hit bits + internal-child mask) on a per-thread stack,
// children visited nearest-first through the octant slot order, triangle hits from a 24-bit mask.
//
// Two triangle tests (template parameter TRI):
//  - kTriMollerTrumbore, the parity mode: the reference's Moller-Trumbore
//    (src/Renderer/Triangle.h:20-63) written with explicitly rounded operations
//    (__fmul_rn/__fadd_rn/__fsub_rn/__fdiv_rn), which the compiler never contracts into FMAs, so
//    t/u/v match the reference's CPU results bit for bit. It is not watertight: a ray through an
//    edge shared by two triangles can miss both (or hit both) by a rounding.
//  - kTriWatertight, the production mode: Woop, Benthin and Wald, "Watertight Ray/Triangle
//    Intersection" (JCGT 2013): the vertices are moved into a ray-aligned space by a shear that
//    depends on the ray only, and the three edge functions are evaluated there; a shared edge
//    gives the two triangles edge functions of exactly opposite sign (rounded products and
//    differences are antisymmetric), so no ray passes between them; exactly zero edge functions
//    are evaluated again in double. Barycentrics are returned as u = weight of b, v = weight of c,
//    as Moller-Trumbore defines them.
// Box tests only
// prune, so their rounding cannot change a result as long as they stay conservative: each node
// widens its children's slab intervals by an absolute slack that bounds every rounding of the test
// (derivation at intersect_children).
#pragma once

#include <stddef.h>
#include <stdint.h>

#include "bvh.h"

#ifdef __CUDACC__
#include <cuda_runtime.h>
#define GBPT_HD __device__ __forceinline__
#define GBPT_LDG(p) __ldg(p)
#else
#include <cmath>
#include <cstring>
#define GBPT_HD inline
#define GBPT_LDG(p) (*(p))
struct uint2 { uint32_t x, y; };
struct uint4 { uint32_t x, y, z, w; };
struct float4 { float x, y, z, w; };
inline uint2 make_uint2(uint32_t x, uint32_t y) { return uint2{x, y}; }
inline float4 make_float4(float x, float y, float z, float w) { return float4{x, y, z, w}; }
inline float __fmul_rn(float a, float b) { return a * b; }
inline float __fadd_rn(float a, float b) { return a + b; }
inline float __fsub_rn(float a, float b) { return a - b; }
inline float __fdiv_rn(float a, float b) { return a / b; }
inline float __frcp_rn(float a) { return 1.0f / a; }
inline double __dmul_rn(double a, double b) { return a * b; }
inline double __dsub_rn(double a, double b) { return a - b; }
inline float __uint_as_float(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
inline float __int_as_float(int32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
inline int32_t __float_as_int(float f) { int32_t u; std::memcpy(&u, &f, 4); return u; }
inline uint32_t __clz(uint32_t x) { return x ? (uint32_t)__builtin_clz(x) : 32u; }
inline uint32_t __popc(uint32_t x) { return (uint32_t)__builtin_popcount(x); }
inline uint32_t __byte_perm(uint32_t x, uint32_t y, uint32_t s)
{
    const uint64_t v = ((uint64_t)y << 32) | x;
    uint32_t r = 0;
    for (int i = 0; i < 4; i++) r |= (uint32_t)((v >> (8 * ((s >> (4 * i)) & 7u))) & 0xFFu) << (8 * i);
    return r;
}
inline int __ffs(uint32_t x) { return __builtin_ffs((int)x); }
using ::copysignf;
using ::fabsf;
using ::fmaf;
using ::fmaxf;
using ::fminf;
#endif

namespace gbpt {
namespace core {

constexpr float kMtEps = 0.0000001f;     // EPSILON of src/Renderer/Triangle.h:24

GBPT_HD float dot_rn(float ax, float ay, float az, float bx, float by, float bz)
{
    return __fadd_rn(__fadd_rn(__fmul_rn(ax, bx), __fmul_rn(ay, by)), __fmul_rn(az, bz));
}

GBPT_HD void cross_rn(float ax, float ay, float az, float bx, float by, float bz, float& cx, float& cy,
                                         float& cz)
{
    cx = __fsub_rn(__fmul_rn(ay, bz), __fmul_rn(az, by));
    cy = __fsub_rn(__fmul_rn(az, bx), __fmul_rn(ax, bz));
    cz = __fsub_rn(__fmul_rn(ax, by), __fmul_rn(ay, bx));
}

constexpr int kTriMollerTrumbore = 0;
constexpr int kTriWatertight = 1;

// Moller-Trumbore in the reference's operation order, from the vertices a, b, c (edges formed
// here as the reference forms them). Returns true with t/u/v on a hit.
GBPT_HD bool mt_test(const float4 a, const float4 b, const float4 c, float ox, float oy, float oz,
                                        float dx, float dy, float dz, float& t, float& u, float& v)
{
    const float4 e1 = make_float4(__fsub_rn(b.x, a.x), __fsub_rn(b.y, a.y), __fsub_rn(b.z, a.z), 0.0f);
    const float4 e2 = make_float4(__fsub_rn(c.x, a.x), __fsub_rn(c.y, a.y), __fsub_rn(c.z, a.z), 0.0f);
    float hx, hy, hz;
    cross_rn(dx, dy, dz, e2.x, e2.y, e2.z, hx, hy, hz);
    const float det = dot_rn(e1.x, e1.y, e1.z, hx, hy, hz);
    if (det > -kMtEps && det < kMtEps) return false;
    const float f = __fdiv_rn(1.0f, det);
    const float sx = __fsub_rn(ox, a.x), sy = __fsub_rn(oy, a.y), sz = __fsub_rn(oz, a.z);
    u = __fmul_rn(f, dot_rn(sx, sy, sz, hx, hy, hz));
    if (u < 0.0f || u > 1.0f) return false;
    float qx, qy, qz;
    cross_rn(sx, sy, sz, e1.x, e1.y, e1.z, qx, qy, qz);
    v = __fmul_rn(f, dot_rn(dx, dy, dz, qx, qy, qz));
    if (v < 0.0f || __fadd_rn(u, v) > 1.0f) return false;
    t = __fmul_rn(f, dot_rn(e2.x, e2.y, e2.z, qx, qy, qz));
    return t > kMtEps;
}

// The per-ray shear of the watertight test: kz the axis of the direction's largest magnitude, kx
// and ky the two others (swapped when d[kz] < 0, which keeps the edge functions' winding), and
// the shear constants sx = d[kx] / d[kz], sy = d[ky] / d[kz], sz = 1 / d[kz].
struct WatertightRay
{
    int kx, ky, kz;
    float sx, sy, sz;
};

GBPT_HD float axis_of(float x, float y, float z, int k) { return k == 0 ? x : (k == 1 ? y : z); }

GBPT_HD WatertightRay watertight_ray(float dx, float dy, float dz)
{
    const float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
    WatertightRay r;
    r.kz = (ax >= ay && ax >= az) ? 0 : (ay >= az ? 1 : 2);
    r.kx = r.kz == 2 ? 0 : r.kz + 1;
    r.ky = r.kx == 2 ? 0 : r.kx + 1;
    const float dkz = axis_of(dx, dy, dz, r.kz);
    if (dkz < 0.0f)
    {
        const int k = r.kx;
        r.kx = r.ky;
        r.ky = k;
    }
    r.sx = __fdiv_rn(axis_of(dx, dy, dz, r.kx), dkz);
    r.sy = __fdiv_rn(axis_of(dx, dy, dz, r.ky), dkz);
    r.sz = __fdiv_rn(1.0f, dkz);
    return r;
}

// Watertight ray/triangle test (Woop et al. 2013, algorithm of section 3, no backface culling).
// Returns true with t (> 1e-7, the parity mode's minimum), u, v on a hit.
GBPT_HD bool wt_test(const WatertightRay& w, const float4 a, const float4 b, const float4 c, float ox, float oy,
                     float oz, float& t, float& u, float& v)
{
    const float Ax = __fsub_rn(axis_of(a.x, a.y, a.z, w.kx), axis_of(ox, oy, oz, w.kx));
    const float Ay = __fsub_rn(axis_of(a.x, a.y, a.z, w.ky), axis_of(ox, oy, oz, w.ky));
    const float Az = __fsub_rn(axis_of(a.x, a.y, a.z, w.kz), axis_of(ox, oy, oz, w.kz));
    const float Bx = __fsub_rn(axis_of(b.x, b.y, b.z, w.kx), axis_of(ox, oy, oz, w.kx));
    const float By = __fsub_rn(axis_of(b.x, b.y, b.z, w.ky), axis_of(ox, oy, oz, w.ky));
    const float Bz = __fsub_rn(axis_of(b.x, b.y, b.z, w.kz), axis_of(ox, oy, oz, w.kz));
    const float Cx = __fsub_rn(axis_of(c.x, c.y, c.z, w.kx), axis_of(ox, oy, oz, w.kx));
    const float Cy = __fsub_rn(axis_of(c.x, c.y, c.z, w.ky), axis_of(ox, oy, oz, w.ky));
    const float Cz = __fsub_rn(axis_of(c.x, c.y, c.z, w.kz), axis_of(ox, oy, oz, w.kz));
    // shear into ray space
    const float ax = __fsub_rn(Ax, __fmul_rn(w.sx, Az)), ay = __fsub_rn(Ay, __fmul_rn(w.sy, Az));
    const float bx = __fsub_rn(Bx, __fmul_rn(w.sx, Bz)), by = __fsub_rn(By, __fmul_rn(w.sy, Bz));
    const float cx = __fsub_rn(Cx, __fmul_rn(w.sx, Cz)), cy = __fsub_rn(Cy, __fmul_rn(w.sy, Cz));
    // edge functions: U for edge (b, c), V for (c, a), W for (a, b)
    float U = __fsub_rn(__fmul_rn(cx, by), __fmul_rn(cy, bx));
    float V = __fsub_rn(__fmul_rn(ax, cy), __fmul_rn(ay, cx));
    float W = __fsub_rn(__fmul_rn(bx, ay), __fmul_rn(by, ax));
    if (U == 0.0f || V == 0.0f || W == 0.0f)
    {
        U = (float)__dsub_rn(__dmul_rn((double)cx, (double)by), __dmul_rn((double)cy, (double)bx));
        V = (float)__dsub_rn(__dmul_rn((double)ax, (double)cy), __dmul_rn((double)ay, (double)cx));
        W = (float)__dsub_rn(__dmul_rn((double)bx, (double)ay), __dmul_rn((double)by, (double)ax));
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = __fadd_rn(__fadd_rn(U, V), W);
    if (det == 0.0f) return false;
    const float az = __fmul_rn(w.sz, Az), bz = __fmul_rn(w.sz, Bz), cz = __fmul_rn(w.sz, Cz);
    const float T = __fadd_rn(__fadd_rn(__fmul_rn(U, az), __fmul_rn(V, bz)), __fmul_rn(W, cz));
    // t = T / det must be positive: T and det of the same sign
    if ((__float_as_int(T) ^ __float_as_int(det)) < 0) return false;
    const float rcp = __fdiv_rn(1.0f, det);
    t = __fmul_rn(T, rcp);
    u = __fmul_rn(V, rcp);
    v = __fmul_rn(W, rcp);
    return t > kMtEps;
}

// The triangle test of mode TRI (w is only read by the watertight test)
template <int TRI>
GBPT_HD bool tri_test(const WatertightRay& w, const float4 a, const float4 b, const float4 c, float ox, float oy,
                      float oz, float dx, float dy, float dz, float& t, float& u, float& v)
{
    if constexpr (TRI == kTriWatertight)
        return wt_test(w, a, b, c, ox, oy, oz, t, u, v);
    else
        return mt_test(a, b, c, ox, oy, oz, dx, dy, dz, t, u, v);
}

GBPT_HD float safe_rcp(float d)
{
    const float tiny = 1e-20f;
    return __frcp_rn(fabsf(d) < tiny ? copysignf(tiny, d) : d);
}

// Quantised plane q (byte k of word w) as the float 2^23 + 256 q, built by one byte permute
GBPT_HD float plane_magic(uint32_t w, int k)
{
    return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7404u | ((uint32_t)k << 4)));
}

GBPT_HD uint32_t byte_of(uint32_t w, int k) { return (w >> (8 * k)) & 0xFFu; }

// Per-axis slab constants of a node: a child plane q on this axis is entered at
// t = fma(2^23 + 256 q, s8, base), with s8 = 2^(e-127) id / 256 (exact: power-of-two scalings)
// and base = (p - o) id - 2^15 * 2^(e-127) id, so that t = q 2^(e-127) id + (p - o) id.
// Rounding: (p - o), the product with id (itself a rounded reciprocal), base and the final FMA
// each err by at most one half ulp of a value bounded by |a| + 2^15 |s| + 255 |s| (a = (p - o) id,
// s = 2^(e-127) id), i.e. in total below 8 (|a| + 2^16 |s|) 2^-24. The slack
// eps = (|a| + 2^16 |s|) 2^-20 is twice that: subtracted from the near planes' base and added to
// the far planes' (those two roundings are covered by the same margin), it keeps the test
// conservative for every child.
struct AxisSlab
{
    float s8, near_base, far_base;
};

GBPT_HD AxisSlab axis_slab(float p, float o, uint32_t e, float id)
{
    const float s = __uint_as_float(e << 23) * id;
    const float a = (p - o) * id;
    const float base = fmaf(-32768.0f, s, a);
    const float eps = (fabsf(a) + 65536.0f * fabsf(s)) * (1.0f / 1048576.0f);
    AxisSlab r;
    r.s8 = s * (1.0f / 256.0f);
    r.near_base = base - eps;
    r.far_base = base + eps;
    return r;
}

// Intersects the 8 children of one node; returns the hit mask (bits 24-31: internal children by
// octant-ordered slot, bits 0-23: triangles relative to the node's triangle base).
GBPT_HD uint32_t intersect_children(const uint4 w0, const uint4 w1, const uint4 w2, const uint4 w3,
                                                       const uint4 w4, float ox, float oy, float oz, float idx,
                                                       float idy, float idz, float tmin, float tmax, uint32_t oct_inv)
{
    const AxisSlab X = axis_slab(__uint_as_float(w0.x), ox, w0.w & 0xFFu, idx);
    const AxisSlab Y = axis_slab(__uint_as_float(w0.y), oy, (w0.w >> 8) & 0xFFu, idy);
    const AxisSlab Z = axis_slab(__uint_as_float(w0.z), oz, (w0.w >> 16) & 0xFFu, idz);

    // near/far planes per axis by ray sign: words hold 4 children's bytes each
    uint32_t nx0 = w2.x, nx1 = w2.y, fx0 = w3.z, fx1 = w3.w;
    uint32_t ny0 = w2.z, ny1 = w2.w, fy0 = w4.x, fy1 = w4.y;
    uint32_t nz0 = w3.x, nz1 = w3.y, fz0 = w4.z, fz1 = w4.w;
    if (idx < 0.0f) { uint32_t t0 = nx0, t1 = nx1; nx0 = fx0; nx1 = fx1; fx0 = t0; fx1 = t1; }
    if (idy < 0.0f) { uint32_t t0 = ny0, t1 = ny1; ny0 = fy0; ny1 = fy1; fy0 = t0; fy1 = t1; }
    if (idz < 0.0f) { uint32_t t0 = nz0, t1 = nz1; nz0 = fz0; nz1 = fz1; fz0 = t0; fz1 = t1; }

    // child meta bytes decoded four at a time: a child is internal when bits 3 and 4 are both set;
    // its hit-mask bit index is meta & 31, xor-ed with the ray octant for internal children; its
    // bits are meta >> 5 (the internal flag, or the unary triangle count)
    uint32_t bidx[2], cbits[2];
#pragma unroll
    for (int h = 0; h < 2; h++)
    {
        const uint32_t m = h == 0 ? w1.z : w1.w;
        const uint32_t inner = (m & (m << 1) & 0x10101010u) >> 4;  // 1 per internal child's byte
        bidx[h] = (m & 0x1F1F1F1Fu) ^ (inner * oct_inv);         // oct_inv <= 7: no carries
        cbits[h] = (m >> 5) & 0x07070707u;
    }

    uint32_t hitmask = 0;
#pragma unroll
    for (int i = 0; i < 8; i++)
    {
        const int k = i & 3;
        const float tx0 = fmaf(plane_magic(i < 4 ? nx0 : nx1, k), X.s8, X.near_base);
        const float tx1 = fmaf(plane_magic(i < 4 ? fx0 : fx1, k), X.s8, X.far_base);
        const float ty0 = fmaf(plane_magic(i < 4 ? ny0 : ny1, k), Y.s8, Y.near_base);
        const float ty1 = fmaf(plane_magic(i < 4 ? fy0 : fy1, k), Y.s8, Y.far_base);
        const float tz0 = fmaf(plane_magic(i < 4 ? nz0 : nz1, k), Z.s8, Z.near_base);
        const float tz1 = fmaf(plane_magic(i < 4 ? fz0 : fz1, k), Z.s8, Z.far_base);
        const float t_enter = fmaxf(fmaxf(tx0, ty0), fmaxf(tz0, tmin));
        const float t_exit = fminf(fminf(tx1, ty1), fminf(tz1, tmax));
        const uint32_t bit_index = byte_of(bidx[i >> 2], k);
        const uint32_t child_bits = byte_of(cbits[i >> 2], k);
        if (t_enter <= t_exit) hitmask |= child_bits << bit_index;
    }
    return hitmask;
}

// A thread's traversal stack: its first SH entries in shared memory (a column of the block's
// array, entry k at col[k * stride] with stride = threads per block, so the 32 lanes of a warp
// touch 32 different bank pairs whatever their depths), the deeper ones in local memory. An
// 8-wide BVH rarely holds more than a handful of entries, so with SH >= 4 nearly every push and
// pop stays in shared memory instead of going through L1 as local-memory traffic.
template <int SH>
struct TraversalStack
{
    uint2 local[kTraversalStack - SH];
    // col / stride stay in the caller's registers (members here would live in local memory)
    GBPT_HD void push(int& sp, uint2 v, uint2* col, int stride)
    {
        if constexpr (SH > 0)
        {
            if (sp < SH)
            {
                col[sp * stride] = v;
                ++sp;
                return;
            }
        }
        local[sp - SH] = v;
        ++sp;
    }
    GBPT_HD uint2 pop(int& sp, const uint2* col, int stride)
    {
        --sp;
        if constexpr (SH > 0)
        {
            if (sp < SH) return col[sp * stride];
        }
        return local[sp - SH];
    }
};

// Traces one ray. Closest hit: returns the hit as (t, u, v, prim bits), prim = -1 and t = -1 on a
// miss. Any hit: returns prim >= 0 iff some accepted hit has t < tmax. Counts visited nodes and
// tested triangles when COUNT is set. SH > 0: the bottom SH stack entries live in the shared
// column sh_col (stride sh_stride). TOP: the n_top nodes nearest the root are read from 'top'
// (shared memory) instead of 'nodes'.
template <bool ANY_HIT, bool COUNT, int SH = 0, int TRI = kTriMollerTrumbore, bool TOP = false>
GBPT_HD float4 trace_ray(const uint4* __restrict__ nodes, const float4* __restrict__ tris, const float4 ot,
                         const float4 dt, const int32_t skip_prim, uint32_t& n_nodes, uint32_t& n_tris,
                         uint2* sh_col = nullptr, int sh_stride = 0, const uint4* top = nullptr, uint32_t n_top = 0)
{
    const float ox = ot.x, oy = ot.y, oz = ot.z, ray_tmin = ot.w;
    const float dx = dt.x, dy = dt.y, dz = dt.z;
    WatertightRay wr = {0, 1, 2, 0.0f, 0.0f, 0.0f};
    if constexpr (TRI == kTriWatertight) wr = watertight_ray(dx, dy, dz);
    const float idx = safe_rcp(dx), idy = safe_rcp(dy), idz = safe_rcp(dz);
    const uint32_t oct_inv = (dx >= 0.0f ? 4u : 0u) | (dy >= 0.0f ? 2u : 0u) | (dz >= 0.0f ? 1u : 0u);

    float t_best = dt.w;  // hits must satisfy t < tmax
    float u_best = 0.0f, v_best = 0.0f;
    int32_t prim_best = -1;

    TraversalStack<SH> stack;
    int sp = 0;
    uint2 ngroup = make_uint2(0u, 0x80000000u);
    uint2 tgroup = make_uint2(0u, 0u);

    for (;;)
    {
        if (ngroup.y & 0xFF000000u)
        {
            const uint32_t hits_imask = ngroup.y;
            const uint32_t bit = 31u - __clz(hits_imask & 0xFF000000u);
            ngroup.y &= ~(1u << bit);
            if (ngroup.y & 0xFF000000u) stack.push(sp, ngroup, sh_col, sh_stride);
            const uint32_t slot = (bit - 24u) ^ oct_inv;
            const uint32_t rel = __popc(hits_imask & ~(0xFFFFFFFFu << slot));
            const uint32_t ni = ngroup.x + rel;
            uint4 w0, w1, w2, w3, w4;
            if (TOP && ni < n_top)
            {
                // one of the nodes nearest the root, staged in shared memory by the kernel
                const uint4* tp = top + 5 * ni;
                w0 = tp[0];
                w1 = tp[1];
                w2 = tp[2];
                w3 = tp[3];
                w4 = tp[4];
            }
            else
            {
                const uint4* np = nodes + 5 * (size_t)ni;
                w0 = GBPT_LDG(np + 0);
                w1 = GBPT_LDG(np + 1);
                w2 = GBPT_LDG(np + 2);
                w3 = GBPT_LDG(np + 3);
                w4 = GBPT_LDG(np + 4);
            }
            if (COUNT) n_nodes++;
            const uint32_t hm = intersect_children(w0, w1, w2, w3, w4, ox, oy, oz, idx, idy, idz, ray_tmin,
                                                   ANY_HIT ? dt.w : t_best, oct_inv);
            ngroup = make_uint2(w1.x, (hm & 0xFF000000u) | (w0.w >> 24));
            tgroup = make_uint2(w1.y, hm & 0x00FFFFFFu);
        }

        while (tgroup.y != 0u)
        {
            const int b = __ffs(tgroup.y) - 1;
            tgroup.y &= tgroup.y - 1u;
            const size_t ti = (size_t)(tgroup.x + (uint32_t)b);
            const float4 a = GBPT_LDG(tris + 3 * ti), vb = GBPT_LDG(tris + 3 * ti + 1), vc = GBPT_LDG(tris + 3 * ti + 2);
            if (COUNT) n_tris++;
            float t, u, v;
            if (!tri_test<TRI>(wr, a, vb, vc, ox, oy, oz, dx, dy, dz, t, u, v)) continue;
            const int32_t prim = __float_as_int(a.w);
            if (t < ray_tmin || prim == skip_prim) continue;
            if (ANY_HIT)
            {
                if (t < dt.w) return make_float4(t, u, v, __int_as_float(prim));
            }
            else if (t < t_best || (t == t_best && prim < prim_best))
            {
                t_best = t;
                u_best = u;
                v_best = v;
                prim_best = prim;
            }
        }

        if (!(ngroup.y & 0xFF000000u))
        {
            if (sp == 0) break;
            ngroup = stack.pop(sp, sh_col, sh_stride);
        }
    }
    return prim_best >= 0 ? make_float4(t_best, u_best, v_best, __int_as_float(prim_best))
                          : make_float4(-1.0f, 0.0f, 0.0f, __int_as_float(-1));
}

}  // namespace core
}  // namespace gbpt
