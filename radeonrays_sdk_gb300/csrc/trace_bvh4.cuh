// trace_bvh4.cuh -- device helpers for the 4-wide fp32 node format, shared
// by the single-level (trace_bvh4.cu) and two-level (trace_scene_bvh4.cu)
// kernels: the node test with its nearest-first ordering, and a short stack
// that spills and refills in full blocks.
#pragma once
#include "trace_persistent.cuh"
#include "trace_precise.cuh"

namespace rr
{
// The short stack spills and refills in blocks of kB4Spill entries (every
// block in the global region is full).
constexpr int kB4Spill = 8;

// Make room for `k` (at most 3) more short-stack entries: when they would not
// fit, the bottom kB4Spill entries go to the global region and the rest move
// down.  A spill happens with sp >= st.depth - 2 >= kB4Spill entries (the
// depth is at least 12).
__device__ __forceinline__ void b4_reserve(int& sp, uint32_t& gsp, const PStack& st, DeviceWords* words, int k)
{
    if (sp + k <= st.depth) return;
    if (gsp + kB4Spill > st.gcap)
    {
        raise_error(words, RR_CUDA_DEVICE_ERROR_STACK_OVERFLOW);
        sp = st.depth - k;  // overwrite the top entries: result flagged invalid
        return;
    }
    for (int j = 0; j < kB4Spill; ++j) st.g[gsp + j] = st.at(j);
    for (int j = kB4Spill; j < sp; ++j) st.at(j - kB4Spill) = st.at(j);
    gsp += kB4Spill;
    sp -= kB4Spill;
}

// Pops into `out`; false when the stack is empty.
__device__ __forceinline__ bool b4_pop(int& sp, uint32_t& gsp, const PStack& st, uint32_t& out)
{
    if (sp == 0 && gsp == 0) return false;
    if (sp == 0)
    {
        gsp -= kB4Spill;
        for (int k = 0; k < kB4Spill; ++k) st.at(k) = st.g[gsp + k];
        sp = kB4Spill;
    }
    out = st.at(--sp);
    return true;
}

// Three-input min / max (one instruction each on sm_100 and later); with
// NaN operands they return the minimum / maximum of the others, like a chain
// of fminf / fmaxf.
__device__ __forceinline__ float b4_max3(float a, float b, float c)
{
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
__device__ __forceinline__ float b4_min3(float a, float b, float c)
{
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// Order (key, ref) pairs ascending by key (misses carry +inf).
__device__ __forceinline__ void b4_cas(float& ka, uint32_t& ra, float& kb, uint32_t& rb)
{
    const bool     sw = kb < ka;
    const float    k  = sw ? kb : ka;
    const uint32_t r  = sw ? rb : ra;
    kb                = sw ? ka : kb;
    rb                = sw ? ra : rb;
    ka                = k;
    ra                = r;
}

// The hit children of a 4-wide node, nearest first: r[0..n).
struct B4Hits
{
    int      n;
    uint32_t r0, r1, r2, r3;
};

// Slab test of the four children with the reference's formula
// (vlk/kernels/common.h:150-164), evaluated on the near and far planes
// picked by the signs of the inverse direction: for inv > 0,
// fma(hi, inv, oxi) >= fma(lo, inv, oxi), so the reference's min / max of
// the two are exactly these.  The boxes are stored lo[3][4] then hi[3][4],
// so the choice is a load offset.
// kRobust (the precise triangle test's traversal, trace_precise.cuh): `inv`
// is the exact reciprocal, `oxi` the ray origin, the distances are
// (p - o) * inv and the far one is moved outward by 2 gamma_3.
template <bool kRobust = false>
__device__ __forceinline__ B4Hits b4_children(const Bvh4Node* node, F3 inv, F3 oxi, float tmin, float ct)
{
    const float4* p  = reinterpret_cast<const float4*>(node);
    const int     ox = inv.x < 0.f ? 3 : 0, oy = inv.y < 0.f ? 3 : 0, oz = inv.z < 0.f ? 3 : 0;
    const float4  nx = __ldg(p + ox), ny = __ldg(p + 1 + oy), nz = __ldg(p + 2 + oz);
    const float4  fx = __ldg(p + 3 - ox), fy = __ldg(p + 4 - oy), fz = __ldg(p + 5 - oz);
    const uint4   cr = __ldg(reinterpret_cast<const uint4*>(p + 6));
    auto          key = [&](float ax, float ay, float az, float bx, float by, float bz, uint32_t r) {
        float t0, t1;
        if (kRobust)
        {
            t0 = fmaxf(b4_max3((ax - oxi.x) * inv.x, (ay - oxi.y) * inv.y, (az - oxi.z) * inv.z), tmin);
            t1 = robust_far(fminf(b4_min3((bx - oxi.x) * inv.x, (by - oxi.y) * inv.y, (bz - oxi.z) * inv.z), ct));
        }
        else
        {
            t0 = fmaxf(b4_max3(fmaf(ax, inv.x, oxi.x), fmaf(ay, inv.y, oxi.y), fmaf(az, inv.z, oxi.z)), tmin);
            t1 = fminf(b4_min3(fmaf(bx, inv.x, oxi.x), fmaf(by, inv.y, oxi.y), fmaf(bz, inv.z, oxi.z)), ct);
        }
        return (t0 <= t1 && r != kInvalid) ? t0 : INFINITY;
    };
    float  k0 = key(nx.x, ny.x, nz.x, fx.x, fy.x, fz.x, cr.x);
    float  k1 = key(nx.y, ny.y, nz.y, fx.y, fy.y, fz.y, cr.y);
    float  k2 = key(nx.z, ny.z, nz.z, fx.z, fy.z, fz.z, cr.z);
    float  k3 = key(nx.w, ny.w, nz.w, fx.w, fy.w, fz.w, cr.w);
    B4Hits h;
    h.r0 = cr.x;
    h.r1 = cr.y;
    h.r2 = cr.z;
    h.r3 = cr.w;
    // A box hit has a finite entry distance: tmin <= t0 <= t1 <= closest t.
    h.n = (k0 < INFINITY) + (k1 < INFINITY) + (k2 < INFINITY) + (k3 < INFINITY);
    // The network runs whatever n is (no branch): misses carry +inf, so the
    // hit children end up first, nearest first, and a single hit in slot 0.
    b4_cas(k0, h.r0, k1, h.r1);
    b4_cas(k2, h.r2, k3, h.r3);
    b4_cas(k0, h.r0, k2, h.r2);
    b4_cas(k1, h.r1, k3, h.r3);
    b4_cas(k1, h.r1, k2, h.r2);
    return h;
}

// The same test on a quantised node (Bvh4QNode, four 16-byte loads instead of
// seven): each child plane decodes exactly to 2^15 + q (byte q permuted into
// the second mantissa byte of 2^15, no conversion) and is evaluated as
// fma(2^15 + q, A, B -+ eps) with A = 2^e * inv (exact) and
// B = fma(p, inv, oxi) - 2^15 A, on the near (-) and far (+) planes picked by
// the direction's signs.  eps = 2^-7 |A| + 2^-20 |B| bounds the roundings of
// B, of B - 2^15 A and of B -+ eps (together at most 2^-8 |A| + 2^-22 |B|),
// so the near distance is never above the reference's on the exact child box
// and the far distance never below it (the argument of the 8-wide kernel,
// trace_wide.cuh): a child the reference's slab test admits on its exact box
// is always admitted.  The magic 2^23 + q (byte in the low mantissa byte)
// would round B - 2^23 A to half a quantisation step and need eps = 1.25 |A|:
// measured on the 16.8 M-ray heightfield, 5 % more node fetches and 5 %
// slower.  Directed roundings instead of eps (every fma rounded down on the
// near planes, up on the far ones) made the resident kernel 0.4 % faster but
// its streamed variant 16 % slower (5.26 against 4.53 ms per e2e step).
//
// kRobust (the precise triangle test's traversal): `inv` is the exact
// reciprocal and `oxi` the origin.  Each plane is decoded to at most (lo
// planes) or at least (hi planes) p + q 2^e by directed roundings, so the
// decoded box still contains the exact child box, and is then tested with
// the robust slab distances of b4_children<true>: a child box the exact ray
// segment touches is never culled.
template <bool kRobust = false>
__device__ __forceinline__ B4Hits b4q_children(const Bvh4QNode* node, F3 inv, F3 oxi, float tmin, float ct,
                                               bool sort = true)
{
    const uint4* p  = reinterpret_cast<const uint4*>(node);
    const uint4  w0 = __ldg(p), cr = __ldg(p + 1), q0 = __ldg(p + 2), q1 = __ldg(p + 3);
    // Planes: q0 = lo x, lo y, lo z, hi x; q1 = hi y, hi z.
    const bool     sx = inv.x < 0.f, sy = inv.y < 0.f, sz = inv.z < 0.f;
    const uint32_t nxw = sx ? q0.w : q0.x, fxw = sx ? q0.x : q0.w;
    const uint32_t nyw = sy ? q1.x : q0.y, fyw = sy ? q0.y : q1.x;
    const uint32_t nzw = sz ? q1.y : q0.z, fzw = sz ? q0.z : q1.y;
    if (kRobust)
    {
        // An axis with a negative direction is mirrored (x -> -x, o -> -o,
        // inv -> -inv: the slab distances are the same fp32 operations), so
        // that its near plane (the hi plane) is evaluated as a lo plane.  In
        // mirrored coordinates every near plane is decoded rounded down and
        // every far plane rounded up, each as one fma on 2^15 + q:
        //   plane = fma(2^15 + q, g, P),  g = +-2^e,
        //   P = p - 2^15 2^e rounded down (near) or up (far), mirrored,
        // so the decoded box still contains the exact child box.
        const float g[3] = {__uint_as_float((w0.w & 0xffu) << 23), __uint_as_float(((w0.w >> 8) & 0xffu) << 23),
                            __uint_as_float(((w0.w >> 16) & 0xffu) << 23)};
        const float p3[3] = {__uint_as_float(w0.x), __uint_as_float(w0.y), __uint_as_float(w0.z)};
        const bool  s3[3] = {sx, sy, sz};
        const float o3[3] = {oxi.x, oxi.y, oxi.z}, i3[3] = {inv.x, inv.y, inv.z};
        float       G[3], Pn[3], Pf[3], O[3], I[3];
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            const float lo = __fadd_rd(p3[k], -32768.0f * g[k]), hi = __fadd_ru(p3[k], -32768.0f * g[k]);
            G[k]  = s3[k] ? -g[k] : g[k];
            Pn[k] = s3[k] ? -hi : lo;
            Pf[k] = s3[k] ? -lo : hi;
            O[k]  = s3[k] ? -o3[k] : o3[k];
            I[k]  = s3[k] ? -i3[k] : i3[k];
        }
#define RR_B4Q(w, c) __int_as_float((int)__byte_perm((w), 0x47000000u, 0x7504u | ((c) << 4)))
        auto key = [&](int c, uint32_t r) {
            const float ax = __fmaf_rd(RR_B4Q(nxw, c), G[0], Pn[0]), ay = __fmaf_rd(RR_B4Q(nyw, c), G[1], Pn[1]),
                        az = __fmaf_rd(RR_B4Q(nzw, c), G[2], Pn[2]);
            const float bx = __fmaf_ru(RR_B4Q(fxw, c), G[0], Pf[0]), by = __fmaf_ru(RR_B4Q(fyw, c), G[1], Pf[1]),
                        bz = __fmaf_ru(RR_B4Q(fzw, c), G[2], Pf[2]);
            const float t0 = fmaxf(b4_max3((ax - O[0]) * I[0], (ay - O[1]) * I[1], (az - O[2]) * I[2]), tmin);
            const float t1 = robust_far(fminf(b4_min3((bx - O[0]) * I[0], (by - O[1]) * I[1], (bz - O[2]) * I[2]), ct));
            return (t0 <= t1 && r != kInvalid) ? t0 : INFINITY;
        };
#undef RR_B4Q
        float  k0 = key(0, cr.x), k1 = key(1, cr.y), k2 = key(2, cr.z), k3 = key(3, cr.w);
        B4Hits h;
        h.r0 = cr.x;
        h.r1 = cr.y;
        h.r2 = cr.z;
        h.r3 = cr.w;
        h.n  = (k0 < INFINITY) + (k1 < INFINITY) + (k2 < INFINITY) + (k3 < INFINITY);
        b4_cas(k0, h.r0, k1, h.r1);
        b4_cas(k2, h.r2, k3, h.r3);
        b4_cas(k0, h.r0, k2, h.r2);
        b4_cas(k1, h.r1, k3, h.r3);
        b4_cas(k1, h.r1, k2, h.r2);
        return h;
    }
    float          A[3], Bn[3], Bf[3];
    {
        const float p3[3] = {__uint_as_float(w0.x), __uint_as_float(w0.y), __uint_as_float(w0.z)};
        const float i3[3] = {inv.x, inv.y, inv.z}, o3[3] = {oxi.x, oxi.y, oxi.z};
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            const float sc  = __uint_as_float(((w0.w >> (8 * k)) & 0xffu) << 23);
            const float a   = sc * i3[k];
            const float b   = fmaf(p3[k], i3[k], o3[k]);
            const float eps = fmaf(fabsf(a), 0.0078125f, fabsf(b) * 9.5367431640625e-07f);
            const float m   = fmaf(-32768.0f, a, b);
            A[k]            = a;
            Bn[k]           = m - eps;
            Bf[k]           = m + eps;
        }
    }
#define RR_B4Q(w, c) __int_as_float((int)__byte_perm((w), 0x47000000u, 0x7504u | ((c) << 4)))
    auto key = [&](int c, uint32_t r) {
        const float t0 = fmaxf(b4_max3(fmaf(RR_B4Q(nxw, c), A[0], Bn[0]), fmaf(RR_B4Q(nyw, c), A[1], Bn[1]),
                                       fmaf(RR_B4Q(nzw, c), A[2], Bn[2])),
                               tmin);
        const float t1 = fminf(b4_min3(fmaf(RR_B4Q(fxw, c), A[0], Bf[0]), fmaf(RR_B4Q(fyw, c), A[1], Bf[1]),
                                       fmaf(RR_B4Q(fzw, c), A[2], Bf[2])),
                               ct);
        return (t0 <= t1 && r != kInvalid) ? t0 : INFINITY;
    };
#undef RR_B4Q
    float  k0 = key(0, cr.x), k1 = key(1, cr.y), k2 = key(2, cr.z), k3 = key(3, cr.w);
    B4Hits h;
    h.r0 = cr.x;
    h.r1 = cr.y;
    h.r2 = cr.z;
    h.r3 = cr.w;
    if (!sort)
    {
        // Hit mask in n, slots as stored (b4_descend_mask).
        h.n = (k0 < INFINITY ? 1 : 0) | (k1 < INFINITY ? 2 : 0) | (k2 < INFINITY ? 4 : 0) | (k3 < INFINITY ? 8 : 0);
        return h;
    }
    h.n  = (k0 < INFINITY) + (k1 < INFINITY) + (k2 < INFINITY) + (k3 < INFINITY);
    b4_cas(k0, h.r0, k1, h.r1);
    b4_cas(k2, h.r2, k3, h.r3);
    b4_cas(k0, h.r0, k2, h.r2);
    b4_cas(k1, h.r1, k3, h.r3);
    b4_cas(k1, h.r1, k2, h.r2);
    return h;
}

// Pushes the hit children after the nearest (farthest first) and returns the
// nearest; the caller has h.n >= 1.
__device__ __forceinline__ uint32_t b4_descend(const B4Hits& h, int& sp, uint32_t& gsp, const PStack& st,
                                               DeviceWords* words)
{
    b4_reserve(sp, gsp, st, words, h.n - 1);
    if (h.n > 3) st.at(sp++) = h.r3;
    if (h.n > 2) st.at(sp++) = h.r2;
    if (h.n > 1) st.at(sp++) = h.r1;
    return h.r0;
}

// Any-hit order over quantised nodes: the first hit slot is visited next, the
// other hit slots are pushed (lowest slot on top); h.n holds the hit mask
// (b4q_children with sort = false).  An occlusion query stops at any hit, so
// it skips the nearest-first sort: measured on the 16.8 M-ray heightfield
// with tmax ~ U[0.01, 0.5], 1.3 % more node fetches and 2.5 % faster.
__device__ __forceinline__ uint32_t b4_descend_mask(const B4Hits& h, int& sp, uint32_t& gsp, const PStack& st,
                                                    DeviceWords* words)
{
    const uint32_t m     = (uint32_t)h.n;
    const int      first = __ffs(m) - 1;
    b4_reserve(sp, gsp, st, words, __popc(m) - 1);
    if ((m & 8u) && first != 3) st.at(sp++) = h.r3;
    if ((m & 4u) && first != 2) st.at(sp++) = h.r2;
    if ((m & 2u) && first != 1) st.at(sp++) = h.r1;
    return first == 0 ? h.r0 : first == 1 ? h.r1 : first == 2 ? h.r2 : h.r3;
}

// Traversal state of one ray of the 4-wide kernels (kept in registers between
// steps so that a persistent kernel can retire finished rays and start new
// ones per lane).
struct B4Ray
{
    Ray      ray;
    F3       inv, oxi;
    float    ct;
    uint32_t best;   // binary leaf node of the closest hit (kInvalid: none)
    uint32_t ref;    // reference to fetch next
    uint32_t gsp;    // entries spilled to global
    uint32_t steps;
    int      sp;     // entries in the short stack
};

// kPrecise: `inv` is the exact reciprocal and `oxi` the origin (the robust
// box test of trace_precise.cuh).
template <bool kPrecise>
__device__ __forceinline__ void b4_start(B4Ray& s, const Ray& r)
{
    s.ray  = r;
    s.inv  = kPrecise ? exact_invdir(r.d) : safe_invdir(r.d);
    s.oxi  = kPrecise ? r.o : f3(-r.o.x * s.inv.x, -r.o.y * s.inv.y, -r.o.z * s.inv.z);
    s.ct   = r.tmax;
    s.best = kInvalid;
    s.ref  = 0;  // the root 4-wide node
    s.gsp = s.steps = 0;
    s.sp            = 0;
}

// One step; returns true when the ray is finished (stack empty, or a hit
// accepted by an any-hit query).  nf / tf count node and leaf fetches.
// kRuntime: the query is `any` (requests of both kinds in one launch).
// kQ8: the nodes are Bvh4QNode (quantised bounds); a leaf triangle's hit
// then counts only if its exact box (min / max of its vertices, the box its
// binary parent holds) passes the reference's slab test too, so a triangle
// whose exact box the reference culls is not reached through the larger
// quantised box either.  With kPrecise the nodes take the robust test and the
// leaves go straight to the precise triangle test (no box test decides a hit
// there, so no re-test is needed).
template <bool kAny, bool kPrecise, bool kRuntime = false, bool kQ8 = false>
__device__ __forceinline__ bool b4_step(B4Ray& s, const Bvh4Node* __restrict__ wn, const BvhNode* __restrict__ nodes,
                                        uint32_t wlim, uint32_t first_leaf, uint32_t node_limit, const PStack& st,
                                        DeviceWords* words, uint32_t& nf, uint32_t& tf, bool any = false)
{
    const uint32_t ref = s.ref;
    const bool     leaf = (ref & kBvh4Leaf) != 0;
    const uint32_t idx  = ref & ~kBvh4Leaf;
    if (++s.steps > kFetchCap || (leaf ? (idx < first_leaf || idx >= node_limit) : idx >= wlim))
    {
        raise_error(words, RR_CUDA_DEVICE_ERROR_NODE_RANGE);
        s.best = kInvalid;
        return true;
    }
    bool pop = true, done = false;
    if (leaf)
    {
        const float4* p = reinterpret_cast<const float4*>(nodes + idx);
        const float4  a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
        ++tf;
        const F3 v0 = f3(a.x, a.y, a.z), v1 = f3(b.x, b.y, b.z), v2 = f3(c.x, c.y, c.z);
        float t = kPrecise ? isect_tri_precise(s.ray, v0, v1, v2, s.ct) : isect_tri(s.ray, v0, v1, v2, s.ct);
        // The exact-box re-test decides only whether a triangle hit counts,
        // so it runs after the triangle test and only on a hit (the same
        // outcome as testing the box first; the precise test needs no
        // re-test, its box test being conservative).
        if (kQ8 && !kPrecise && t < s.ct)
        {
            float b0, b1;
            isect_box(f3(b4_min3(v0.x, v1.x, v2.x), b4_min3(v0.y, v1.y, v2.y), b4_min3(v0.z, v1.z, v2.z)),
                      f3(b4_max3(v0.x, v1.x, v2.x), b4_max3(v0.y, v1.y, v2.y), b4_max3(v0.z, v1.z, v2.z)), s.inv,
                      s.oxi, s.ct, s.ray.tmin, b0, b1);
            if (!(b0 <= b1)) t = s.ct;
        }
        if (t < s.ct)
        {
            s.ct   = t;
            s.best = idx;
            if (kAny || (kRuntime && any)) done = true;
        }
    }
    else
    {
        // Any-hit queries over quantised nodes take the unsorted order (the
        // multi-request kernel decides per ray, so that a request's hits
        // equal its trace alone).
        const bool   mask = kQ8 && !kPrecise && (kAny || (kRuntime && any));
        const B4Hits h    = kQ8 ? b4q_children<kPrecise>(reinterpret_cast<const Bvh4QNode*>(wn) + idx, s.inv, s.oxi,
                                                         s.ray.tmin, s.ct, !mask)
                                : b4_children<kPrecise>(wn + idx, s.inv, s.oxi, s.ray.tmin, s.ct);
        ++nf;
        if (h.n)
        {
            s.ref = mask ? b4_descend_mask(h, s.sp, s.gsp, st, words) : b4_descend(h, s.sp, s.gsp, st, words);
            pop   = false;
        }
    }
    if (pop && !done && !b4_pop(s.sp, s.gsp, st, s.ref)) done = true;
    return done;
}

}  // namespace rr
