// trace_wide.cuh -- traversal of one ray through an 8-wide BVH (device code
// shared by the single-level kernel, trace_wide.cu, and the two-level kernel,
// scene.cu).  Node format and conservativeness argument: wide.cu.
//
// Per node: the 8 child boxes are decoded to fp32 (fma(q, 2^e, p), exact
// byte -> float via a PRMT-built 2^15 + q) and slab-tested with the
// reference's formula (vlk/kernels/common.h:150-164), evaluating only the
// near plane and the far plane of each axis (chosen by the sign of the
// inverse direction, which yields exactly the reference's min/max result).
// Children are visited in the order i = 0..7 of slot i ^ octant(ray): the
// build places children in octant slots, so this order is roughly front to
// back.  The traversal stack holds node groups (first child index, internal
// slot mask, remaining hit mask), one entry per visited node, not per child.
#pragma once
#include "trace_common.cuh"

namespace rr
{
constexpr int kWideShortStack = 16;

struct WideEntry
{
    uint32_t base;  // index of the group's first internal child
    uint32_t bits;  // [7:0] internal-slot mask of the parent, [15:8] remaining hits (visit order)
};

// Per-thread traversal stack: a short stack in shared memory that spills
// kWideShortStack entries at a time to a per-thread global region.
constexpr int kWideBlock = 128;  // threads per block of the wide kernels

struct WideStack
{
    WideEntry* s;  // this thread's first short-stack entry (shared); entries are
                   // interleaved across the block (kWideBlock apart): no bank conflicts
    WideEntry* g;  // gcap entries (global scratch)
    uint32_t   gcap;
    __device__ __forceinline__ WideEntry& at(int k) const { return s[k * kWideBlock]; }
};

// Exact float of byte b (compile-time index) of w: bits of 2^23 + q, minus 2^23.
template <int b>
__device__ __forceinline__ float qbyte(uint32_t w)
{
    return __int_as_float((int)__byte_perm(w, 0x4B000000u, 0x7540u | b)) - 8388608.0f;
}

// Three-input min / max (one instruction each on sm_100 and later).
__device__ __forceinline__ float max3f(float a, float b, float c)
{
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
__device__ __forceinline__ float min3f(float a, float b, float c)
{
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// Bit 7 of each byte of w gathered into bits 0..3.
__device__ __forceinline__ uint32_t byte_msbs(uint32_t w) { return (((w >> 7) & 0x01010101u) * 0x01020408u) >> 24; }

// Traversal state of one ray (kept in registers between steps so that a
// persistent kernel can retire finished rays and start new ones per lane).
struct WideRay
{
    Ray      ray;
    F3       inv, oxi;
    float    ct;     // closest hit distance so far
    uint32_t best;   // triangle index of the closest hit
    uint32_t node;   // next node to fetch (kInvalid: pop a group)
    uint32_t gbase;  // current node group
    uint32_t gbits;
    uint32_t gsp;    // entries spilled to global
    uint32_t steps;
    int      sp;     // entries in the short stack
};

__device__ __forceinline__ void wide_begin(WideRay& s, const Ray& r, bool empty)
{
    s.ray   = r;
    s.inv   = safe_invdir(r.d);
    s.oxi   = f3(-r.o.x * s.inv.x, -r.o.y * s.inv.y, -r.o.z * s.inv.z);
    s.ct    = r.tmax;
    s.best  = kInvalid;
    s.node  = empty ? kInvalid : 0u;
    s.gbase = s.gbits = s.gsp = s.steps = 0;
    s.sp    = 0;
}

// One traversal step: fetch and test one node (popping a group first when no
// node is pending), test the triangles of its hit leaf slots, push the
// remaining hit internal children as a group.  Returns true when the ray is
// finished: stack empty (closest hit) or a triangle accepted (any hit).
template <bool kAny>
__device__ __forceinline__ bool wide_step(WideRay& s, const WideNode* __restrict__ wn, const WideTri* __restrict__ wt,
                                          uint32_t wlim, uint32_t tlim, const WideStack& st, DeviceWords* words,
                                          uint32_t& nfetch, uint32_t& tfetch, uint32_t amask = 0u)
{
    const bool     bx = s.inv.x < 0.f, by = s.inv.y < 0.f, bz = s.inv.z < 0.f;
    const uint32_t oct = (bx ? 4u : 0u) | (by ? 2u : 0u) | (bz ? 1u : 0u);
    const uint32_t o2  = oct & 3u;
    const uint32_t ps  = (0u ^ o2) | ((1u ^ o2) << 4) | ((2u ^ o2) << 8) | ((3u ^ o2) << 12);
    const bool     sw  = (oct & 4u) != 0;

    // Pick the node to fetch.  Written without early exits so that lanes that
    // pop and lanes that already have a node reconverge before the node test
    // (an exit inside this branch would let the two groups run it separately).
    bool done = false;
    if (s.node == kInvalid)
    {
        if ((s.gbits >> 8) == 0)
        {
            if (s.sp == 0 && s.gsp == 0)
                done = true;
            else
            {
                if (s.sp == 0)
                {
                    s.gsp -= kWideShortStack;
                    for (int k = 0; k < kWideShortStack; ++k) st.at(k) = st.g[s.gsp + k];
                    s.sp = kWideShortStack;
                }
                const WideEntry e = st.at(--s.sp);
                s.gbase           = e.base;
                s.gbits           = e.bits;
            }
        }
        if (!done)
        {
            const uint32_t i    = __ffs(s.gbits >> 8) - 1;
            s.gbits &= ~(0x100u << i);
            const uint32_t slot = i ^ oct;
            s.node              = s.gbase + __popc(s.gbits & ((1u << slot) - 1u) & 0xffu);
        }
    }
    if (!done && (++s.steps > kFetchCap || s.node >= wlim))
    {
        raise_error(words, RR_CUDA_DEVICE_ERROR_NODE_RANGE);
        s.best = kInvalid;
        done   = true;
    }
    // amask (when given) holds every lane of the warp that is in this step:
    // the lanes that go on to the node test wait for each other here so that
    // the node test runs once for all of them.
    const uint32_t go = amask ? __ballot_sync(amask, !done) : 0u;
    if (done) return true;
    if (amask) __syncwarp(go);

    const uint4* np = reinterpret_cast<const uint4*>(wn + s.node);
    const uint4  w0 = __ldg(np), w1 = __ldg(np + 1), w2 = __ldg(np + 2), w3 = __ldg(np + 3), w4 = __ldg(np + 4);
    ++nfetch;
    const float    px = __uint_as_float(w0.x), py = __uint_as_float(w0.y), pz = __uint_as_float(w0.z);
    const float    sx = __uint_as_float((w0.w & 0xffu) << 23);
    const float    sy = __uint_as_float(((w0.w >> 8) & 0xffu) << 23);
    const float    sz = __uint_as_float(((w0.w >> 16) & 0xffu) << 23);
    const uint32_t imask      = w0.w >> 24;
    const uint32_t child_base = w1.x, tri_base = w1.y;
    const F3       inv = s.inv, oxi = s.oxi;
    const float    tmin = s.ray.tmin, ct = s.ct;

    // Near / far byte arrays per axis, permuted into visit order.
    auto vis = [&](uint32_t a0, uint32_t a1, uint32_t& o0, uint32_t& o1) {
        const uint32_t t0 = sw ? a1 : a0, t1 = sw ? a0 : a1;
        o0 = __byte_perm(t0, 0u, ps);
        o1 = __byte_perm(t1, 0u, ps);
    };
    uint32_t nx0, nx1, fx0, fx1, ny0, ny1, fy0, fy1, nz0, nz1, fz0, fz1, m0, m1;
    vis(bx ? w3.z : w2.x, bx ? w3.w : w2.y, nx0, nx1);
    vis(bx ? w2.x : w3.z, bx ? w2.y : w3.w, fx0, fx1);
    vis(by ? w4.x : w2.z, by ? w4.y : w2.w, ny0, ny1);
    vis(by ? w2.z : w4.x, by ? w2.w : w4.y, fy0, fy1);
    vis(bz ? w4.z : w3.x, bz ? w4.w : w3.y, nz0, nz1);
    vis(bz ? w3.x : w4.z, bz ? w3.y : w4.w, fz0, fz1);
    vis(w1.z, w1.w, m0, m1);

    // Slab distances in quantised space.  For a plane at byte q of axis a the
    // reference evaluates fma(c, inv, oxi) on the child coordinate c; here
    //   t = fma(2^15 + q, A, B -+ eps),  A = 2^e * inv (exact),
    //   B = fma(p, inv, oxi) - 2^15 * A (rounded),
    // with eps = 2^-7 |A| + 2^-20 |B| on the near (-) and far (+) planes.  eps
    // bounds the rounding of B, of B - 2^15 A and of B -+ eps (together at
    // most 2^-8 |A| + 2^-22 |B|: the magic 2^15 + q, placed in the second
    // mantissa byte, keeps B - 2^15 A within 2^15 |A| + |B|, where 2^23 + q
    // cost half a quantisation step); as the decoded coordinate lies outside
    // the exact child bound and rounding is monotone, the near distance never
    // exceeds the reference's on the exact box and the far distance is never
    // below it.  A ray the reference's test admits is therefore always
    // admitted.  (The 2^23 form with eps = 1.25 |A| visited 7 % more nodes.
    // Directed roundings instead of eps, as in the 4-wide kernel, were 1.6 %
    // slower here.)
    float An[3], Bn[3], Bf[3];
    {
        const float s3[3] = {sx, sy, sz}, p3[3] = {px, py, pz}, i3[3] = {inv.x, inv.y, inv.z},
                    o3[3] = {oxi.x, oxi.y, oxi.z};
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            const float A   = s3[k] * i3[k];
            const float B   = fmaf(p3[k], i3[k], o3[k]);
            const float eps = fmaf(fabsf(A), 0.0078125f, fabsf(B) * 9.5367431640625e-07f);
            const float M   = fmaf(-32768.0f, A, B);
            An[k]           = A;
            Bn[k]           = M - eps;
            Bf[k]           = M + eps;
        }
    }
    // Hit bits per visit position; empty slots are masked out below through
    // the meta bytes (internal: bit 7; leaf: bit 7 clear, count in bits 5-6).
    uint32_t hits = 0;
#define RR_WIDE_Q(w, b) __int_as_float((int)__byte_perm((w), 0x47000000u, 0x7504u | ((b) << 4)))
#define RR_WIDE_CHILD(i, W)                                                                                         \
    {                                                                                                               \
        const float tnx = fmaf(RR_WIDE_Q(W##nx, (i) & 3), An[0], Bn[0]);                                            \
        const float tfx = fmaf(RR_WIDE_Q(W##fx, (i) & 3), An[0], Bf[0]);                                            \
        const float tny = fmaf(RR_WIDE_Q(W##ny, (i) & 3), An[1], Bn[1]);                                            \
        const float tfy = fmaf(RR_WIDE_Q(W##fy, (i) & 3), An[1], Bf[1]);                                            \
        const float tnz = fmaf(RR_WIDE_Q(W##nz, (i) & 3), An[2], Bn[2]);                                            \
        const float tfz = fmaf(RR_WIDE_Q(W##fz, (i) & 3), An[2], Bf[2]);                                            \
        const float t0  = fmaxf(max3f(tnx, tny, tnz), tmin);                                                        \
        const float t1  = fminf(min3f(tfx, tfy, tfz), ct);                                                          \
        hits |= (t0 <= t1) ? (1u << (i)) : 0u;                                                                      \
    }
    {
        const uint32_t lo_nx = nx0, lo_fx = fx0, lo_ny = ny0, lo_fy = fy0, lo_nz = nz0, lo_fz = fz0;
        const uint32_t hi_nx = nx1, hi_fx = fx1, hi_ny = ny1, hi_fy = fy1, hi_nz = nz1, hi_fz = fz1;
        RR_WIDE_CHILD(0, lo_)
        RR_WIDE_CHILD(1, lo_)
        RR_WIDE_CHILD(2, lo_)
        RR_WIDE_CHILD(3, lo_)
        RR_WIDE_CHILD(4, hi_)
        RR_WIDE_CHILD(5, hi_)
        RR_WIDE_CHILD(6, hi_)
        RR_WIDE_CHILD(7, hi_)
    }
#undef RR_WIDE_CHILD
#undef RR_WIDE_Q
    const uint32_t int_mask  = byte_msbs(m0) | (byte_msbs(m1) << 4);
    const uint32_t leaf_mask = byte_msbs(((m0 << 1) | (m0 << 2)) & ~m0) | (byte_msbs(((m1 << 1) | (m1 << 2)) & ~m1) << 4);
    const uint32_t ihit      = hits & int_mask;
    uint32_t       lhit      = hits & leaf_mask;

    // Leaf slots: test their triangles in visit order.
    while (lhit)
    {
        const uint32_t i    = __ffs(lhit) - 1;
        lhit &= lhit - 1;
        const uint32_t meta = ((i < 4 ? m0 : m1) >> (8 * (i & 3))) & 0xffu;
        uint32_t       cnt = (meta >> 5) & 3u;
        const uint32_t off = meta & 31u;
        if (tri_base + off + cnt > tlim)
        {
            raise_error(words, RR_CUDA_DEVICE_ERROR_NODE_RANGE);
            cnt = 0;
        }
        for (uint32_t j = 0; j < cnt; ++j)
        {
            const uint32_t ti = tri_base + off + j;
            const float4*  tp = reinterpret_cast<const float4*>(wt + ti);
            const float4   A = __ldg(tp), B = __ldg(tp + 1), C = __ldg(tp + 2);
            ++tfetch;
            // The binary path reaches a triangle only through its exact box
            // (its slot in the binary parent: the refit's min / max of the
            // vertices) and the reference's fp32 slab test.  The quantised
            // slot box here is larger, so a hit counts only if the exact box
            // passes that test too: a grazing ray that the fp32 slab test
            // rejects on the exact box does not hit the triangle here either.
            // (The box decides only whether a hit counts, so it is tested
            // after the triangle, on hits only.)
            const float t = isect_tri(s.ray, f3(A.x, A.y, A.z), f3(B.x, B.y, B.z), f3(C.x, C.y, C.z), s.ct);
            if (t < s.ct)
            {
                float b0, b1;
                isect_box(f3(fminf(fminf(A.x, B.x), C.x), fminf(fminf(A.y, B.y), C.y), fminf(fminf(A.z, B.z), C.z)),
                          f3(fmaxf(fmaxf(A.x, B.x), C.x), fmaxf(fmaxf(A.y, B.y), C.y), fmaxf(fmaxf(A.z, B.z), C.z)),
                          s.inv, s.oxi, s.ct, s.ray.tmin, b0, b1);
                if (b0 > b1) continue;
                s.ct   = t;
                s.best = ti;
                if (kAny) done = true;
            }
        }
        if (kAny && done) break;
    }
    if (kAny && done) return true;

    if (ihit)
    {
        if (s.gbits >> 8)
        {
            if (s.sp == kWideShortStack)
            {
                if (s.gsp + kWideShortStack > st.gcap)
                {
                    raise_error(words, RR_CUDA_DEVICE_ERROR_STACK_OVERFLOW);
                    s.sp = kWideShortStack - 1;  // overwrite the top entry: result flagged invalid
                }
                else
                {
                    for (int k = 0; k < kWideShortStack; ++k) st.g[s.gsp + k] = st.at(k);
                    s.gsp += kWideShortStack;
                    s.sp = 0;
                }
            }
            st.at(s.sp++) = WideEntry{s.gbase, s.gbits};
        }
        s.gbase             = child_base;
        s.gbits             = imask | (ihit << 8);
        const uint32_t i    = __ffs(ihit) - 1;
        s.gbits &= ~(0x100u << i);
        const uint32_t slot = i ^ oct;
        s.node              = s.gbase + __popc(s.gbits & ((1u << slot) - 1u) & 0xffu);
    }
    else
        s.node = kInvalid;
    return false;
}

// Whole traversal of one ray (used where a thread owns its ray to the end).
// Closest hit: shrinks `ct` and sets `best` (triangle index).  Any hit (kAny):
// returns true at the first accepted triangle.
template <bool kAny>
__device__ __forceinline__ bool wide_traverse(const Ray& ray, const WideNode* __restrict__ wn,
                                              const WideTri* __restrict__ wt, uint32_t wlim, uint32_t tlim, float& ct,
                                              uint32_t& best, const WideStack& st, DeviceWords* words,
                                              uint32_t& nfetch, uint32_t& tfetch)
{
    WideRay s;
    wide_begin(s, ray, false);
    s.ct = ct;
    while (!wide_step<kAny>(s, wn, wt, wlim, tlim, st, words, nfetch, tfetch))
    {
    }
    const bool hit = kAny && s.best != kInvalid;
    if (s.best != kInvalid)
    {
        ct   = s.ct;
        best = s.best;
    }
    return hit;
}

}  // namespace rr
