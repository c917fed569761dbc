// rr_oracle.cpp -- CPU oracle for the RadeonRays BVH build + ray intersection path.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, in plain C++, the reference's
// Vulkan compute shaders for the LBVH build and the closest/any-hit traversal so
// that the CUDA kernels of the product can be checked against it bit for bit.
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load
// it; the product library never links or calls it.
//
// Floating-point rules (chosen once, used by the CUDA kernels too):
//   * IEEE binary32 + - * / with round-to-nearest; no contraction
//     (compiled with -ffp-contract=off); fmaf only where the shader writes fma
//     (vlk/kernels/common.h:157-158).
//   * dot(a,b) = (a.x*b.x + a.y*b.y) + a.z*b.z, cross as written.
//   * GLSL's min/max on floats -> fminf/fmaxf (identical for non-NaN inputs;
//     NaN Morton inputs map to 0).
// Pinning: tests compare this oracle with the reference's own CPU traversal
// (bvh_analyzer, compiled unmodified from the reference sources into
// oracle/_ref) and with the reference tests' structural checks
// (test/test_vk/hlbvh_test.h:69-100, test/test_vk/algos_test.h:372-378); the
// results are frozen as fixtures in tests/golden/.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "rr_oracle.h"

namespace
{
constexpr uint32_t kInvalid  = 0xffffffffu;
constexpr uint32_t kSentinel = 0xfffffffeu;  // isect_2l.comp:28

struct F3
{
    float x, y, z;
};
static inline F3 f3(float x, float y, float z) { return F3{x, y, z}; }
static inline F3 sub(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline F3 add(F3 a, F3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline F3 scl(float s, F3 a) { return f3(s * a.x, s * a.y, s * a.z); }
static inline F3 vmin(F3 a, F3 b) { return f3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }
static inline F3 vmax(F3 a, F3 b) { return f3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }
static inline float dot(F3 a, F3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline F3 cross(F3 a, F3 b)
{
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline F3 ld3(const float* p) { return f3(p[0], p[1], p[2]); }
static inline void st3(float* p, F3 v)
{
    p[0] = v.x;
    p[1] = v.y;
    p[2] = v.z;
}

struct Box
{
    F3 lo, hi;
};

// common.h:68-79 Float3ToUint3: order-preserving float -> uint map.
static inline uint32_t f2ord(float f)
{
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u ^ ((1u + ~(u >> 31)) | 0x80000000u);
}
// common.h:83-90 Uint3ToFloat3.
static inline float ord2f(uint32_t u)
{
    u ^= (((u >> 31) - 1u) | 0x80000000u);
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

// Vertex fetch: vertex_stride is in bytes (reference: >>2 floats).
struct Mesh
{
    const float*    v;
    uint64_t        stride_f;
    const void*     idx;
    int             idx16;
    uint32_t        ntri;
    inline uint32_t index(uint64_t k) const
    {
        return idx16 ? (uint32_t)((const uint16_t*)idx)[k] : ((const uint32_t*)idx)[k];
    }
    inline void tri(uint32_t t, F3& a, F3& b, F3& c) const
    {
        a = ld3(v + (uint64_t)index(3ull * t + 0) * stride_f);
        b = ld3(v + (uint64_t)index(3ull * t + 1) * stride_f);
        c = ld3(v + (uint64_t)index(3ull * t + 2) * stride_f);
    }
};

// common.h:241-248 calculate_aabb_for_triangle.
static inline Box tri_box(F3 a, F3 b, F3 c)
{
    Box r{a, a};
    r.lo = vmin(r.lo, b);
    r.hi = vmax(r.hi, b);
    r.lo = vmin(r.lo, c);
    r.hi = vmax(r.hi, c);
    return r;
}

// common.h:251-258 expand_bits.
static inline uint32_t expand_bits(uint32_t r)
{
    r = (r * 0x00010001u) & 0xFF0000FFu;
    r = (r * 0x00000101u) & 0x0F00F00Fu;
    r = (r * 0x00000011u) & 0xC30C30C3u;
    r = (r * 0x00000005u) & 0x49249249u;
    return r;
}
// 63-bit variant (21 bits per axis) used by the 63-bit key option.
static inline uint64_t expand_bits21(uint64_t v)
{
    v &= 0x1fffffull;
    v = (v | (v << 32)) & 0x1f00000000ffffull;
    v = (v | (v << 16)) & 0x1f0000ff0000ffull;
    v = (v | (v << 8)) & 0x100f00f00f00f00full;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}

// common.h:261-268 calculate_morton_code with clamp(NaN) := 0.
static inline float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
static inline uint32_t morton30(F3 p)
{
    const float s = 1024.0f;
    float       x = clampf(p.x * s, 0.0f, s - 1.0f);
    float       y = clampf(p.y * s, 0.0f, s - 1.0f);
    float       z = clampf(p.z * s, 0.0f, s - 1.0f);
    return (expand_bits((uint32_t)x) << 2) | (expand_bits((uint32_t)y) << 1) | expand_bits((uint32_t)z);
}
static inline uint64_t morton63(F3 p)
{
    const float s = 2097152.0f;
    float       x = clampf(p.x * s, 0.0f, s - 1.0f);
    float       y = clampf(p.y * s, 0.0f, s - 1.0f);
    float       z = clampf(p.z * s, 0.0f, s - 1.0f);
    return (expand_bits21((uint64_t)x) << 2) | (expand_bits21((uint64_t)y) << 1) | expand_bits21((uint64_t)z);
}

// lbvh_calc_morton_codes_mesh.comp:114-128: normalised centroid of the box.
static inline F3 norm_centroid(const Box& b, F3 mlo, F3 ext)
{
    F3 c = scl(0.5f, add(b.lo, b.hi));
    F3 d = sub(c, mlo);
    return f3(d.x / ext.x, d.y / ext.y, d.z / ext.z);
}

template <class F>
void parallel_for(uint64_t n, int threads, F&& f)
{
    if (threads <= 1 || n < 4096)
    {
        for (uint64_t i = 0; i < n; ++i) f(i);
        return;
    }
    std::atomic<uint64_t> next{0};
    const uint64_t        chunk = 1024;
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t)
        pool.emplace_back([&]() {
            for (;;)
            {
                uint64_t b = next.fetch_add(chunk);
                if (b >= n) break;
                uint64_t e = std::min(n, b + chunk);
                for (uint64_t i = b; i < e; ++i) f(i);
            }
        });
    for (auto& th : pool) th.join();
}

// ---- Karras emit (lbvh_emit_hierarchy_mesh.comp:78-217) ----------------------
// clz as the shader defines it: 32 - findMSB(v); findMSB(0) = -1, so clz(0) = 33.
static inline int clz_p1(uint32_t v)
{
    if (v == 0) return 33;
    int msb = 31;
    while (!(v >> msb)) --msb;
    return 32 - msb;
}
static inline int clz64_p1(uint64_t v)
{
    if (v == 0) return 65;
    int msb = 63;
    while (!(v >> msb)) --msb;
    return 64 - msb;
}

struct Emitter
{
    const uint32_t* codes32;
    const uint64_t* codes64;
    int64_t         n;

    // CalcCommonPrefixLength (:85-103); the 64-bit variant offsets the index
    // fallback by 64 instead of 32.
    inline int delta(int64_t i1, int64_t i2) const
    {
        int64_t l = std::min(i1, i2), r = std::max(i1, i2);
        if (l < 0 || r >= n) return 0;
        if (codes64)
        {
            uint64_t a = codes64[l], b = codes64[r];
            return a != b ? clz64_p1(a ^ b) : 64 + clz_p1((uint32_t)(l ^ r));
        }
        uint32_t a = codes32[l], b = codes32[r];
        return a != b ? clz_p1(a ^ b) : 32 + clz_p1((uint32_t)(l ^ r));
    }
    // FindSpan (:105-140).
    inline void span(int64_t i, int64_t& sx, int64_t& sy) const
    {
        int     dd   = delta(i, i + 1) - delta(i, i - 1);
        int64_t d    = dd > 0 ? 1 : (dd < 0 ? -1 : 0);
        int     dmin = delta(i, i - d);
        int64_t lmax = 2;
        while (delta(i, i + lmax * d) > dmin) lmax *= 2;
        int64_t l = 0, t = lmax;
        do
        {
            t /= 2;
            if (delta(i, i + (l + t) * d) > dmin) l += t;
        } while (t > 1);
        int64_t e = i + l * d;
        sx        = std::max<int64_t>(std::min(i, e), 0);
        sy        = std::min<int64_t>(std::max(i, e), n - 1);
    }
    // FindSplit (:142-168).
    inline int64_t split(int64_t left, int64_t right) const
    {
        int nid = delta(left, right);
        do
        {
            int64_t ns = (right + left) / 2;
            if (delta(left, ns) > nid)
                left = ns;
            else
                right = ns;
        } while (right > left + 1);
        return left;
    }
};

static void emit_tree(const uint32_t* codes32,
                      const uint64_t* codes64,
                      const uint32_t* sorted_idx,
                      uint32_t        n,
                      rro_node*       nodes,
                      int             threads)
{
    if (n == 0) return;
    Emitter em{codes32, codes64, (int64_t)n};
    // Leaves (:175-183): child0 = invalid, child1 = primitive, update = 0.
    for (uint32_t k = 0; k < n; ++k)
    {
        rro_node& L = nodes[n - 1 + k];
        L.child0    = kInvalid;
        L.child1    = sorted_idx[k];
        L.update    = 0;
    }
    // A single leaf is the root: the reference never writes its parent; this
    // build defines it as invalid.
    if (n == 1)
    {
        nodes[0].parent = kInvalid;
        return;
    }
    parallel_for(n - 1, threads, [&](uint64_t i) {
        int64_t sx, sy;
        em.span((int64_t)i, sx, sy);
        int64_t  s  = em.split(sx, sy);
        uint32_t al = (s == sx) ? (uint32_t)(n - 1 + s) : (uint32_t)s;
        uint32_t ar = (s + 1 == sy) ? (uint32_t)(n - 1 + s + 1) : (uint32_t)(s + 1);
        nodes[i].child0 = al;
        nodes[i].child1 = ar;
        nodes[i].update = 0;
        nodes[al].parent = (uint32_t)i;
        nodes[ar].parent = (uint32_t)i;
    });
    nodes[0].parent = kInvalid;
}

// lbvh_fit_aabb_mesh.comp:94-205 (the order of the climb does not change the
// result, so the oracle refits recursively from the leaves).
static inline Box node_box(const rro_node& nd)
{
    if (nd.child0 != kInvalid)
    {
        Box l{ld3(nd.aabb0_min_or_v0), ld3(nd.aabb0_max_or_v1)};
        Box r{ld3(nd.aabb1_min_or_v2), ld3(nd.aabb1_max_or_v3)};
        return Box{vmin(l.lo, r.lo), vmax(l.hi, r.hi)};
    }
    return tri_box(ld3(nd.aabb0_min_or_v0), ld3(nd.aabb0_max_or_v1), ld3(nd.aabb1_min_or_v2));
}

static void refit(rro_node* nodes, uint32_t n)
{
    if (n <= 1) return;
    // Post-order over internal nodes with an explicit stack.
    std::vector<std::pair<uint32_t, int>> st;
    st.reserve(128);
    st.push_back({0u, 0});
    while (!st.empty())
    {
        auto& top = st.back();
        rro_node& nd = nodes[top.first];
        if (top.second == 0)
        {
            top.second = 1;
            if (nodes[nd.child1].child0 != kInvalid) st.push_back({nd.child1, 0});
            if (nodes[nd.child0].child0 != kInvalid) st.push_back({nd.child0, 0});
            continue;
        }
        Box l = node_box(nodes[nd.child0]);
        Box r = node_box(nodes[nd.child1]);
        st3(nd.aabb0_min_or_v0, l.lo);
        st3(nd.aabb0_max_or_v1, l.hi);
        st3(nd.aabb1_min_or_v2, r.lo);
        st3(nd.aabb1_max_or_v3, r.hi);
        nd.update = 1;
        st.pop_back();
    }
}

// ---- traversal helpers (common.h:103-209) ------------------------------------
struct RayF
{
    F3    o;
    float tmin;
    F3    d;
    float tmax;
};
static inline RayF load_ray(const rro_ray& r)
{
    return RayF{ld3(r.origin), r.min_t, ld3(r.direction), r.max_t};
}
// mycopysign (common.h:166-169): b < 0 ? -a : a.
static inline float mycopysign(float a, float b) { return b < 0.f ? -a : a; }
// safe_invdir (common.h:172-183).
static inline F3 safe_invdir(F3 d)
{
    const float e = 1e-5f;
    return f3(1.0f / (fabsf(d.x) > e ? d.x : mycopysign(e, d.x)),
              1.0f / (fabsf(d.y) > e ? d.y : mycopysign(e, d.y)),
              1.0f / (fabsf(d.z) > e ? d.z : mycopysign(e, d.z)));
}
// fast_intersect_aabb (common.h:150-164); hit iff t0 <= t1.
static inline void isect_box(const float* lo, const float* hi, F3 inv, F3 oxi, float tmax_, float tmin_,
                             float& t0, float& t1)
{
    float fx = fmaf(hi[0], inv.x, oxi.x), fy = fmaf(hi[1], inv.y, oxi.y), fz = fmaf(hi[2], inv.z, oxi.z);
    float nx = fmaf(lo[0], inv.x, oxi.x), ny = fmaf(lo[1], inv.y, oxi.y), nz = fmaf(lo[2], inv.z, oxi.z);
    float ax = fmaxf(fx, nx), ay = fmaxf(fy, ny), az = fmaxf(fz, nz);
    float ix = fminf(fx, nx), iy = fminf(fy, ny), iz = fminf(fz, nz);
    t1 = fminf(fminf(az, fminf(ax, ay)), tmax_);
    t0 = fmaxf(fmaxf(iz, fmaxf(ix, iy)), tmin_);
}
// fast_intersect_triangle (common.h:103-137): returns t_max on a miss.
static inline float isect_tri(const RayF& r, F3 v1, F3 v2, F3 v3, float t_max)
{
    F3    e1    = sub(v2, v1);
    F3    e2    = sub(v3, v1);
    F3    s1    = cross(r.d, e2);
    float denom = dot(s1, e1);
    if (denom == 0.f) return t_max;
    float invd = 1.0f / denom;
    F3    d    = sub(r.o, v1);
    float b1   = dot(d, s1) * invd;
    F3    s2   = cross(d, e1);
    float b2   = dot(r.d, s2) * invd;
    float tmp  = dot(e2, s2) * invd;
    if (b1 < 0.0f || b1 > 1.0f || b2 < 0.0f || b1 + b2 > 1.0f || tmp < r.tmin || tmp > t_max) return t_max;
    return tmp;
}
// calculate_barycentrics (common.h:187-209).
static inline void barycentrics(F3 p, F3 v1, F3 v2, F3 v3, float& u, float& v)
{
    F3    e1  = sub(v2, v1);
    F3    e2  = sub(v3, v1);
    F3    e   = sub(p, v1);
    float d00 = dot(e1, e1), d01 = dot(e1, e2), d11 = dot(e2, e2), d20 = dot(e, e1), d21 = dot(e, e2);
    float den = d00 * d11 - d01 * d01;
    if (den == 0.f)
    {
        u = v = 0.f;
        return;
    }
    float inv = 1.0f / (d00 * d11 - d01 * d01);
    u         = (d11 * d20 - d01 * d21) * inv;
    v         = (d00 * d21 - d01 * d20) * inv;
}
static inline F3 hit_point(const RayF& r, float t) { return add(r.o, scl(t, r.d)); }

// transform_ray (common.h:310-324) with a row-major 3x4 matrix.
static inline RayF xform_ray(const float* m, RayF r)
{
    F3 o = f3(dot(ld3(m + 0), r.o) + m[3], dot(ld3(m + 4), r.o) + m[7], dot(ld3(m + 8), r.o) + m[11]);
    F3 d = f3(dot(ld3(m + 0), r.d), dot(ld3(m + 4), r.d), dot(ld3(m + 8), r.d));
    r.o  = o;
    r.d  = d;
    return r;
}

// Single-level traversal of one ray (isect.comp:105-245).  The shader's split
// 16-entry LDS stack + 64-entry global spill is a plain LIFO; the oracle uses a
// vector with the same push/pop order.
// Leaf of an AABB-list geometry (RR_PRIMITIVE_TYPE_AABB_LIST, which the
// reference declares but does not implement, radeonrays.cpp:286-289): the leaf
// holds its box as (min, max, max) in its three vertex slots.  The hit
// distance is the slab entry distance (clamped to min_t); a miss returns
// t_max.  Hit records of box leaves carry uv = (0, 0).
static inline float isect_leaf_box(const RayF& r, F3 inv, F3 oxi, const float* lo, const float* hi, float t_max)
{
    float t0, t1;
    isect_box(lo, hi, inv, oxi, t_max, r.tmin, t0, t1);
    return t0 <= t1 ? t0 : t_max;
}

// ---- the precise triangle test (this build's opt-in mode, no reference
// counterpart): the FP32 twin of csrc/trace_precise.cuh, operation for
// operation, so that the kernels' hits can be checked bit for bit.
//   decision: Woop, Benthin, Wald, "Watertight Ray/Triangle Intersection",
//     JCGT 2013 (shear to the ray, 2-D edge functions with exact signs);
//   t, u, v: exact input differences and compensated products (error-free
//     transformations: TwoSum, TwoProduct with fma), quotient corrected by
//     its exact remainder;
//   box test: Ize, "Robust BVH Ray Traversal", JCGT 2013 ((p - o) * (1 / d),
//     far distance moved outward by 2 gamma_3).
namespace precise
{
const float kRobustFar = 1.00000036f;
struct DF
{
    float h, l;
};
static inline DF two_sum(float a, float b)
{
    const float s = a + b, bb = s - a;
    return DF{s, (a - (s - bb)) + (b - bb)};
}
static inline DF two_diff(float a, float b)
{
    const float s = a - b, bb = s - a;
    return DF{s, (a - (s - bb)) - (b + bb)};
}
static inline DF fast_two_sum(float a, float b)
{
    const float s = a + b;
    return DF{s, b - (s - a)};
}
static inline DF two_prod(float a, float b)
{
    const float p = a * b;
    return DF{p, fmaf(a, b, -p)};
}
static inline float exact_sign_dop(float a, float b, float c, float d)
{
    const float p1 = a * b, p2 = c * d, r = p1 - p2;
    if (r != 0.0f) return r;
    return fmaf(a, b, -p1) - fmaf(c, d, -p2);
}
static inline DF df_dop(DF a, DF b, DF c, DF d)
{
    const DF    p = two_prod(a.h, b.h), q = two_prod(c.h, d.h), s = two_diff(p.h, q.h);
    const float lo = s.l + (p.l - q.l) + ((a.h * b.l + a.l * b.h) - (c.h * d.l + c.l * d.h));
    return fast_two_sum(s.h, lo);
}
static inline DF df_dot3(DF ax, DF ay, DF az, DF bx, DF by, DF bz)
{
    const DF    px = two_prod(ax.h, bx.h), py = two_prod(ay.h, by.h), pz = two_prod(az.h, bz.h);
    const DF    s1 = two_sum(px.h, py.h), s2 = two_sum(s1.h, pz.h);
    const float lx = px.l + (ax.h * bx.l + ax.l * bx.h);
    const float ly = py.l + (ay.h * by.l + ay.l * by.h);
    const float lz = pz.l + (az.h * bz.l + az.l * bz.h);
    return fast_two_sum(s2.h, ((s1.l + s2.l) + lx) + (ly + lz));
}
static inline DF df_div(DF n, DF d)
{
    const float q = n.h / d.h;
    const float r = fmaf(-q, d.h, n.h) + (n.l - q * d.l);
    return fast_two_sum(q, r / d.h);
}
struct Tri
{
    DF w[3], e1[3], e2[3], n[3];
};
static inline Tri setup(const RayF& r, F3 v0, F3 v1, F3 v2)
{
    Tri         p;
    const float o[3] = {r.o.x, r.o.y, r.o.z}, a[3] = {v0.x, v0.y, v0.z}, b[3] = {v1.x, v1.y, v1.z},
                c[3] = {v2.x, v2.y, v2.z};
    for (int k = 0; k < 3; ++k)
    {
        p.w[k]  = two_diff(a[k], o[k]);
        p.e1[k] = two_diff(b[k], a[k]);
        p.e2[k] = two_diff(c[k], a[k]);
    }
    p.n[0] = df_dop(p.e1[1], p.e2[2], p.e1[2], p.e2[1]);
    p.n[1] = df_dop(p.e1[2], p.e2[0], p.e1[0], p.e2[2]);
    p.n[2] = df_dop(p.e1[0], p.e2[1], p.e1[1], p.e2[0]);
    return p;
}
static inline DF t_of(const Tri& p, const RayF& r, bool& ok)
{
    const DF N = df_dot3(p.n[0], p.n[1], p.n[2], p.w[0], p.w[1], p.w[2]);
    const DF D = df_dot3(p.n[0], p.n[1], p.n[2], DF{r.d.x, 0.f}, DF{r.d.y, 0.f}, DF{r.d.z, 0.f});
    ok         = D.h != 0.0f;
    return ok ? df_div(N, D) : DF{0.f, 0.f};
}
// Watertight decision, then the accurate t; t_max on a miss.
static inline float isect_tri(const RayF& r, F3 v0, F3 v1, F3 v2, float t_max)
{
    const float adx = fabsf(r.d.x), ady = fabsf(r.d.y), adz = fabsf(r.d.z);
    const int   kz  = (adx >= ady && adx >= adz) ? 0 : (ady >= adz ? 1 : 2);
    int         kx = kz == 2 ? 0 : kz + 1, ky = kx == 2 ? 0 : kx + 1;
    const float d[3] = {r.d.x, r.d.y, r.d.z};
    if (d[kz] < 0.0f) std::swap(kx, ky);
    const float sx = d[kx] / d[kz], sy = d[ky] / d[kz];
    const float o[3] = {r.o.x, r.o.y, r.o.z};
    const float a[3] = {v0.x - o[0], v0.y - o[1], v0.z - o[2]};
    const float b[3] = {v1.x - o[0], v1.y - o[1], v1.z - o[2]};
    const float c[3] = {v2.x - o[0], v2.y - o[1], v2.z - o[2]};
    const float ax = a[kx] - sx * a[kz], ay = a[ky] - sy * a[kz];
    const float bx = b[kx] - sx * b[kz], by = b[ky] - sy * b[kz];
    const float cx = c[kx] - sx * c[kz], cy = c[ky] - sy * c[kz];
    const float U = exact_sign_dop(cx, by, cy, bx), V = exact_sign_dop(ax, cy, ay, cx), W = exact_sign_dop(bx, ay, by, ax);
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return t_max;
    if (U + V + W == 0.0f) return t_max;
    bool      ok;
    const Tri p = setup(r, v0, v1, v2);
    const DF  t = t_of(p, r, ok);
    if (!ok || !(t.h >= r.tmin) || t.h > t_max) return t_max;
    return t.h;
}
static inline void barycentrics(const RayF& r, F3 v0, F3 v1, F3 v2, float& u_out, float& v_out)
{
    u_out = v_out = 0.f;
    bool      ok;
    const Tri p = setup(r, v0, v1, v2);
    const DF  t = t_of(p, r, ok);
    if (!ok) return;
    const float dd[3] = {r.d.x, r.d.y, r.d.z};
    DF          q[3];
    for (int k = 0; k < 3; ++k)
    {
        const DF    pr = two_prod(t.h, dd[k]);
        const DF    s  = two_diff(pr.h, p.w[k].h);
        q[k]           = fast_two_sum(s.h, s.l + ((pr.l + t.l * dd[k]) - p.w[k].l));
    }
    const float an[3] = {fabsf(p.n[0].h), fabsf(p.n[1].h), fabsf(p.n[2].h)};
    int         ia, ib, in;
    if (an[2] >= an[0] && an[2] >= an[1])
        ia = 0, ib = 1, in = 2;
    else if (an[0] >= an[1])
        ia = 1, ib = 2, in = 0;
    else
        ia = 2, ib = 0, in = 1;
    const DF det = p.n[in];
    if (det.h == 0.0f) return;
    u_out = df_div(df_dop(q[ia], p.e2[ib], q[ib], p.e2[ia]), det).h;
    v_out = df_div(df_dop(p.e1[ia], q[ib], p.e1[ib], q[ia]), det).h;
}
static inline float robust_far(float t1) { return t1 * (t1 >= 0.0f ? kRobustFar : 2.0f - kRobustFar); }
static inline void isect_box(const float* lo, const float* hi, F3 inv, F3 o, float tmax_, float tmin_, float& t0,
                             float& t1)
{
    const float fx = (hi[0] - o.x) * inv.x, fy = (hi[1] - o.y) * inv.y, fz = (hi[2] - o.z) * inv.z;
    const float nx = (lo[0] - o.x) * inv.x, ny = (lo[1] - o.y) * inv.y, nz = (lo[2] - o.z) * inv.z;
    t1 = robust_far(fminf(fminf(fmaxf(fz, nz), fminf(fmaxf(fx, nx), fmaxf(fy, ny))), tmax_));
    t0 = fmaxf(fmaxf(fminf(fz, nz), fmaxf(fminf(fx, nx), fminf(fy, ny))), tmin_);
}
}  // namespace precise

// precise: the precise triangle test's traversal (same visit order, robust
// box test, precise triangle test and barycentrics); out_t (optional)
// receives the fp32 distance of the closest hit (+inf on a miss).
static void trace_one(const rro_node* nodes, const rro_ray& rr, int any, int full, void* hits, uint64_t gi,
                      uint64_t* fetches, int box_leaves = 0, int precise_test = 0, float* out_t = nullptr)
{
    RayF     r      = load_ray(rr);
    F3       inv    = precise_test ? f3(1.0f / r.d.x, 1.0f / r.d.y, 1.0f / r.d.z) : safe_invdir(r.d);
    F3       oxi    = f3(-r.o.x * inv.x, -r.o.y * inv.y, -r.o.z * inv.z);
    float    ct     = r.tmax;
    uint32_t caddr  = kInvalid;
    uint64_t nfetch = 0;
    uint32_t stack[256];
    int      sp   = 0;
    stack[sp++]   = kInvalid;
    uint32_t addr = 0;
    while (addr != kInvalid)
    {
        const rro_node& nd = nodes[addr];
        ++nfetch;
        if (nd.child0 != kInvalid)
        {
            float a0, a1, b0, b1;
            if (precise_test)
            {
                precise::isect_box(nd.aabb0_min_or_v0, nd.aabb0_max_or_v1, inv, r.o, ct, r.tmin, a0, a1);
                precise::isect_box(nd.aabb1_min_or_v2, nd.aabb1_max_or_v3, inv, r.o, ct, r.tmin, b0, b1);
            }
            else
            {
                isect_box(nd.aabb0_min_or_v0, nd.aabb0_max_or_v1, inv, oxi, ct, r.tmin, a0, a1);
                isect_box(nd.aabb1_min_or_v2, nd.aabb1_max_or_v3, inv, oxi, ct, r.tmin, b0, b1);
            }
            bool tc0 = a0 <= a1, tc1 = b0 <= b1;
            bool c1f = tc1 && (a0 > b0);
            if (tc0 || tc1)
            {
                uint32_t deferred;
                if (c1f || !tc0)
                {
                    addr     = nd.child1;
                    deferred = nd.child0;
                }
                else
                {
                    addr     = nd.child0;
                    deferred = nd.child1;
                }
                if (tc0 && tc1 && sp < 256) stack[sp++] = deferred;
                continue;
            }
        }
        else
        {
            float t = box_leaves     ? isect_leaf_box(r, inv, oxi, nd.aabb0_min_or_v0, nd.aabb0_max_or_v1, ct)
                      : precise_test ? precise::isect_tri(r, ld3(nd.aabb0_min_or_v0), ld3(nd.aabb0_max_or_v1),
                                                          ld3(nd.aabb1_min_or_v2), ct)
                                     : isect_tri(r, ld3(nd.aabb0_min_or_v0), ld3(nd.aabb0_max_or_v1),
                                                 ld3(nd.aabb1_min_or_v2), ct);
            if (t < ct)
            {
                if (!any)
                {
                    ct    = t;
                    caddr = addr;
                }
                else
                {
                    if (full)
                    {
                        rro_hit& h = ((rro_hit*)hits)[gi];
                        if (box_leaves)
                            h.uv[0] = h.uv[1] = 0.f;
                        else if (precise_test)
                            precise::barycentrics(r, ld3(nd.aabb0_min_or_v0), ld3(nd.aabb0_max_or_v1),
                                                  ld3(nd.aabb1_min_or_v2), h.uv[0], h.uv[1]);
                        else
                            barycentrics(hit_point(r, t), ld3(nd.aabb0_min_or_v0), ld3(nd.aabb0_max_or_v1),
                                         ld3(nd.aabb1_min_or_v2), h.uv[0], h.uv[1]);
                        h.prim_id = nd.child1;
                        h.inst_id = 0;
                    }
                    else
                        ((uint32_t*)hits)[gi] = nd.child1;
                    if (fetches) fetches[gi] = nfetch;
                    if (out_t) out_t[gi] = t;
                    return;
                }
            }
        }
        addr = stack[--sp];
    }
    if (out_t) out_t[gi] = caddr != kInvalid ? ct : INFINITY;
    if (caddr != kInvalid)
    {
        const rro_node& nd = nodes[caddr];
        if (full)
        {
            rro_hit& h = ((rro_hit*)hits)[gi];
            if (box_leaves)
                h.uv[0] = h.uv[1] = 0.f;
            else if (precise_test)
                precise::barycentrics(r, ld3(nd.aabb0_min_or_v0), ld3(nd.aabb0_max_or_v1), ld3(nd.aabb1_min_or_v2),
                                      h.uv[0], h.uv[1]);
            else
                barycentrics(hit_point(r, ct), ld3(nd.aabb0_min_or_v0), ld3(nd.aabb0_max_or_v1),
                             ld3(nd.aabb1_min_or_v2), h.uv[0], h.uv[1]);
            h.prim_id = nd.child1;
            h.inst_id = 0;
        }
        else
            ((uint32_t*)hits)[gi] = nd.child1;
    }
    else
    {
        if (full)
            ((rro_hit*)hits)[gi].inst_id = kInvalid;
        else
            ((uint32_t*)hits)[gi] = kInvalid;
    }
    if (fetches) fetches[gi] = nfetch;
}

// Two-level traversal of one ray (isect_2l.comp:136-323).
static void trace_scene_one(const rro_node*         tlas,
                            const float*            xforms,
                            const rro_node* const*  blas,
                            const rro_ray&          rr,
                            int                     any,
                            int                     full,
                            void*                   hits,
                            uint64_t                gi)
{
    const RayF world = load_ray(rr);
    RayF       r     = world;
    F3         inv   = safe_invdir(r.d);
    F3         oxi   = f3(-r.o.x * inv.x, -r.o.y * inv.y, -r.o.z * inv.z);
    float      ct    = r.tmax;
    uint32_t   caddr = kInvalid, cinst = kInvalid, cprim = kInvalid, inst = kInvalid;
    std::vector<uint32_t> stack;
    stack.reserve(64);
    stack.push_back(kInvalid);
    uint32_t addr = 0;
    while (addr != kInvalid)
    {
        const rro_node& nd = (inst == kInvalid) ? tlas[addr] : blas[inst][addr];
        bool            popped = false;
        if (nd.child0 != kInvalid)
        {
            float a0, a1, b0, b1;
            isect_box(nd.aabb0_min_or_v0, nd.aabb0_max_or_v1, inv, oxi, ct, r.tmin, a0, a1);
            isect_box(nd.aabb1_min_or_v2, nd.aabb1_max_or_v3, inv, oxi, ct, r.tmin, b0, b1);
            bool tc0 = a0 <= a1, tc1 = b0 <= b1;
            bool c1f = tc1 && (a0 > b0);
            if (tc0 || tc1)
            {
                uint32_t deferred;
                if (c1f || !tc0)
                {
                    addr     = nd.child1;
                    deferred = nd.child0;
                }
                else
                {
                    addr     = nd.child0;
                    deferred = nd.child1;
                }
                if (tc0 && tc1) stack.push_back(deferred);
                continue;
            }
        }
        else if (inst == kInvalid)
        {
            // A TLAS leaf whose BLAS is empty (null here) is a miss; the
            // reference would traverse an undefined buffer.
            if (blas[nd.child1] != nullptr)
            {
                inst = nd.child1;
                r    = xform_ray(xforms + 24ull * inst, r);
                inv  = safe_invdir(r.d);
                oxi  = f3(-r.o.x * inv.x, -r.o.y * inv.y, -r.o.z * inv.z);
                stack.push_back(kSentinel);
                addr = 0;
                continue;
            }
        }
        else
        {
            float t = isect_tri(r, ld3(nd.aabb0_min_or_v0), ld3(nd.aabb0_max_or_v1), ld3(nd.aabb1_min_or_v2), ct);
            if (t < ct)
            {
                if (!any)
                {
                    ct    = t;
                    caddr = addr;
                    cprim = nd.child1;
                    cinst = inst;
                }
                else
                {
                    if (full)
                    {
                        rro_hit& h = ((rro_hit*)hits)[gi];
                        barycentrics(hit_point(r, t), ld3(nd.aabb0_min_or_v0), ld3(nd.aabb0_max_or_v1),
                                     ld3(nd.aabb1_min_or_v2), h.uv[0], h.uv[1]);
                        h.prim_id = nd.child1;
                        h.inst_id = inst;
                    }
                    else
                        ((uint32_t*)hits)[gi] = inst;
                    return;
                }
            }
        }
        (void)popped;
        addr = stack.back();
        stack.pop_back();
        if (addr == kSentinel)
        {
            inst = kInvalid;
            r    = world;
            inv  = safe_invdir(r.d);
            oxi  = f3(-r.o.x * inv.x, -r.o.y * inv.y, -r.o.z * inv.z);
            addr = stack.back();
            stack.pop_back();
        }
    }
    if (caddr != kInvalid)
    {
        if (full)
        {
            const rro_node& nd = blas[cinst][caddr];
            RayF            lr = xform_ray(xforms + 24ull * cinst, world);
            rro_hit&        h  = ((rro_hit*)hits)[gi];
            barycentrics(hit_point(lr, ct), ld3(nd.aabb0_min_or_v0), ld3(nd.aabb0_max_or_v1), ld3(nd.aabb1_min_or_v2),
                         h.uv[0], h.uv[1]);
            h.prim_id = cprim;
            h.inst_id = cinst;
        }
        else
            ((uint32_t*)hits)[gi] = cinst;
    }
    else
    {
        if (full)
            ((rro_hit*)hits)[gi].inst_id = kInvalid;
        else
            ((uint32_t*)hits)[gi] = kInvalid;
    }
}

// 3x4 affine inverse in double, rounded once to float (this build's
// replacement for GLSL inverse() in lbvh_fit_aabb_scene.comp:118).
static void inverse34(const float* m, float* out)
{
    double a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[6], g = m[8], h = m[9], i = m[10];
    double A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;
    double det = a * A + b * B + c * C;
    double inv[9];
    if (det == 0.0)
    {
        for (int k = 0; k < 12; ++k) out[k] = 0.f;
        return;
    }
    double r = 1.0 / det;
    inv[0]   = A * r;
    inv[1]   = -(b * i - c * h) * r;
    inv[2]   = (b * f - c * e) * r;
    inv[3]   = B * r;
    inv[4]   = (a * i - c * g) * r;
    inv[5]   = -(a * f - c * d) * r;
    inv[6]   = C * r;
    inv[7]   = -(a * h - b * g) * r;
    inv[8]   = (a * e - b * d) * r;
    double tx = m[3], ty = m[7], tz = m[11];
    for (int row = 0; row < 3; ++row)
    {
        out[row * 4 + 0] = (float)inv[row * 3 + 0];
        out[row * 4 + 1] = (float)inv[row * 3 + 1];
        out[row * 4 + 2] = (float)inv[row * 3 + 2];
        out[row * 4 + 3] = (float)(-(inv[row * 3 + 0] * tx + inv[row * 3 + 1] * ty + inv[row * 3 + 2] * tz));
    }
}

// Instance box: the BLAS root box carried through all 8 corners of the
// transform.  (The reference's transform_aabb, common.h:280-308, drops the
// corner (max.x, min.y, min.z); this build uses all eight.)
static inline F3 xform_point(const float* m, F3 p)
{
    return f3(dot(ld3(m + 0), p) + m[3], dot(ld3(m + 4), p) + m[7], dot(ld3(m + 8), p) + m[11]);
}
static Box xform_box(const float* m, Box b)
{
    Box r;
    for (int k = 0; k < 8; ++k)
    {
        F3 p = f3((k & 4) ? b.hi.x : b.lo.x, (k & 2) ? b.hi.y : b.lo.y, (k & 1) ? b.hi.z : b.lo.z);
        F3 q = xform_point(m, p);
        if (k == 0)
            r = Box{q, q};
        else
        {
            r.lo = vmin(r.lo, q);
            r.hi = vmax(r.hi, q);
        }
    }
    return r;
}

// Stable LSD radix sort of (key, value) pairs by key, 8-bit digits.
template <class K>
static void stable_sort_kv(const K* keys, uint32_t n, K* out_keys, uint32_t* out_vals, const uint32_t* in_vals)
{
    std::vector<K>        k0(keys, keys + n), k1(n);
    std::vector<uint32_t> v0(n), v1(n);
    for (uint32_t i = 0; i < n; ++i) v0[i] = in_vals ? in_vals[i] : i;
    K any = 0;
    for (uint32_t i = 0; i < n; ++i) any |= keys[i];
    for (int shift = 0; shift < (int)(8 * sizeof(K)); shift += 8)
    {
        if (((any >> shift) & 0xff) == 0 && shift > 0) continue;
        uint32_t cnt[257] = {0};
        for (uint32_t i = 0; i < n; ++i) cnt[((k0[i] >> shift) & 0xff) + 1]++;
        for (int b = 0; b < 256; ++b) cnt[b + 1] += cnt[b];
        for (uint32_t i = 0; i < n; ++i)
        {
            uint32_t p = cnt[(k0[i] >> shift) & 0xff]++;
            k1[p]      = k0[i];
            v1[p]      = v0[i];
        }
        k0.swap(k1);
        v0.swap(v1);
    }
    std::memcpy(out_keys, k0.data(), sizeof(K) * n);
    std::memcpy(out_vals, v0.data(), sizeof(uint32_t) * n);
}

}  // namespace

extern "C" {

int rro_version(void) { return 1; }

// lbvh_calc_mesh_aabb.comp:121-179 as an exact min/max over every vertex of
// every triangle, in the order-preserving uint encoding ([0..2] min, [4..6]
// max, [3] and [7] unused and zero).
void rro_mesh_aabb(const float* vertices, uint32_t vertex_stride, const void* indices, int index16, uint32_t ntri,
                   uint32_t out[8])
{
    Mesh m{vertices, vertex_stride >> 2, indices, index16, ntri};
    uint32_t lo[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, hi[3] = {0, 0, 0};
    for (uint32_t t = 0; t < ntri; ++t)
    {
        F3 a, b, c;
        m.tri(t, a, b, c);
        Box bx = tri_box(a, b, c);
        const float l[3] = {bx.lo.x, bx.lo.y, bx.lo.z}, h[3] = {bx.hi.x, bx.hi.y, bx.hi.z};
        for (int k = 0; k < 3; ++k)
        {
            lo[k] = std::min(lo[k], f2ord(l[k]));
            hi[k] = std::max(hi[k], f2ord(h[k]));
        }
    }
    out[0] = lo[0];
    out[1] = lo[1];
    out[2] = lo[2];
    out[3] = 0;
    out[4] = hi[0];
    out[5] = hi[1];
    out[6] = hi[2];
    out[7] = 0;
}

// lbvh_calc_morton_codes_mesh.comp:78-130.  bits = 30 (uint32 codes) or 63
// (uint64 codes).
void rro_morton(const float* vertices, uint32_t vertex_stride, const void* indices, int index16, uint32_t ntri,
                const uint32_t aabb[8], int bits, void* codes)
{
    Mesh m{vertices, vertex_stride >> 2, indices, index16, ntri};
    F3   mlo = f3(ord2f(aabb[0]), ord2f(aabb[1]), ord2f(aabb[2]));
    F3   mhi = f3(ord2f(aabb[4]), ord2f(aabb[5]), ord2f(aabb[6]));
    F3   ext = sub(mhi, mlo);
    for (uint32_t t = 0; t < ntri; ++t)
    {
        F3 a, b, c;
        m.tri(t, a, b, c);
        F3 p = norm_centroid(tri_box(a, b, c), mlo, ext);
        if (bits == 63)
            ((uint64_t*)codes)[t] = morton63(p);
        else
            ((uint32_t*)codes)[t] = morton30(p);
    }
}

// Stable key/value sort (semantics of vlk/radix_sort.cpp:157-338): values are
// the original positions 0..n-1.
void rro_sort32(const uint32_t* codes, uint32_t n, uint32_t* sorted_codes, uint32_t* sorted_idx)
{
    stable_sort_kv<uint32_t>(codes, n, sorted_codes, sorted_idx, nullptr);
}
void rro_sort64(const uint64_t* codes, uint32_t n, uint64_t* sorted_codes, uint32_t* sorted_idx)
{
    stable_sort_kv<uint64_t>(codes, n, sorted_codes, sorted_idx, nullptr);
}

// Karras topology (lbvh_emit_hierarchy_mesh.comp:170-217).
void rro_emit(const void* sorted_codes, int bits, const uint32_t* sorted_idx, uint32_t n, rro_node* nodes, int threads)
{
    emit_tree(bits == 63 ? nullptr : (const uint32_t*)sorted_codes, bits == 63 ? (const uint64_t*)sorted_codes : nullptr,
              sorted_idx, n, nodes, threads);
}

// Treelet restructure (the reference's optional quality pass,
// restructure_hlbvh.cpp:133-278 + restructure_bvh.comp, after Karras & Aila
// 2013), restated deterministically: in post-order, every internal node X
// whose subtree holds at least `min_prims` triangles roots a treelet of up to
// 7 subtrees (grown by splitting the treelet leaf with the largest surface
// area, first on ties), the topology of its internal nodes is replaced by the
// one minimising the sum of node half-areas (dynamic programming over the 127
// subsets, first minimum in enumeration order), if strictly cheaper, and the
// treelet's boxes are refitted.  Node slots are reused, so the layout (root 0,
// internal [0, n-2], leaves [n-1, 2n-2]) is kept.
} // extern "C"

static inline float half_area(const Box& b)
{
    const F3 e = sub(b.hi, b.lo);
    return (e.x * e.y + e.y * e.z) + e.z * e.x;
}

static inline Box box_union(const Box& a, const Box& b) { return Box{vmin(a.lo, b.lo), vmax(a.hi, b.hi)}; }

static void set_child_boxes(rro_node* nodes, uint32_t x)
{
    rro_node& nd = nodes[x];
    const Box l  = node_box(nodes[nd.child0]);
    const Box r  = node_box(nodes[nd.child1]);
    st3(nd.aabb0_min_or_v0, l.lo);
    st3(nd.aabb0_max_or_v1, l.hi);
    st3(nd.aabb1_min_or_v2, r.lo);
    st3(nd.aabb1_max_or_v3, r.hi);
}

// Restructure the treelet rooted at internal node x; returns true if changed.
static bool restructure_treelet(rro_node* nodes, uint32_t n, uint32_t x)
{
    uint32_t leaf[7], inner[6];
    float    la[7];
    int      nl = 2, ni = 1;
    inner[0]    = x;
    leaf[0]     = nodes[x].child0;
    leaf[1]     = nodes[x].child1;
    la[0]       = half_area(node_box(nodes[leaf[0]]));
    la[1]       = half_area(node_box(nodes[leaf[1]]));
    while (nl < 7)
    {
        int   best = -1;
        float ba   = -1.f;
        for (int k = 0; k < nl; ++k)
            if (leaf[k] < n - 1 && la[k] > ba)
            {
                ba   = la[k];
                best = k;
            }
        if (best < 0) break;
        const uint32_t c = leaf[best];
        inner[ni++]      = c;
        leaf[best]       = nodes[c].child0;
        la[best]         = half_area(node_box(nodes[leaf[best]]));
        leaf[nl]         = nodes[c].child1;
        la[nl]           = half_area(node_box(nodes[leaf[nl]]));
        ++nl;
    }
    if (nl < 3) return false;
    const uint32_t full = (1u << nl) - 1;
    Box            bx[7];
    for (int k = 0; k < nl; ++k) bx[k] = node_box(nodes[leaf[k]]);
    float   area[128], cost[128];
    uint8_t part[128];
    for (uint32_t s = 1; s <= full; ++s)
    {
        const int lo = __builtin_ctz(s);
        Box       u  = bx[lo];
        for (int k = lo + 1; k < nl; ++k)
            if (s >> k & 1u) u = box_union(u, bx[k]);
        area[s] = half_area(u);
        if ((s & (s - 1)) == 0)
        {
            cost[s] = area[s];
            part[s] = 0;
            continue;
        }
        // Proper subsets p of s holding s's lowest bit, in decreasing order.
        const uint32_t low  = s & (0u - s);
        float          best = 0.f;
        uint32_t       bp   = 0;
        for (uint32_t p = (s - 1) & s; p; p = (p - 1) & s)
        {
            if (!(p & low)) continue;
            const float c = cost[p] + cost[s ^ p];
            if (bp == 0 || c < best)
            {
                best = c;
                bp   = p;
            }
        }
        cost[s] = area[s] + best;
        part[s] = (uint8_t)bp;
    }
    // Cost of the current topology: every treelet node's half-area.
    float cur = area[full];
    for (int k = 1; k < ni; ++k) cur += half_area(node_box(nodes[inner[k]]));
    for (int k = 0; k < nl; ++k) cur += la[k];
    if (!(cost[full] < cur)) return false;
    // Rebuild top-down in preorder; internal slots are reused in inner[] order.
    uint32_t sset[6], sslot[6];
    int      sp = 0, next = 1;
    sset[sp]    = full;
    sslot[sp++] = x;
    uint32_t order[6];
    int      no = 0;
    while (sp > 0)
    {
        --sp;
        const uint32_t s = sset[sp], slot = sslot[sp];
        order[no++]      = slot;
        const uint32_t p = part[s], q = s ^ p;
        uint32_t       ch[2];
        const uint32_t sides[2] = {p, q};
        for (int k = 0; k < 2; ++k)
        {
            const uint32_t t = sides[k];
            if ((t & (t - 1)) == 0)
                ch[k] = leaf[__builtin_ctz(t)];
            else
            {
                ch[k]       = inner[next++];
                sset[sp]    = t;
                sslot[sp++] = ch[k];
            }
        }
        nodes[slot].child0   = ch[0];
        nodes[slot].child1   = ch[1];
        nodes[ch[0]].parent = slot;
        nodes[ch[1]].parent = slot;
    }
    for (int k = no - 1; k >= 0; --k) set_child_boxes(nodes, order[k]);
    return true;
}

extern "C" {

uint32_t rro_restructure(rro_node* nodes, uint32_t n, uint32_t min_prims, int passes)
{
    if (n < 3) return 0;
    uint32_t              changed = 0;
    std::vector<uint32_t> cnt(2 * (size_t)n - 1, 1u);
    for (int pass = 0; pass < passes; ++pass)
    {
        // Post-order over internal nodes (children before parents).
        std::vector<std::pair<uint32_t, int>> st;
        st.push_back({0u, 0});
        while (!st.empty())
        {
            auto& top = st.back();
            const uint32_t x = top.first;
            if (top.second == 0)
            {
                top.second = 1;
                const uint32_t c0 = nodes[x].child0, c1 = nodes[x].child1;
                if (c1 < n - 1) st.push_back({c1, 0});
                if (c0 < n - 1) st.push_back({c0, 0});
                continue;
            }
            st.pop_back();
            cnt[x] = cnt[nodes[x].child0] + cnt[nodes[x].child1];
            if (cnt[x] >= min_prims && restructure_treelet(nodes, n, x)) ++changed;
        }
    }
    return changed;
}

// Leaf vertices + bottom-up boxes (lbvh_fit_aabb_mesh.comp:94-205).
void rro_fit(const float* vertices, uint32_t vertex_stride, const void* indices, int index16, uint32_t n,
             rro_node* nodes)
{
    Mesh m{vertices, vertex_stride >> 2, indices, index16, n};
    for (uint32_t k = 0; k < n; ++k)
    {
        rro_node& L = nodes[n - 1 + k];
        F3        a, b, c;
        m.tri(L.child1, a, b, c);
        st3(L.aabb0_min_or_v0, a);
        st3(L.aabb0_max_or_v1, b);
        st3(L.aabb1_min_or_v2, c);
        st3(L.aabb1_max_or_v3, f3(0.f, 0.f, 0.f));
    }
    refit(nodes, n);
}

// Whole mesh build: nodes must hold max(2n-1, 0) entries.
void rro_build_mesh(const float* vertices, uint32_t vertex_stride, const void* indices, int index16, uint32_t n,
                    int bits, rro_node* nodes, uint32_t* out_sorted_idx, void* out_sorted_codes, int threads)
{
    if (n == 0) return;
    uint32_t aabb[8];
    rro_mesh_aabb(vertices, vertex_stride, indices, index16, n, aabb);
    std::vector<uint32_t> idx(n);
    if (bits == 63)
    {
        std::vector<uint64_t> c(n), sc(n);
        rro_morton(vertices, vertex_stride, indices, index16, n, aabb, 63, c.data());
        rro_sort64(c.data(), n, sc.data(), idx.data());
        std::memset(nodes, 0, sizeof(rro_node) * (2ull * n - 1));
        rro_emit(sc.data(), 63, idx.data(), n, nodes, threads);
        if (out_sorted_codes) std::memcpy(out_sorted_codes, sc.data(), 8ull * n);
    }
    else
    {
        std::vector<uint32_t> c(n), sc(n);
        rro_morton(vertices, vertex_stride, indices, index16, n, aabb, 30, c.data());
        rro_sort32(c.data(), n, sc.data(), idx.data());
        std::memset(nodes, 0, sizeof(rro_node) * (2ull * n - 1));
        rro_emit(sc.data(), 30, idx.data(), n, nodes, threads);
        if (out_sorted_codes) std::memcpy(out_sorted_codes, sc.data(), 4ull * n);
    }
    if (out_sorted_idx) std::memcpy(out_sorted_idx, idx.data(), 4ull * n);
    rro_fit(vertices, vertex_stride, indices, index16, n, nodes);
}

// isect.comp semantics.  query: 0 closest, 1 any.  output: 0 full RRHit
// (16 B), 1 instance-id (uint32; the single-level kernel writes the primitive
// id there, isect.comp:197,235).  An empty geometry (n_nodes == 0) misses.
// fetches (optional): node fetches per ray.
void rro_trace_leaves(const rro_node* nodes, uint32_t n_nodes, const rro_ray* rays, uint32_t nrays, int query,
                      int output, void* hits, uint64_t* fetches, int threads, int box_leaves)
{
    const int any = query == 1, full = output == 0;
    parallel_for(nrays, threads, [&](uint64_t i) {
        if (n_nodes == 0)
        {
            if (full)
                ((rro_hit*)hits)[i].inst_id = kInvalid;
            else
                ((uint32_t*)hits)[i] = kInvalid;
            if (fetches) fetches[i] = 0;
            return;
        }
        trace_one(nodes, rays[i], any, full, hits, i, fetches, box_leaves);
    });
}

void rro_trace(const rro_node* nodes, uint32_t n_nodes, const rro_ray* rays, uint32_t nrays, int query, int output,
               void* hits, uint64_t* fetches, int threads)
{
    const int any = query == 1, full = output == 0;
    parallel_for(nrays, threads, [&](uint64_t i) {
        if (n_nodes == 0)
        {
            if (full)
                ((rro_hit*)hits)[i].inst_id = kInvalid;
            else
                ((uint32_t*)hits)[i] = kInvalid;
            if (fetches) fetches[i] = 0;
            return;
        }
        trace_one(nodes, rays[i], any, full, hits, i, fetches);
    });
}

// TLAS build (lbvh_*_scene.comp).  blas_roots[i] = root node of instance i's
// BLAS; blas_leaf_counts[i] its triangle count.  transforms: 12 floats per
// instance (row-major object->world).  out_nodes: 2*count-1 nodes;
// out_xforms: 24 floats per instance ([inverse, forward], fit_aabb_scene:118-119).
void rro_build_scene(const rro_node* const* blas_roots, const uint32_t* blas_leaf_counts, const float* transforms,
                     uint32_t count, rro_node* out_nodes, float* out_xforms)
{
    if (count == 0) return;
    std::vector<Box> ib(count);
    uint32_t         lo[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, hi[3] = {0, 0, 0};
    for (uint32_t i = 0; i < count; ++i)
    {
        const rro_node& root = *blas_roots[i];
        Box             b;
        if (blas_leaf_counts[i] == 0)
            b = Box{f3(0, 0, 0), f3(0, 0, 0)};
        else
            b = node_box(root);
        ib[i]            = xform_box(transforms + 12ull * i, b);
        const float l[3] = {ib[i].lo.x, ib[i].lo.y, ib[i].lo.z}, h[3] = {ib[i].hi.x, ib[i].hi.y, ib[i].hi.z};
        for (int k = 0; k < 3; ++k)
        {
            lo[k] = std::min(lo[k], f2ord(l[k]));
            hi[k] = std::max(hi[k], f2ord(h[k]));
        }
        inverse34(transforms + 12ull * i, out_xforms + 24ull * i);
        std::memcpy(out_xforms + 24ull * i + 12, transforms + 12ull * i, 48);
    }
    F3                    mlo = f3(ord2f(lo[0]), ord2f(lo[1]), ord2f(lo[2]));
    F3                    ext = sub(f3(ord2f(hi[0]), ord2f(hi[1]), ord2f(hi[2])), mlo);
    std::vector<uint32_t> codes(count), sc(count), idx(count);
    for (uint32_t i = 0; i < count; ++i) codes[i] = morton30(norm_centroid(ib[i], mlo, ext));
    stable_sort_kv<uint32_t>(codes.data(), count, sc.data(), idx.data(), nullptr);
    std::memset(out_nodes, 0, sizeof(rro_node) * (2ull * count - 1));
    emit_tree(sc.data(), nullptr, idx.data(), count, out_nodes, 1);
    for (uint32_t k = 0; k < count; ++k)
    {
        rro_node& L = out_nodes[count - 1 + k];
        const Box& b = ib[L.child1];
        st3(L.aabb0_min_or_v0, b.lo);
        st3(L.aabb0_max_or_v1, b.hi);
        st3(L.aabb1_min_or_v2, b.lo);
        st3(L.aabb1_max_or_v3, b.hi);
    }
    // Internal boxes: union of both slots of each child (fit_aabb_scene:87-97).
    if (count > 1)
    {
        std::vector<std::pair<uint32_t, int>> st;
        st.push_back({0u, 0});
        auto slots_box = [&](const rro_node& nd) {
            Box l{ld3(nd.aabb0_min_or_v0), ld3(nd.aabb0_max_or_v1)};
            Box r{ld3(nd.aabb1_min_or_v2), ld3(nd.aabb1_max_or_v3)};
            return Box{vmin(l.lo, r.lo), vmax(l.hi, r.hi)};
        };
        while (!st.empty())
        {
            auto&     top = st.back();
            rro_node& nd  = out_nodes[top.first];
            if (top.second == 0)
            {
                top.second = 1;
                if (out_nodes[nd.child1].child0 != kInvalid) st.push_back({nd.child1, 0});
                if (out_nodes[nd.child0].child0 != kInvalid) st.push_back({nd.child0, 0});
                continue;
            }
            Box l = slots_box(out_nodes[nd.child0]);
            Box r = slots_box(out_nodes[nd.child1]);
            st3(nd.aabb0_min_or_v0, l.lo);
            st3(nd.aabb0_max_or_v1, l.hi);
            st3(nd.aabb1_min_or_v2, r.lo);
            st3(nd.aabb1_max_or_v3, r.hi);
            nd.update = 1;
            st.pop_back();
        }
    }
}

// Two-level traversal (isect_2l.comp); output 1 writes the instance id.
void rro_trace_scene(const rro_node* tlas, const float* xforms, const rro_node* const* blas, const rro_ray* rays,
                     uint32_t nrays, int query, int output, void* hits, int threads)
{
    const int any = query == 1, full = output == 0;
    parallel_for(nrays, threads,
                 [&](uint64_t i) { trace_scene_one(tlas, xforms, blas, rays[i], any, full, hits, i); });
}

// FP64 twin of the triangle test + barycentrics on a given triangle: the exact
// (double) intersection of ray i with the triangle of prim[i] (vertices tri[i*9..]).
// Writes t, u, v in double; rays whose prim is invalid are skipped.
void rro_fp64_hit(const rro_ray* rays, const float* tri9, const uint32_t* valid, uint32_t nrays, double* out_tuv)
{
    for (uint32_t i = 0; i < nrays; ++i)
    {
        if (!valid[i]) continue;
        const float* v  = tri9 + 9ull * i;
        double       o[3] = {rays[i].origin[0], rays[i].origin[1], rays[i].origin[2]};
        double       d[3] = {rays[i].direction[0], rays[i].direction[1], rays[i].direction[2]};
        double       a[3] = {v[0], v[1], v[2]}, b[3] = {v[3], v[4], v[5]}, c[3] = {v[6], v[7], v[8]};
        double       e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
        double       e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
        double       s1[3] = {d[1] * e2[2] - d[2] * e2[1], d[2] * e2[0] - d[0] * e2[2], d[0] * e2[1] - d[1] * e2[0]};
        double       den   = s1[0] * e1[0] + s1[1] * e1[1] + s1[2] * e1[2];
        double       dd[3] = {o[0] - a[0], o[1] - a[1], o[2] - a[2]};
        double       s2[3] = {dd[1] * e1[2] - dd[2] * e1[1], dd[2] * e1[0] - dd[0] * e1[2], dd[0] * e1[1] - dd[1] * e1[0]};
        double       t     = (e2[0] * s2[0] + e2[1] * s2[1] + e2[2] * s2[2]) / den;
        double       p[3]  = {o[0] + t * d[0], o[1] + t * d[1], o[2] + t * d[2]};
        double       e[3]  = {p[0] - a[0], p[1] - a[1], p[2] - a[2]};
        double       d00 = e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2];
        double       d01 = e1[0] * e2[0] + e1[1] * e2[1] + e1[2] * e2[2];
        double       d11 = e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2];
        double       d20 = e[0] * e1[0] + e[1] * e1[1] + e[2] * e1[2];
        double       d21 = e[0] * e2[0] + e[1] * e2[1] + e[2] * e2[2];
        double       q   = d00 * d11 - d01 * d01;
        out_tuv[3ull * i + 0] = t;
        out_tuv[3ull * i + 1] = q != 0.0 ? (d11 * d20 - d01 * d21) / q : 0.0;
        out_tuv[3ull * i + 2] = q != 0.0 ? (d00 * d21 - d01 * d20) / q : 0.0;
    }
}

// FP32 t of the closest hit per ray (same arithmetic as rro_trace): used to
// report t error against rro_fp64_hit.  Writes +inf on a miss.
void rro_trace_t(const rro_node* nodes, uint32_t n_nodes, const rro_ray* rays, uint32_t nrays, float* out_t,
                 int threads)
{
    parallel_for(nrays, threads, [&](uint64_t gi) {
        out_t[gi] = INFINITY;
        if (n_nodes == 0) return;
        RayF     r   = load_ray(rays[gi]);
        F3       inv = safe_invdir(r.d);
        F3       oxi = f3(-r.o.x * inv.x, -r.o.y * inv.y, -r.o.z * inv.z);
        float    ct  = r.tmax;
        bool     hit = false;
        uint32_t stack[256];
        int      sp   = 0;
        stack[sp++]   = kInvalid;
        uint32_t addr = 0;
        while (addr != kInvalid)
        {
            const rro_node& nd = nodes[addr];
            if (nd.child0 != kInvalid)
            {
                float a0, a1, b0, b1;
                isect_box(nd.aabb0_min_or_v0, nd.aabb0_max_or_v1, inv, oxi, ct, r.tmin, a0, a1);
                isect_box(nd.aabb1_min_or_v2, nd.aabb1_max_or_v3, inv, oxi, ct, r.tmin, b0, b1);
                bool tc0 = a0 <= a1, tc1 = b0 <= b1, c1f = tc1 && (a0 > b0);
                if (tc0 || tc1)
                {
                    uint32_t deferred;
                    if (c1f || !tc0)
                    {
                        addr     = nd.child1;
                        deferred = nd.child0;
                    }
                    else
                    {
                        addr     = nd.child0;
                        deferred = nd.child1;
                    }
                    if (tc0 && tc1 && sp < 256) stack[sp++] = deferred;
                    continue;
                }
            }
            else
            {
                float t =
                    isect_tri(r, ld3(nd.aabb0_min_or_v0), ld3(nd.aabb0_max_or_v1), ld3(nd.aabb1_min_or_v2), ct);
                if (t < ct)
                {
                    ct  = t;
                    hit = true;
                }
            }
            addr = stack[--sp];
        }
        if (hit) out_t[gi] = ct;
    });
}

// The precise triangle test's traversal (csrc/trace_precise.cuh twin): hits
// as rro_trace, and (optional) the fp32 distance of each closest / first hit.
void rro_trace_precise(const rro_node* nodes, uint32_t n_nodes, const rro_ray* rays, uint32_t nrays, int query,
                       int output, void* hits, float* out_t, int threads)
{
    parallel_for(nrays, threads, [&](uint64_t gi) {
        if (out_t) out_t[gi] = INFINITY;
        if (n_nodes == 0) return;
        trace_one(nodes, rays[gi], query == 1, output == 0, hits, gi, nullptr, 0, 1, out_t);
    });
}

// The precise test of ray i against triangle tri9[i]: t (or +inf) and uv.
void rro_tri_test_precise(const rro_ray* rays, const float* tri9, uint32_t nrays, float* out_tuv)
{
    for (uint32_t i = 0; i < nrays; ++i)
    {
        RayF         r = load_ray(rays[i]);
        const float* v = tri9 + 9ull * i;
        const float  t = precise::isect_tri(r, ld3(v), ld3(v + 3), ld3(v + 6), r.tmax);
        float        u = 0.f, w = 0.f;
        if (t < r.tmax) precise::barycentrics(r, ld3(v), ld3(v + 3), ld3(v + 6), u, w);
        out_tuv[3ull * i + 0] = t < r.tmax ? t : INFINITY;
        out_tuv[3ull * i + 1] = u;
        out_tuv[3ull * i + 2] = w;
    }
}

// Per-triangle FP32 test (isect_tri + barycentrics) of ray i against the
// triangle tri9[i]: t (or +inf) and uv.  Used to classify equal-t ties.
void rro_tri_test(const rro_ray* rays, const float* tri9, uint32_t nrays, float* out_tuv)
{
    for (uint32_t i = 0; i < nrays; ++i)
    {
        RayF  r = load_ray(rays[i]);
        const float* v = tri9 + 9ull * i;
        float t = isect_tri(r, ld3(v), ld3(v + 3), ld3(v + 6), r.tmax);
        float u = 0.f, w = 0.f;
        if (t < r.tmax) barycentrics(hit_point(r, t), ld3(v), ld3(v + 3), ld3(v + 6), u, w);
        out_tuv[3ull * i + 0] = t < r.tmax ? t : INFINITY;
        out_tuv[3ull * i + 1] = u;
        out_tuv[3ull * i + 2] = w;
    }
}

}  // extern "C"
