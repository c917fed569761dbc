// trace_common.cuh -- ray/box/triangle arithmetic shared by the traversal
// kernels.  Each function restates one helper of the reference's shader
// library (vlk/kernels/common.h) with the oracle's fp32 rules: IEEE
// round-to-nearest, fma only where the shader writes fma, no contraction
// (the .cu files are compiled with --fmad=false).
#pragma once
#include "rr_internal.h"

namespace rr
{
constexpr size_t kTraceScratchHeader = 256;  // control words at the start of the trace scratch

// Node visits after which a ray is abandoned with RR_CUDA_DEVICE_ERROR_NODE_RANGE
// (a well-formed BVH needs a few thousand at most; the cap only stops a
// corrupted, cyclic buffer from spinning a warp forever).
constexpr uint32_t kFetchCap = 1u << 22;

__device__ __forceinline__ void raise_error(DeviceWords* w, uint32_t bits) { atomicOr(&w->error_bits, bits); }

struct F3
{
    float x, y, z;
};
__device__ __forceinline__ F3 f3(float x, float y, float z) { return F3{x, y, z}; }
__device__ __forceinline__ F3 sub3(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float dot3(F3 a, F3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ F3 cross3(F3 a, F3 b)
{
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

struct Ray
{
    F3    o;
    float tmin;
    F3    d;
    float tmax;
};

__device__ __forceinline__ Ray load_ray(const uint8_t* rays, uint32_t i)
{
    const float4* p = reinterpret_cast<const float4*>(rays) + 2ull * i;
    float4        a = __ldg(p), b = __ldg(p + 1);
    return Ray{f3(a.x, a.y, a.z), a.w, f3(b.x, b.y, b.z), b.w};
}

// mycopysign + safe_invdir (common.h:166-183).
__device__ __forceinline__ float inv_component(float d)
{
    const float e = 1e-5f;
    return 1.0f / (fabsf(d) > e ? d : (d < 0.f ? -e : e));
}
__device__ __forceinline__ F3 safe_invdir(F3 d) { return f3(inv_component(d.x), inv_component(d.y), inv_component(d.z)); }

// fast_intersect_aabb (common.h:150-164): hit iff t0 <= t1.
__device__ __forceinline__ void isect_box(F3 lo, F3 hi, F3 inv, F3 oxi, float tmax_, float tmin_, float& t0,
                                          float& t1)
{
    const float fx = fmaf(hi.x, inv.x, oxi.x), fy = fmaf(hi.y, inv.y, oxi.y), fz = fmaf(hi.z, inv.z, oxi.z);
    const float nx = fmaf(lo.x, inv.x, oxi.x), ny = fmaf(lo.y, inv.y, oxi.y), nz = fmaf(lo.z, inv.z, oxi.z);
    t1 = fminf(fminf(fmaxf(fz, nz), fminf(fmaxf(fx, nx), fmaxf(fy, ny))), tmax_);
    t0 = fmaxf(fmaxf(fminf(fz, nz), fmaxf(fminf(fx, nx), fminf(fy, ny))), tmin_);
}

// fast_intersect_triangle (common.h:103-137): returns t_max on a miss.
__device__ __forceinline__ float isect_tri(const Ray& r, F3 v1, F3 v2, F3 v3, float t_max)
{
    const F3    e1    = sub3(v2, v1);
    const F3    e2    = sub3(v3, v1);
    const F3    s1    = cross3(r.d, e2);
    const float denom = dot3(s1, e1);
    if (denom == 0.f) return t_max;
    const float invd = 1.0f / denom;
    const F3    d    = sub3(r.o, v1);
    const float b1   = dot3(d, s1) * invd;
    const F3    s2   = cross3(d, e1);
    const float b2   = dot3(r.d, s2) * invd;
    const float tmp  = dot3(e2, s2) * invd;
    if (b1 < 0.0f || b1 > 1.0f || b2 < 0.0f || b1 + b2 > 1.0f || tmp < r.tmin || tmp > t_max) return t_max;
    return tmp;
}

// calculate_barycentrics (common.h:187-209) of p = o + t*d.
__device__ __forceinline__ float2 barycentrics(const Ray& r, float t, F3 v1, F3 v2, F3 v3)
{
    const F3    p   = f3(r.o.x + t * r.d.x, r.o.y + t * r.d.y, r.o.z + t * r.d.z);
    const F3    e1  = sub3(v2, v1);
    const F3    e2  = sub3(v3, v1);
    const F3    e   = sub3(p, v1);
    const float d00 = dot3(e1, e1), d01 = dot3(e1, e2), d11 = dot3(e2, e2), d20 = dot3(e, e1), d21 = dot3(e, e2);
    const float den = d00 * d11 - d01 * d01;
    if (den == 0.f) return make_float2(0.f, 0.f);
    const float inv = 1.0f / (d00 * d11 - d01 * d01);
    return make_float2((d11 * d20 - d01 * d21) * inv, (d00 * d21 - d01 * d20) * inv);
}

struct NodeView
{
    F3       l0, h0, l1, h1;  // child boxes (or v0, v1, v2 of a leaf)
    uint32_t child0, child1;
};

__device__ __forceinline__ NodeView load_binary_node(const BvhNode* nodes, uint32_t i)
{
    const float4* p = reinterpret_cast<const float4*>(nodes + i);
    const float4  a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2), d = __ldg(p + 3);
    NodeView      n;
    n.l0     = f3(a.x, a.y, a.z);
    n.child0 = __float_as_uint(a.w);
    n.h0     = f3(b.x, b.y, b.z);
    n.child1 = __float_as_uint(b.w);
    n.l1     = f3(c.x, c.y, c.z);
    n.h1     = f3(d.x, d.y, d.z);
    return n;
}

// Full hit: {uv, inst_id, prim_id} in one 16-byte store.  Instance-id output:
// `id_out` (the single-level kernels write the primitive id there,
// isect.comp:197,235; the two-level kernels the instance id, isect_2l.comp:252,315).
template <bool kFull>
__device__ __forceinline__ void write_hit(void* hits, uint32_t gid, const Ray& r, float t, F3 v0, F3 v1, F3 v2,
                                          uint32_t inst, uint32_t prim, uint32_t id_out)
{
    if (kFull)
    {
        const float2 uv = barycentrics(r, t, v0, v1, v2);
        reinterpret_cast<uint4*>(hits)[gid] =
            make_uint4(__float_as_uint(uv.x), __float_as_uint(uv.y), inst, prim);
    }
    else
        reinterpret_cast<uint32_t*>(hits)[gid] = id_out;
}

// Leaf of an AABB-list geometry: the box is stored in the leaf's first two
// vertex slots (min, max).  The hit distance is the slab entry distance,
// clamped to min_t; a miss returns t_max.  (The reference declares AABB lists
// but does not implement them, radeonrays.cpp:286-289; this is this build's
// definition, shared with the oracle.)
__device__ __forceinline__ float isect_leaf_box(const Ray& r, F3 inv, F3 oxi, F3 lo, F3 hi, float t_max)
{
    float t0, t1;
    isect_box(lo, hi, inv, oxi, t_max, r.tmin, t0, t1);
    return t0 <= t1 ? t0 : t_max;
}

// Hit record of a box leaf: uv = (0, 0).
template <bool kFull>
__device__ __forceinline__ void write_box_hit(void* hits, uint32_t gid, uint32_t inst, uint32_t prim, uint32_t id_out)
{
    if (kFull)
        reinterpret_cast<uint4*>(hits)[gid] = make_uint4(0u, 0u, inst, prim);
    else
        reinterpret_cast<uint32_t*>(hits)[gid] = id_out;
}

// A miss writes only inst_id (isect.comp:238-244).
template <bool kFull>
__device__ __forceinline__ void write_miss(void* hits, uint32_t gid)
{
    if (kFull)
        reinterpret_cast<uint32_t*>(hits)[4ull * gid + 2] = kInvalid;
    else
        reinterpret_cast<uint32_t*>(hits)[gid] = kInvalid;
}

// Warp-aggregated fetch counters.
__device__ __forceinline__ void add_stats(DeviceWords* w, uint32_t nodes, uint32_t tris)
{
    const uint32_t mask = __activemask();
    const uint32_t sn = __reduce_add_sync(mask, nodes), st = __reduce_add_sync(mask, tris),
                   sr = __popc(mask);
    if ((threadIdx.x & 31) == (uint32_t)(__ffs(mask) - 1))
    {
        atomicAdd(&w->rays, (unsigned long long)sr);
        atomicAdd(&w->node_fetches, (unsigned long long)sn);
        atomicAdd(&w->tri_fetches, (unsigned long long)st);
    }
}

}  // namespace rr
