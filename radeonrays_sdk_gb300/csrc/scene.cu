// scene.cu -- top-level (instance) BVH build and two-level traversal.
//
// Build (reference: vlk/hlbvh_top_level_builder.cpp:204-346 with kernels
// lbvh_calc_scene_aabb.comp, lbvh_calc_morton_codes_scene.comp,
// lbvh_emit_hierarchy_scene.comp, lbvh_fit_aabb_scene.comp):
//   instance box = BLAS root box carried through the forward transform (all
//   8 corners; the reference's transform_aabb, common.h:280-308, drops the
//   (max.x, min.y, min.z) corner), scene box by order-preserving atomics,
//   30-bit Morton codes of the box centres, stable sort, Karras emit, leaves
//   {child0 = invalid, child1 = instance, both slots = instance box}, refit by
//   slot unions.  Result layout: binary nodes | [inverse, forward] transforms
//   (48 B each, fit_aabb_scene:118-119) | trailer | per-instance BLAS records.
//
// Traversal (reference: vlk/kernels/isect_2l.comp:136-323): the plain kernel
// restates the reference (one thread per ray, sentinel-marked instance entry,
// binary BLAS nodes); the wide kernel traverses the binary TLAS per ray and
// each entered instance's 8-wide BLAS (trace_wide.cuh), persistent and
// warp-scheduled.  A TLAS leaf whose BLAS is empty is treated as a miss.
#include <algorithm>

#include "rr_internal.h"
#include "trace_wide.cuh"

namespace rr
{
cudaError_t launch_emit(const void* sorted_codes, int bits, uint32_t n, BvhNode* nodes, cudaStream_t s);

namespace
{
__device__ __forceinline__ uint32_t f2o(float f)
{
    uint32_t u = __float_as_uint(f);
    return u ^ ((1u + ~(u >> 31)) | 0x80000000u);
}
__device__ __forceinline__ float o2f(uint32_t u)
{
    u ^= (((u >> 31) - 1u) | 0x80000000u);
    return __uint_as_float(u);
}
__device__ __forceinline__ F3 vmin3(F3 a, F3 b) { return f3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }
__device__ __forceinline__ F3 vmax3(F3 a, F3 b) { return f3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }
__device__ __forceinline__ F3 ld3(const float* p) { return f3(p[0], p[1], p[2]); }

// transform_point (common.h:270-278), row-major 3x4.
__device__ __forceinline__ F3 xpoint(const float* m, F3 p)
{
    return f3(dot3(ld3(m), p) + m[3], dot3(ld3(m + 4), p) + m[7], dot3(ld3(m + 8), p) + m[11]);
}
// transform_ray (common.h:310-324).
__device__ __forceinline__ Ray xray(const float* m, Ray r)
{
    const F3 o = xpoint(m, r.o);
    const F3 d = f3(dot3(ld3(m), r.d), dot3(ld3(m + 4), r.d), dot3(ld3(m + 8), r.d));
    r.o        = o;
    r.d        = d;
    return r;
}

struct Box6
{
    F3 lo, hi;
};

__device__ Box6 blas_root_box(const InstanceDesc& d)
{
    if (d.leaf_count == 0) return Box6{f3(0.f, 0.f, 0.f), f3(0.f, 0.f, 0.f)};
    const BvhNode* r = reinterpret_cast<const BvhNode*>(d.blas);
    if (r->child0 != kInvalid) return Box6{vmin3(ld3(r->a0), ld3(r->b0)), vmax3(ld3(r->a1), ld3(r->b1))};
    const F3 a = ld3(r->a0), b = ld3(r->a1), c = ld3(r->b0);
    return Box6{vmin3(vmin3(a, b), c), vmax3(vmax3(a, b), c)};
}

__global__ void k_scene_boxes(SceneBuildArgs a, float* boxes, uint32_t* bounds)
{
    uint32_t lo[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, hi[3] = {0, 0, 0};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x)
    {
        const InstanceDesc d  = a.inst[i];
        const Box6         b  = blas_root_box(d);
        const float*       m  = a.forward + 24ull * i + 12;
        Box6               r{};
        for (int k = 0; k < 8; ++k)
        {
            const F3 p = f3((k & 4) ? b.hi.x : b.lo.x, (k & 2) ? b.hi.y : b.lo.y, (k & 1) ? b.hi.z : b.lo.z);
            const F3 q = xpoint(m, p);
            if (k == 0)
                r = Box6{q, q};
            else
            {
                r.lo = vmin3(r.lo, q);
                r.hi = vmax3(r.hi, q);
            }
        }
        float* o = boxes + 6ull * i;
        o[0] = r.lo.x; o[1] = r.lo.y; o[2] = r.lo.z; o[3] = r.hi.x; o[4] = r.hi.y; o[5] = r.hi.z;
        lo[0] = min(lo[0], f2o(r.lo.x)); lo[1] = min(lo[1], f2o(r.lo.y)); lo[2] = min(lo[2], f2o(r.lo.z));
        hi[0] = max(hi[0], f2o(r.hi.x)); hi[1] = max(hi[1], f2o(r.hi.y)); hi[2] = max(hi[2], f2o(r.hi.z));
    }
    for (int k = 0; k < 3; ++k)
    {
        const uint32_t l = __reduce_min_sync(0xffffffffu, lo[k]), h = __reduce_max_sync(0xffffffffu, hi[k]);
        if ((threadIdx.x & 31) == 0)
        {
            atomicMin(&bounds[k], l);
            atomicMax(&bounds[4 + k], h);
        }
    }
}

__device__ __forceinline__ uint32_t expand10(uint32_t r)
{
    r = (r * 0x00010001u) & 0xFF0000FFu;
    r = (r * 0x00000101u) & 0x0F00F00Fu;
    r = (r * 0x00000011u) & 0xC30C30C3u;
    r = (r * 0x00000005u) & 0x49249249u;
    return r;
}

__global__ void k_scene_morton(const float* boxes, uint32_t n, const uint32_t* bounds, uint32_t* codes)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const F3     mlo = f3(o2f(bounds[0]), o2f(bounds[1]), o2f(bounds[2]));
    const F3     mhi = f3(o2f(bounds[4]), o2f(bounds[5]), o2f(bounds[6]));
    const F3     ext = f3(mhi.x - mlo.x, mhi.y - mlo.y, mhi.z - mlo.z);
    const float* b   = boxes + 6ull * i;
    const F3     p   = f3((0.5f * (b[0] + b[3]) - mlo.x) / ext.x, (0.5f * (b[1] + b[4]) - mlo.y) / ext.y,
                          (0.5f * (b[2] + b[5]) - mlo.z) / ext.z);
    const float  s   = 1024.0f;
    const uint32_t x = (uint32_t)fminf(fmaxf(p.x * s, 0.f), s - 1.f), y = (uint32_t)fminf(fmaxf(p.y * s, 0.f), s - 1.f),
                   z = (uint32_t)fminf(fmaxf(p.z * s, 0.f), s - 1.f);
    codes[i] = (expand10(x) << 2) | (expand10(y) << 1) | expand10(z);
}

__device__ __forceinline__ void slots_union(const BvhNode* nodes, uint32_t c, F3& lo, F3& hi)
{
    const BvhNode* nd = nodes + c;
    const F3 a = f3(__ldcg(&nd->a0[0]), __ldcg(&nd->a0[1]), __ldcg(&nd->a0[2]));
    const F3 b = f3(__ldcg(&nd->a1[0]), __ldcg(&nd->a1[1]), __ldcg(&nd->a1[2]));
    const F3 p = f3(__ldcg(&nd->b0[0]), __ldcg(&nd->b0[1]), __ldcg(&nd->b0[2]));
    const F3 q = f3(__ldcg(&nd->b1[0]), __ldcg(&nd->b1[1]), __ldcg(&nd->b1[2]));
    lo = vmin3(a, p);
    hi = vmax3(b, q);
}

__global__ void k_scene_refit(const float* boxes, const uint32_t* sorted_idx, uint32_t n, BvhNode* nodes,
                              DeviceWords* words)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t leaf   = n - 1 + k;
    const uint32_t inst   = sorted_idx[k];
    const float*   b      = boxes + 6ull * inst;
    const uint32_t parent = n == 1 ? kInvalid : __ldcg(&nodes[leaf].parent);
    float4*        dst    = reinterpret_cast<float4*>(nodes + leaf);
    __stcg(dst + 0, make_float4(b[0], b[1], b[2], __uint_as_float(kInvalid)));
    __stcg(dst + 1, make_float4(b[3], b[4], b[5], __uint_as_float(inst)));
    __stcg(dst + 2, make_float4(b[0], b[1], b[2], __uint_as_float(parent)));
    __stcg(dst + 3, make_float4(b[3], b[4], b[5], __uint_as_float(0u)));
    uint32_t addr = parent;
    for (int level = 0; addr != kInvalid; ++level)
    {
        if (addr >= n - 1 || level > 96)
        {
            atomicOr(&words->error_bits, (uint32_t)RR_CUDA_DEVICE_ERROR_NODE_RANGE);
            return;
        }
        __threadfence();
        if (atomicExch(&nodes[addr].update, 1u) == 0u) return;
        __threadfence();
        BvhNode*       nd = nodes + addr;
        const uint32_t c0 = __ldcg(&nd->child0), c1 = __ldcg(&nd->child1);
        if (c0 >= 2 * n - 1 || c1 >= 2 * n - 1)
        {
            atomicOr(&words->error_bits, (uint32_t)RR_CUDA_DEVICE_ERROR_NODE_RANGE);
            return;
        }
        F3 l0, h0, l1, h1;
        slots_union(nodes, c0, l0, h0);
        slots_union(nodes, c1, l1, h1);
        __stcg(&nd->a0[0], l0.x); __stcg(&nd->a0[1], l0.y); __stcg(&nd->a0[2], l0.z);
        __stcg(&nd->a1[0], h0.x); __stcg(&nd->a1[1], h0.y); __stcg(&nd->a1[2], h0.z);
        __stcg(&nd->b0[0], l1.x); __stcg(&nd->b0[1], l1.y); __stcg(&nd->b0[2], l1.z);
        __stcg(&nd->b1[0], h1.x); __stcg(&nd->b1[1], h1.y); __stcg(&nd->b1[2], h1.z);
        addr = __ldcg(&nd->parent);
    }
}

__global__ void k_scene_trailer(Trailer* t, Trailer v, const uint32_t* bounds)
{
    if (threadIdx.x == 0) *t = v;
    __syncthreads();
    if (bounds && threadIdx.x < 8) t->bounds[threadIdx.x] = (threadIdx.x & 3) == 3 ? 0u : bounds[threadIdx.x];
}

// ---- two-level traversal -------------------------------------------------
constexpr int kBlock    = 128;
constexpr int kLdsStack = 16;
constexpr int kGlobalStack = 64;

// Plain two-level kernel: restates isect_2l.comp.
template <bool kAny, bool kFull, bool kStats>
__global__ void __launch_bounds__(kBlock) k_trace_scene_binary(SceneTraceArgs sa)
{
    const TraceArgs& a = sa.base;
    __shared__ uint32_t lds[kBlock * kLdsStack];
    const uint32_t      gid   = blockIdx.x * kBlock + threadIdx.x;
    uint32_t            count = a.ray_count;
    if (a.indirect) count = min(count, __ldg(a.indirect));
    if (gid >= count) return;

    const BvhNode* tlas  = reinterpret_cast<const BvhNode*>(a.bvh);
    const Ray      world = load_ray(a.rays, gid);
    Ray            ray   = world;
    F3             inv   = safe_invdir(ray.d);
    F3             oxi   = f3(-ray.o.x * inv.x, -ray.o.y * inv.y, -ray.o.z * inv.z);
    float          ct    = ray.tmax;
    uint32_t       caddr = kInvalid, cinst = kInvalid, cprim = kInvalid, inst = kInvalid;
    const BvhNode* blas  = nullptr;
    uint32_t       fetches = 0;

    uint32_t* gstack = reinterpret_cast<uint32_t*>(a.scratch + kTraceScratchHeader) + (uint64_t)gid * kGlobalStack;
    uint32_t  sptr   = 0;
    const uint32_t bottom = threadIdx.x * kLdsStack;
    uint32_t       lsp    = bottom;
    lds[lsp++]            = kInvalid;
    uint32_t addr         = a.empty ? kInvalid : 0u;

    auto push = [&](uint32_t v) {
        if (lsp - bottom >= kLdsStack)
        {
            if (sptr + kLdsStack > kGlobalStack)
            {
                atomicOr(&a.words->error_bits, (uint32_t)RR_CUDA_DEVICE_ERROR_STACK_OVERFLOW);
                return;
            }
            for (int i = 1; i < kLdsStack; ++i) gstack[sptr + i] = lds[bottom + i];
            sptr += kLdsStack;
            lsp = bottom + 1;
        }
        lds[lsp++] = v;
    };
    auto pop = [&]() -> uint32_t {
        uint32_t v = lds[--lsp];
        if (v == kInvalid && sptr > 0)
        {
            sptr -= kLdsStack;
            for (int i = 1; i < kLdsStack; ++i) lds[bottom + i] = gstack[sptr + i];
            lsp = bottom + kLdsStack - 1;
            v   = lds[lsp];
        }
        return v;
    };

    uint32_t blas_lim = kInvalid;
    while (addr != kInvalid)
    {
        if (addr >= (inst == kInvalid ? a.node_limit : blas_lim) || fetches >= kFetchCap)
        {
            raise_error(a.words, RR_CUDA_DEVICE_ERROR_NODE_RANGE);
            caddr = kInvalid;
            break;
        }
        const NodeView nd = load_binary_node(inst == kInvalid ? tlas : blas, addr);
        ++fetches;
        bool descend = false;
        if (nd.child0 != kInvalid)
        {
            float a0, a1, b0, b1;
            isect_box(nd.l0, nd.h0, inv, oxi, ct, ray.tmin, a0, a1);
            isect_box(nd.l1, nd.h1, inv, oxi, ct, ray.tmin, b0, b1);
            const bool tc0 = a0 <= a1, tc1 = b0 <= b1, c1f = tc1 && (a0 > b0);
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
                if (tc0 && tc1) push(deferred);
                descend = true;
            }
        }
        else if (inst == kInvalid)
        {
            const uint32_t     id = nd.child1;
            const InstanceDesc d  = sa.inst[id];
            if (d.leaf_count != 0)
            {
                inst     = id;
                blas     = reinterpret_cast<const BvhNode*>(d.blas);
                blas_lim = d.leaf_count == kInvalid ? kInvalid : 2 * d.leaf_count - 1;
                ray  = xray(sa.xforms + 24ull * inst, world);
                inv  = safe_invdir(ray.d);
                oxi  = f3(-ray.o.x * inv.x, -ray.o.y * inv.y, -ray.o.z * inv.z);
                push(kSentinel);
                addr    = 0;
                descend = true;
            }
        }
        else
        {
            const float t = isect_tri(ray, nd.l0, nd.h0, nd.l1, ct);
            if (t < ct)
            {
                if (!kAny)
                {
                    ct    = t;
                    caddr = addr;
                    cprim = nd.child1;
                    cinst = inst;
                }
                else
                {
                    write_hit<kFull>(a.hits, gid, ray, t, nd.l0, nd.h0, nd.l1, inst, nd.child1, inst);
                    if (kStats) add_stats(a.words, fetches, 0);
                    return;
                }
            }
        }
        if (descend) continue;
        addr = pop();
        if (addr == kSentinel)
        {
            inst = kInvalid;
            ray  = world;
            inv  = safe_invdir(ray.d);
            oxi  = f3(-ray.o.x * inv.x, -ray.o.y * inv.y, -ray.o.z * inv.z);
            addr = pop();
        }
    }
    if (caddr != kInvalid)
    {
        const InstanceDesc d  = sa.inst[cinst];
        const NodeView     nd = load_binary_node(reinterpret_cast<const BvhNode*>(d.blas), caddr);
        const Ray          lr = xray(sa.xforms + 24ull * cinst, world);
        write_hit<kFull>(a.hits, gid, lr, ct, nd.l0, nd.h0, nd.l1, cinst, cprim, cinst);
    }
    else
        write_miss<kFull>(a.hits, gid);
    if (kStats) add_stats(a.words, fetches, 0);
}

// Chosen two-level kernel: binary TLAS, 8-wide BLAS, persistent warps.
constexpr int kTlasStack = 64;

template <bool kAny, bool kFull, bool kStats>
__global__ void k_trace_scene_wide(SceneTraceArgs sa, uint32_t gcap)
{
    const TraceArgs& a = sa.base;
    extern __shared__ WideEntry s_stack[];
    const uint32_t tglob = blockIdx.x * blockDim.x + threadIdx.x;
    WideStack      st;
    st.s    = s_stack + threadIdx.x;
    st.g    = reinterpret_cast<WideEntry*>(a.scratch + kTraceScratchHeader) + (uint64_t)tglob * gcap;
    st.gcap = gcap;
    uint32_t* ray_ctr = reinterpret_cast<uint32_t*>(a.scratch);
    const int lane    = threadIdx.x & 31;
    uint32_t  count   = a.ray_count;
    if (a.indirect) count = min(count, __ldg(a.indirect));
    const BvhNode* tlas = reinterpret_cast<const BvhNode*>(a.bvh);

    for (;;)
    {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(ray_ctr, 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= count) return;
        const uint32_t gid = base + lane;
        if (gid < count)
        {
            const Ray world = load_ray(a.rays, gid);
            const F3  winv  = safe_invdir(world.d);
            const F3  woxi  = f3(-world.o.x * winv.x, -world.o.y * winv.y, -world.o.z * winv.z);
            float     ct    = world.tmax;
            uint32_t  cinst = kInvalid, cbest = kInvalid, nf = 0, tf = 0;
            bool      found_any = false;
            uint32_t  stack[kTlasStack];
            int       sp   = 0;
            uint32_t  addr = a.empty ? kInvalid : 0u;
            for (;;)
            {
                if (addr == kInvalid)
                {
                    if (sp == 0) break;
                    addr = stack[--sp];
                }
                if (addr >= a.node_limit || nf >= kFetchCap)
                {
                    raise_error(a.words, RR_CUDA_DEVICE_ERROR_NODE_RANGE);
                    cbest = kInvalid;
                    break;
                }
                const NodeView nd = load_binary_node(tlas, addr);
                ++nf;
                addr = kInvalid;
                if (nd.child0 != kInvalid)
                {
                    float a0, a1, b0, b1;
                    isect_box(nd.l0, nd.h0, winv, woxi, ct, world.tmin, a0, a1);
                    isect_box(nd.l1, nd.h1, winv, woxi, ct, world.tmin, b0, b1);
                    const bool tc0 = a0 <= a1, tc1 = b0 <= b1, c1f = tc1 && (a0 > b0);
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
                        if (tc0 && tc1)
                        {
                            if (sp < kTlasStack)
                                stack[sp++] = deferred;
                            else
                                atomicOr(&a.words->error_bits, (uint32_t)RR_CUDA_DEVICE_ERROR_STACK_OVERFLOW);
                        }
                    }
                }
                else
                {
                    const uint32_t     id = nd.child1;
                    const InstanceDesc d  = sa.inst[id];
                    if (d.leaf_count == 0) continue;
                    const Ray      lr   = xray(sa.xforms + 24ull * id, world);
                    uint32_t       best = kInvalid;
                    const uint32_t wlim = d.leaf_count > 1 ? d.leaf_count - 1 : 1;
                    const bool hit = wide_traverse<kAny>(lr, reinterpret_cast<const WideNode*>(d.wide_nodes),
                                                         reinterpret_cast<const WideTri*>(d.wide_tris), wlim,
                                                         d.leaf_count, ct, best, st, a.words, nf, tf);
                    if (best != kInvalid)
                    {
                        cinst = id;
                        cbest = best;
                    }
                    if (kAny && hit)
                    {
                        found_any = true;
                        break;
                    }
                }
            }
            (void)found_any;
            if (cbest != kInvalid)
            {
                const InstanceDesc d  = sa.inst[cinst];
                const float4*      tp = reinterpret_cast<const float4*>(reinterpret_cast<const WideTri*>(d.wide_tris) + cbest);
                const float4       A = __ldg(tp), B = __ldg(tp + 1), C = __ldg(tp + 2);
                const Ray          lr = xray(sa.xforms + 24ull * cinst, world);
                write_hit<kFull>(a.hits, gid, lr, ct, f3(A.x, A.y, A.z), f3(B.x, B.y, B.z), f3(C.x, C.y, C.z), cinst,
                                 __float_as_uint(A.w), cinst);
            }
            else
                write_miss<kFull>(a.hits, gid);
            if (kStats) add_stats(a.words, nf, tf);
        }
        __syncwarp();
    }
}

template <bool kAny, bool kFull, bool kStats>
cudaError_t go(const SceneTraceArgs& sa, cudaStream_t s)
{
    const TraceArgs& a = sa.base;
    if (!sa.use_wide)
    {
        const int blocks = (int)((a.ray_count + kBlock - 1) / kBlock);
        k_trace_scene_binary<kAny, kFull, kStats><<<blocks, kBlock, 0, s>>>(sa);
        return cudaGetLastError();
    }
    auto         kern  = k_trace_scene_wide<kAny, kFull, kStats>;
    const int    block = kWideBlock;
    const size_t smem  = (size_t)block * kWideShortStack * sizeof(WideEntry);
    int          per_sm = a.blocks_per_sm;
    if (per_sm <= 0)
    {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, smem) != cudaSuccess) per_sm = 1;
        per_sm = per_sm > 0 ? per_sm : 1;
    }
    uint64_t       threads = (uint64_t)a.sm_count * per_sm * block;
    const uint64_t need    = ((uint64_t)a.ray_count + 31) / 32 * 32;
    if (threads > need) threads = (need + block - 1) / block * block;
    const int      blocks = (int)(threads / block);
    const uint64_t avail  = (a.scratch_bytes - kTraceScratchHeader) / sizeof(WideEntry);
    uint64_t       gcap   = avail / ((uint64_t)blocks * block);
    gcap                  = gcap / kWideShortStack * kWideShortStack;
    if (gcap > 4096) gcap = 4096;
    cudaError_t e = cudaMemsetAsync(a.scratch, 0, kTraceScratchHeader, s);
    if (e != cudaSuccess) return e;
    kern<<<blocks, block, smem, s>>>(sa, (uint32_t)gcap);
    return cudaGetLastError();
}

inline int grid_for(uint64_t n, int block) { return (int)std::max<uint64_t>(1, (n + block - 1) / block); }

}  // namespace

SceneLayout scene_layout(uint32_t n)
{
    SceneLayout L{};
    L.n           = n;
    L.nodes_bytes = n == 0 ? 0 : (2ull * n - 1) * sizeof(BvhNode);
    L.xforms_off  = L.nodes_bytes;
    L.trailer_off = align_up(L.xforms_off + 2ull * n * 48, kAlign);
    L.inst_off    = L.trailer_off + sizeof(Trailer);
    L.total       = align_up(L.inst_off + (size_t)n * sizeof(InstanceDesc), kAlign);
    L.s_bounds    = 0;
    L.s_boxes     = kAlign;
    L.s_codes     = align_up(L.s_boxes + 24ull * n, kAlign);
    L.s_codes_alt = align_up(L.s_codes + 4ull * n, kAlign);
    L.s_idx       = align_up(L.s_codes_alt + 4ull * n, kAlign);
    L.s_idx_alt   = align_up(L.s_idx + 4ull * n, kAlign);
    L.s_sort      = align_up(L.s_idx_alt + 4ull * n, kAlign);
    L.s_sort_bytes = radix_sort_scratch_bytes(n, 30, &L.sort_tiles, &L.sort_passes);
    L.s_total     = align_up(L.s_sort + L.s_sort_bytes, kAlign);
    return L;
}

cudaError_t launch_build_scene(const SceneBuildArgs& a, const SceneLayout& L, uint8_t* scratch, uint8_t* result,
                               DeviceWords* words, cudaStream_t s)
{
    Trailer tr{};
    tr.magic      = kMagic;
    tr.version    = kVersion;
    tr.kind       = kKindScene;
    tr.leaf_count = a.n;
    tr.node_count = a.n == 0 ? 0 : 2 * a.n - 1;
    tr.morton_bits = 30;
    tr.xforms_off = L.xforms_off;
    tr.inst_off   = L.inst_off;
    Trailer* dtr  = reinterpret_cast<Trailer*>(result + L.trailer_off);
    if (a.n == 0)
    {
        k_scene_trailer<<<1, 32, 0, s>>>(dtr, tr, nullptr);
        return cudaGetLastError();
    }
    uint32_t*   bounds = reinterpret_cast<uint32_t*>(scratch + L.s_bounds);
    float*      boxes  = reinterpret_cast<float*>(scratch + L.s_boxes);
    cudaError_t e      = cudaMemsetAsync(bounds, 0xff, 16, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(bounds + 4, 0, 16, s);
    if (e != cudaSuccess) return e;
    k_scene_boxes<<<std::min(grid_for(a.n, 128), 1024), 128, 0, s>>>(a, boxes, bounds);
    uint32_t* codes     = reinterpret_cast<uint32_t*>(scratch + L.s_codes);
    uint32_t* codes_alt = reinterpret_cast<uint32_t*>(scratch + L.s_codes_alt);
    uint32_t* idx       = reinterpret_cast<uint32_t*>(scratch + L.s_idx);
    uint32_t* idx_alt   = reinterpret_cast<uint32_t*>(scratch + L.s_idx_alt);
    k_scene_morton<<<grid_for(a.n, 128), 128, 0, s>>>(boxes, a.n, bounds, codes);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    bool alt = false;
    e = launch_radix_sort(codes, codes_alt, idx, idx_alt, a.n, 30, scratch + L.s_sort, L.sort_tiles, words, s, &alt);
    if (e != cudaSuccess) return e;
    BvhNode* nodes = reinterpret_cast<BvhNode*>(result);
    if (a.n > 1)
    {
        e = launch_emit(alt ? codes_alt : codes, 30, a.n, nodes, s);
        if (e != cudaSuccess) return e;
    }
    k_scene_refit<<<grid_for(a.n, 128), 128, 0, s>>>(boxes, alt ? idx_alt : idx, a.n, nodes, words);
    k_scene_trailer<<<1, 32, 0, s>>>(dtr, tr, bounds);
    return cudaGetLastError();
}

cudaError_t launch_trace_scene(const SceneTraceArgs& sa, cudaStream_t s)
{
    const TraceArgs& a = sa.base;
    if (a.ray_count == 0) return cudaSuccess;
    if (sa.use_bvh4) return launch_trace_scene_bvh4(sa, s);
    if (sa.use_persistent) return launch_trace_scene_persistent(sa, s);
    const bool any = a.query == RR_INTERSECT_QUERY_ANY, full = a.output == RR_INTERSECT_QUERY_OUTPUT_FULL_HIT;
    if (a.collect_stats)
    {
        if (any) return full ? go<true, true, true>(sa, s) : go<true, false, true>(sa, s);
        return full ? go<false, true, true>(sa, s) : go<false, false, true>(sa, s);
    }
    if (any) return full ? go<true, true, false>(sa, s) : go<true, false, false>(sa, s);
    return full ? go<false, true, false>(sa, s) : go<false, false, false>(sa, s);
}

}  // namespace rr
