// trace_scene_bvh4.cu -- persistent lane-refill two-level traversal of a
// scene whose instances all have 4-wide nodes of one form
// (RR_CUDA_NODE_FORMAT_BVH4 or _BVH4Q8 BLASes; no reference counterpart for
// the BLAS part, see trace_bvh4.cu).
//
// The instance tree is binary and traversed as in isect_2l.comp:153-322:
// near child first, one stack for both levels, an instance leaf pushes the
// sentinel, transforms the ray by the instance's inverse transform and
// enters the BLAS; popping the sentinel restores the world ray.  Inside a
// BLAS the 4-wide nodes are visited nearest first (b4_children).  The
// closest hit is the reference's except exact equal-t ties, and any-hit
// hit/miss flags are the reference's.  Both levels share one short stack
// that spills in full blocks of kB4Spill entries.
#include "trace_bvh4.cuh"

namespace rr
{
namespace
{
__device__ __forceinline__ F3 ld3(const float* p) { return f3(p[0], p[1], p[2]); }
// transform_point / transform_ray (common.h:270-278, 310-324), row-major 3x4.
__device__ __forceinline__ Ray xray(const float* m, Ray r)
{
    const F3 o = f3(dot3(ld3(m), r.o) + m[3], dot3(ld3(m + 4), r.o) + m[7], dot3(ld3(m + 8), r.o) + m[11]);
    const F3 d = f3(dot3(ld3(m), r.d), dot3(ld3(m + 4), r.d), dot3(ld3(m + 8), r.d));
    r.o        = o;
    r.d        = d;
    return r;
}

// Capacity of the 4-wide node array of a BLAS with n triangles (geom_layout).
__device__ __forceinline__ uint32_t b4_capacity(uint32_t n) { return (n - 1) / 3 + n / 3 + 1; }

struct S4Ray
{
    Ray             ray;  // in the current frame
    F3              inv, oxi;
    float           ct;
    uint32_t        addr;   // TLAS: binary node; BLAS: 4-wide reference
    uint32_t        caddr;  // BLAS binary leaf of the closest hit
    uint32_t        inst;   // instance being traversed, kInvalid in the TLAS
    uint32_t        cinst;  // instance of the closest hit
    const BvhNode*  blas;   // binary nodes of the current BLAS (its leaves)
    const Bvh4Node* blas4;  // its 4-wide nodes
    uint32_t        n;      // its triangle count
    uint32_t        gsp, steps;
    int             sp;
};

__device__ __forceinline__ void set_frame(S4Ray& s, const Ray& r)
{
    s.ray = r;
    s.inv = safe_invdir(r.d);
    s.oxi = f3(-r.o.x * s.inv.x, -r.o.y * s.inv.y, -r.o.z * s.inv.z);
}

// One step; true when the ray is finished.
// kQ8: the BLASes' 4-wide nodes have 8-bit bounds (Bvh4QNode); as in the
// single-level kernel, a leaf triangle's hit counts only if its exact box
// passes the reference's slab test too.
template <bool kAny, bool kQ8>
__device__ __forceinline__ bool s4_step(S4Ray& s, const SceneTraceArgs& sa, uint32_t gid, const PStack& st,
                                        uint32_t& nf)
{
    const TraceArgs& a   = sa.base;
    const bool       top = s.inst == kInvalid;
    if (++s.steps > kFetchCap)
    {
        raise_error(a.words, RR_CUDA_DEVICE_ERROR_NODE_RANGE);
        s.caddr = kInvalid;
        return true;
    }
    bool descend = false;
    if (top)
    {
        if (s.addr >= a.node_limit)
        {
            raise_error(a.words, RR_CUDA_DEVICE_ERROR_NODE_RANGE);
            s.caddr = kInvalid;
            return true;
        }
        const NodeView nd = load_binary_node(reinterpret_cast<const BvhNode*>(a.bvh), s.addr);
        ++nf;
        if (nd.child0 != kInvalid)
        {
            float a0, a1, b0, b1;
            isect_box(nd.l0, nd.h0, s.inv, s.oxi, s.ct, s.ray.tmin, a0, a1);
            isect_box(nd.l1, nd.h1, s.inv, s.oxi, s.ct, s.ray.tmin, b0, b1);
            const bool tc0 = a0 <= a1, tc1 = b0 <= b1, c1f = tc1 && (a0 > b0);
            if (tc0 || tc1)
            {
                const bool first1 = c1f || !tc0;
                if (tc0 && tc1)
                {
                    b4_reserve(s.sp, s.gsp, st, a.words, 1);
                    st.at(s.sp++) = first1 ? nd.child0 : nd.child1;
                }
                s.addr  = first1 ? nd.child1 : nd.child0;
                descend = true;
            }
        }
        else
        {
            const uint32_t     id = nd.child1;
            const InstanceDesc d  = sa.inst[id];
            if (d.leaf_count != 0)
            {
                s.inst  = id;
                s.blas  = reinterpret_cast<const BvhNode*>(d.blas);
                s.blas4 = reinterpret_cast<const Bvh4Node*>(d.wide_nodes);
                s.n     = d.leaf_count;
                set_frame(s, xray(sa.xforms + 24ull * id, load_ray(a.rays, gid)));
                b4_reserve(s.sp, s.gsp, st, a.words, 1);
                st.at(s.sp++) = kSentinel;
                s.addr        = 0;  // the BLAS's root 4-wide node
                descend       = true;
            }
        }
    }
    else
    {
        const uint32_t ref  = s.addr;
        const bool     leaf = (ref & kBvh4Leaf) != 0;
        const uint32_t idx  = ref & ~kBvh4Leaf;
        if (leaf ? (idx < s.n - 1 || idx >= 2 * s.n - 1) : idx >= b4_capacity(s.n))
        {
            raise_error(a.words, RR_CUDA_DEVICE_ERROR_NODE_RANGE);
            s.caddr = kInvalid;
            return true;
        }
        ++nf;
        if (leaf)
        {
            const float4* p = reinterpret_cast<const float4*>(s.blas + idx);
            const float4  v0 = __ldg(p), v1 = __ldg(p + 1), v2 = __ldg(p + 2);
            float t = isect_tri(s.ray, f3(v0.x, v0.y, v0.z), f3(v1.x, v1.y, v1.z), f3(v2.x, v2.y, v2.z), s.ct);
            if (kQ8 && t < s.ct)  // exact-box re-test of a hit (see b4_step)
            {
                float b0, b1;
                isect_box(f3(b4_min3(v0.x, v1.x, v2.x), b4_min3(v0.y, v1.y, v2.y), b4_min3(v0.z, v1.z, v2.z)),
                          f3(b4_max3(v0.x, v1.x, v2.x), b4_max3(v0.y, v1.y, v2.y), b4_max3(v0.z, v1.z, v2.z)), s.inv,
                          s.oxi, s.ct, s.ray.tmin, b0, b1);
                if (!(b0 <= b1)) t = s.ct;
            }
            if (t < s.ct)
            {
                s.ct    = t;
                s.caddr = idx;
                s.cinst = s.inst;
                if (kAny) return true;
            }
        }
        else
        {
            const B4Hits h = kQ8 ? b4q_children(reinterpret_cast<const Bvh4QNode*>(s.blas4) + idx, s.inv, s.oxi,
                                                s.ray.tmin, s.ct)
                                 : b4_children(s.blas4 + idx, s.inv, s.oxi, s.ray.tmin, s.ct);
            if (h.n)
            {
                s.addr  = b4_descend(h, s.sp, s.gsp, st, a.words);
                descend = true;
            }
        }
    }
    if (descend) return false;
    if (!b4_pop(s.sp, s.gsp, st, s.addr)) return true;
    if (s.addr == kSentinel)
    {
        s.inst = kInvalid;
        set_frame(s, load_ray(a.rays, gid));
        if (!b4_pop(s.sp, s.gsp, st, s.addr)) return true;
    }
    return false;
}

template <bool kAny, bool kFull, bool kStats, bool kQ8>
__global__ void __launch_bounds__(kPBlock, 8) k_trace_scene_bvh4(SceneTraceArgs sa, uint32_t gcap)
{
    const TraceArgs&    a = sa.base;
    __shared__ uint32_t s_stack[kPBlock * kPShort];
    const uint32_t      tglob = blockIdx.x * blockDim.x + threadIdx.x;
    PStack              st;
    st.s    = s_stack + threadIdx.x;
    st.g    = reinterpret_cast<uint32_t*>(a.scratch + kTraceScratchHeader) + (uint64_t)tglob * gcap;
    st.gcap = gcap;
    uint32_t*      ray_ctr = reinterpret_cast<uint32_t*>(a.scratch);
    const uint32_t lane    = threadIdx.x & 31;
    const uint32_t lt      = (1u << lane) - 1u;
    uint32_t       count   = a.ray_count;
    if (a.indirect) count = min(count, __ldg(a.indirect));

    S4Ray    s;
    uint32_t gid = kInvalid, nf = 0;
    bool     active = false, pending = false, exhausted = false;
    uint32_t it = 0;
    for (;;)
    {
        __syncwarp();
        const uint32_t idle = __ballot_sync(0xffffffffu, !active);
        if (idle && (__popc(idle) >= kPRefillMin || exhausted || idle == 0xffffffffu))
        {
            const uint32_t n    = exhausted ? 0u : __popc(idle);
            uint32_t       base = 0;
            if (n)
            {
                const int leader = __ffs(idle) - 1;
                if ((int)lane == leader) base = atomicAdd(ray_ctr, n);
                base      = __shfl_sync(0xffffffffu, base, leader);
                exhausted = base + n >= count;
            }
            if (!active)
            {
                if (pending)
                {
                    if (s.caddr != kInvalid)
                    {
                        // Barycentrics in the hit instance's frame (isect_2l.comp:293-305).
                        const InstanceDesc d  = sa.inst[s.cinst];
                        const NodeView     nd = load_binary_node(reinterpret_cast<const BvhNode*>(d.blas), s.caddr);
                        const Ray          lr = xray(sa.xforms + 24ull * s.cinst, load_ray(a.rays, gid));
                        write_hit<kFull>(a.hits, gid, lr, s.ct, nd.l0, nd.h0, nd.l1, s.cinst, nd.child1, s.cinst);
                    }
                    else
                        write_miss<kFull>(a.hits, gid);
                    if (kStats)
                    {
                        atomicAdd(&a.words->rays, 1ull);
                        atomicAdd(&a.words->node_fetches, (unsigned long long)nf);
                    }
                    pending = false;
                }
                const uint32_t my = base + __popc(idle & lt);
                if (n && my < count)
                {
                    gid = my;
                    if (a.empty)
                        write_miss<kFull>(a.hits, gid);
                    else
                    {
                        active = true;
                        nf     = 0;
                        const Ray r = load_ray(a.rays, gid);
                        set_frame(s, r);
                        s.ct    = r.tmax;
                        s.addr  = 0;
                        s.caddr = kInvalid;
                        s.inst = s.cinst = kInvalid;
                        s.blas  = nullptr;
                        s.blas4 = nullptr;
                        s.n     = 0;
                        s.gsp = s.steps = 0;
                        s.sp            = 0;
                    }
                }
            }
        }
        const uint32_t amask = __ballot_sync(0xffffffffu, active);
        if (amask == 0 && exhausted && __ballot_sync(0xffffffffu, pending) == 0) break;
        // Step batching: a lane's next step is an instance-tree node, a
        // BLAS 4-wide node or a BLAS leaf, three different paths.  Each
        // iteration only the lanes of the most common kind step (every
        // fourth iteration all of them, so that no lane waits long); the
        // others wait.  Every ray's own sequence of steps is unchanged, so
        // hits are too.  Measured 4 Mi / 8.4 M incoherent rays on 256, 512
        // and 2,048 instanced soups: 6 %, 11 % and 11.5 % faster.  Holding
        // back only the leaf lanes (the single-level kernel's rule) was
        // 4-6 % slower, and majority steps without the all-lane iterations
        // gained nothing.
        const bool     in_top  = active && s.inst == kInvalid;
        const bool     in_leaf = active && !in_top && (s.addr & kBvh4Leaf) != 0;
        const uint32_t nt      = __popc(__ballot_sync(0xffffffffu, in_top));
        const uint32_t nl      = __popc(__ballot_sync(0xffffffffu, in_leaf));
        const uint32_t nn      = __popc(amask) - nt - nl;
        const int      kind    = (nt >= nn && nt >= nl) ? 0 : (nn >= nl ? 1 : 2);
        ++it;
        const bool go = (it & 3u) == 0 || (in_top ? kind == 0 : in_leaf ? kind == 2 : kind == 1);
        if (active && go && s4_step<kAny, kQ8>(s, sa, gid, st, nf))
        {
            active  = false;
            pending = true;
        }
    }
}

template <bool kAny, bool kFull, bool kStats>
cudaError_t go(const SceneTraceArgs& sa, cudaStream_t s)
{
    const TraceArgs& a      = sa.base;
    auto             kern   = sa.bvh4_q8 ? k_trace_scene_bvh4<kAny, kFull, kStats, true>
                                         : k_trace_scene_bvh4<kAny, kFull, kStats, false>;
    int              per_sm = a.blocks_per_sm;
    if (per_sm <= 0)
    {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kPBlock, 0) != cudaSuccess) per_sm = 1;
        per_sm = per_sm > 0 ? per_sm : 1;
    }
    const PGrid g = persistent_grid(a.sm_count, per_sm, a.ray_count, a.scratch_bytes, kTraceScratchHeader);
    cudaError_t e = cudaMemsetAsync(a.scratch, 0, kTraceScratchHeader, s);
    if (e != cudaSuccess) return e;
    kern<<<g.blocks, kPBlock, 0, s>>>(sa, g.gcap);
    return cudaGetLastError();
}
}  // namespace

cudaError_t launch_trace_scene_bvh4(const SceneTraceArgs& sa, cudaStream_t s)
{
    const TraceArgs& a = sa.base;
    if (a.ray_count == 0) return cudaSuccess;
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
