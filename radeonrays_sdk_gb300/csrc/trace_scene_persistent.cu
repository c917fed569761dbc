// trace_scene_persistent.cu -- persistent lane-refill two-level traversal
// (instance tree over binary-node BLASes).
//
// The per-ray algorithm restates isect_2l.comp:153-322 exactly as the plain
// two-level kernel (scene.cu) does: one stack for both levels, an instance
// leaf pushes the sentinel, transforms the world ray by the instance's
// inverse transform and restarts at the BLAS root; popping the sentinel
// restores the world ray.  Near child first, strict `t < closest_t`, so the
// hits are bit-identical to the plain two-level kernel (ties and any-hit
// choices included).  The scheduling is that of trace_persistent.cuh: lanes
// advance their own ray one node per iteration and refill from a counter.
// The world ray is re-read from the ray buffer when the sentinel is popped
// (an L1/L2 hit) instead of being kept in registers.
#include "trace_persistent.cuh"

namespace rr
{
namespace
{
__device__ __forceinline__ F3 ld3(const float* p) { return f3(p[0], p[1], p[2]); }
// transform_point / transform_ray (common.h:270-278, 310-324), row-major 3x4.
__device__ __forceinline__ Ray xray2(const float* m, Ray r)
{
    const F3 o = f3(dot3(ld3(m), r.o) + m[3], dot3(ld3(m + 4), r.o) + m[7], dot3(ld3(m + 8), r.o) + m[11]);
    const F3 d = f3(dot3(ld3(m), r.d), dot3(ld3(m + 4), r.d), dot3(ld3(m + 8), r.d));
    r.o        = o;
    r.d        = d;
    return r;
}

struct P2Ray
{
    PRay           p;        // ray in the current frame, closest t, stack state
    const BvhNode* blas;     // BLAS of the instance being traversed
    uint32_t       blas_lim;
    uint32_t       inst;     // instance being traversed, kInvalid in the TLAS
    uint32_t       cinst;    // instance of the closest hit
};

__device__ __forceinline__ void set_frame(PRay& s, const Ray& r)
{
    s.ray = r;
    s.inv = safe_invdir(r.d);
    s.oxi = f3(-r.o.x * s.inv.x, -r.o.y * s.inv.y, -r.o.z * s.inv.z);
}

__device__ __forceinline__ void push(PRay& s, const PStack& st, uint32_t v, DeviceWords* words)
{
    if (s.sp == kPShort)
    {
        if (s.gsp + kPShort > st.gcap)
        {
            raise_error(words, RR_CUDA_DEVICE_ERROR_STACK_OVERFLOW);
            s.sp = kPShort - 1;  // overwrite the top entry: result flagged invalid
        }
        else
        {
            for (int k = 0; k < kPShort; ++k) st.g[s.gsp + k] = st.at(k);
            s.gsp += kPShort;
            s.sp = 0;
        }
    }
    st.at(s.sp++) = v;
}

// Pops into s.addr; false when the stack is empty.
__device__ __forceinline__ bool pop(PRay& s, const PStack& st)
{
    if (s.sp == 0 && s.gsp == 0) return false;
    if (s.sp == 0)
    {
        s.gsp -= kPShort;
        for (int k = 0; k < kPShort; ++k) st.at(k) = st.g[s.gsp + k];
        s.sp = kPShort;
    }
    s.addr = st.at(--s.sp);
    return true;
}

// One iteration of isect_2l.comp's loop; true when the ray is finished.
template <bool kAny>
__device__ __forceinline__ bool p2_step(P2Ray& q, const SceneTraceArgs& sa, uint32_t gid, const PStack& st,
                                        uint32_t& nf)
{
    const TraceArgs& a = sa.base;
    PRay&            s = q.p;
    const bool       top = q.inst == kInvalid;
    if (++s.steps > kFetchCap || s.addr >= (top ? a.node_limit : q.blas_lim))
    {
        raise_error(a.words, RR_CUDA_DEVICE_ERROR_NODE_RANGE);
        s.caddr = kInvalid;
        return true;
    }
    const NodeView nd = load_binary_node(top ? reinterpret_cast<const BvhNode*>(a.bvh) : q.blas, s.addr);
    ++nf;
    bool descend = false;
    if (nd.child0 != kInvalid)
    {
        float a0, a1, b0, b1;
        isect_box(nd.l0, nd.h0, s.inv, s.oxi, s.ct, s.ray.tmin, a0, a1);
        isect_box(nd.l1, nd.h1, s.inv, s.oxi, s.ct, s.ray.tmin, b0, b1);
        const bool tc0 = a0 <= a1, tc1 = b0 <= b1, c1f = tc1 && (a0 > b0);
        if (tc0 || tc1)
        {
            const bool first1 = c1f || !tc0;
            if (tc0 && tc1) push(s, st, first1 ? nd.child0 : nd.child1, a.words);
            s.addr  = first1 ? nd.child1 : nd.child0;
            descend = true;
        }
    }
    else if (top)
    {
        const uint32_t     id = nd.child1;
        const InstanceDesc d  = sa.inst[id];
        if (d.leaf_count != 0)
        {
            q.inst     = id;
            q.blas     = reinterpret_cast<const BvhNode*>(d.blas);
            q.blas_lim = d.leaf_count == kInvalid ? kInvalid : 2 * d.leaf_count - 1;
            set_frame(s, xray2(sa.xforms + 24ull * id, load_ray(a.rays, gid)));
            push(s, st, kSentinel, a.words);
            s.addr  = 0;
            descend = true;
        }
    }
    else
    {
        const float t = isect_tri(s.ray, nd.l0, nd.h0, nd.l1, s.ct);
        if (t < s.ct)
        {
            s.ct    = t;
            s.caddr = s.addr;
            q.cinst = q.inst;
            if (kAny) return true;
        }
    }
    if (descend) return false;
    if (!pop(s, st)) return true;
    if (s.addr == kSentinel)
    {
        q.inst = kInvalid;
        set_frame(s, load_ray(a.rays, gid));
        if (!pop(s, st)) return true;
    }
    return false;
}

template <bool kAny, bool kFull, bool kStats>
__global__ void __launch_bounds__(kPBlock, 8) k_trace_scene_persistent(SceneTraceArgs sa, uint32_t gcap)
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

    P2Ray    q;
    uint32_t gid = kInvalid, nf = 0;
    bool     active = false, pending = false, exhausted = false;
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
                    if (q.p.caddr != kInvalid)
                    {
                        // Barycentrics in the hit instance's frame (isect_2l.comp:293-305).
                        const InstanceDesc d  = sa.inst[q.cinst];
                        const NodeView     nd = load_binary_node(reinterpret_cast<const BvhNode*>(d.blas), q.p.caddr);
                        const Ray          lr = xray2(sa.xforms + 24ull * q.cinst, load_ray(a.rays, gid));
                        write_hit<kFull>(a.hits, gid, lr, q.p.ct, nd.l0, nd.h0, nd.l1, q.cinst, nd.child1, q.cinst);
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
                        p_start(q.p, a.rays, gid);
                        q.inst = q.cinst = kInvalid;
                        q.blas     = nullptr;
                        q.blas_lim = 0;
                    }
                }
            }
        }
        const uint32_t amask = __ballot_sync(0xffffffffu, active);
        if (amask == 0 && exhausted && __ballot_sync(0xffffffffu, pending) == 0) break;
        if (active && p2_step<kAny>(q, sa, gid, st, nf))
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
    auto             kern   = k_trace_scene_persistent<kAny, kFull, kStats>;
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

cudaError_t launch_trace_scene_persistent(const SceneTraceArgs& sa, cudaStream_t s)
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
