// trace_batch.cu -- many intersection requests (different geometries, ray
// counts, query kinds and outputs) traced by one persistent launch.
//
// No reference counterpart: the reference dispatches isect.comp once per
// rrCmdIntersect.  This is the launch a serving loop packs its admitted
// requests into.  The ray space of the launch is the concatenation of the
// requests' rays; a lane that takes global ray g finds its request by a binary
// search over the requests' exclusive ray prefix and then runs the same
// per-ray state machine as the single-request persistent kernel
// (trace_persistent.cuh): the reference's visit order and arithmetic, so every
// hit is bit-identical to tracing that request alone with rrCmdIntersect.
//
// With 4-wide geometries (use_bvh4: every request's buffer carries 4-wide
// nodes, all fp32 or all 8-bit) the lanes run the 4-wide kernel's state
// machine (trace_bvh4.cuh) instead, so each hit equals that request traced
// alone with RR_CUDA_TRAVERSAL_BVH4.
#include "trace_bvh4.cuh"
#include "trace_persistent.cuh"

namespace rr
{
namespace
{
constexpr size_t kBatchHeader = 256;  // ray counter

template <bool kStats>
__global__ void __launch_bounds__(kPBlock, 8) k_trace_batch(BatchTraceArgs a, uint32_t gcap)
{
    __shared__ uint32_t s_stack[kPBlock * kPShort];
    const uint32_t      tglob = blockIdx.x * blockDim.x + threadIdx.x;
    PStack              st;
    st.s    = s_stack + threadIdx.x;
    st.g    = reinterpret_cast<uint32_t*>(a.scratch + a.spill_off) + (uint64_t)tglob * gcap;
    st.gcap = gcap;
    uint32_t*      ray_ctr = reinterpret_cast<uint32_t*>(a.scratch);
    const uint32_t lane    = threadIdx.x & 31;
    const uint32_t lt      = (1u << lane) - 1u;
    const uint32_t count   = a.total;

    PRay           s;
    const BvhNode* nodes = nullptr;
    uint32_t       gid = kInvalid, r = 0, nlim = 0, nf = 0;
    bool           any = false, box = false, active = false, pending = false, exhausted = false;
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
                    void*      hits = a.req[r].hits;
                    const bool full = (a.req[r].flags & kReqFull) != 0;
                    if (s.caddr != kInvalid)
                    {
                        const NodeView nd = load_binary_node(nodes, s.caddr);
                        if (box)
                        {
                            if (full)
                                write_box_hit<true>(hits, gid, 0u, nd.child1, nd.child1);
                            else
                                write_box_hit<false>(hits, gid, 0u, nd.child1, nd.child1);
                        }
                        else if (full)
                            write_hit<true>(hits, gid, s.ray, s.ct, nd.l0, nd.h0, nd.l1, 0u, nd.child1, nd.child1);
                        else
                            write_hit<false>(hits, gid, s.ray, s.ct, nd.l0, nd.h0, nd.l1, 0u, nd.child1, nd.child1);
                    }
                    else if (full)
                        write_miss<true>(hits, gid);
                    else
                        write_miss<false>(hits, gid);
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
                    r                     = batch_find(a.prefix, a.count, my);
                    gid                   = my - __ldg(a.prefix + r);
                    const BatchTraceReq& q = a.req[r];
                    const uint32_t       fl = q.flags;
                    if (fl & kReqEmpty)
                    {
                        if (fl & kReqFull)
                            write_miss<true>(q.hits, gid);
                        else
                            write_miss<false>(q.hits, gid);
                    }
                    else
                    {
                        active = true;
                        nf     = 0;
                        nodes  = reinterpret_cast<const BvhNode*>(q.bvh);
                        nlim   = q.node_limit;
                        any    = (fl & kReqAny) != 0;
                        box    = (fl & kReqBoxes) != 0;
                        p_start(s, q.rays, gid);
                    }
                }
            }
        }
        const uint32_t amask = __ballot_sync(0xffffffffu, active);
        if (amask == 0 && exhausted && __ballot_sync(0xffffffffu, pending) == 0) break;
        if (active && p_step<false, true>(s, nodes, nlim, st, a.words, nf, any, box))
        {
            active  = false;
            pending = true;
        }
    }
}

// The 4-wide variant: the same refill loop around b4_step; a request's
// 4-wide nodes sit wide_off256 * 256 bytes into its buffer, its binary leaves
// (the triangles) at [n - 1, 2n - 2].
// kQ8: every request's 4-wide nodes have 8-bit bounds (b4_step's kQ8).
template <bool kStats, bool kQ8>
__global__ void __launch_bounds__(kPBlock, 8) k_trace_batch_bvh4(BatchTraceArgs a, uint32_t gcap)
{
    __shared__ uint32_t s_stack[kPBlock * kPShort];
    const uint32_t      tglob = blockIdx.x * blockDim.x + threadIdx.x;
    PStack              st;
    st.s     = s_stack + threadIdx.x;
    st.g     = reinterpret_cast<uint32_t*>(a.scratch + a.spill_off) + (uint64_t)tglob * gcap;
    st.gcap  = gcap;
    st.depth = kPShort;
    uint32_t*      ray_ctr = reinterpret_cast<uint32_t*>(a.scratch);
    const uint32_t lane    = threadIdx.x & 31;
    const uint32_t lt      = (1u << lane) - 1u;
    const uint32_t count   = a.total;

    B4Ray           s;
    const BvhNode*  nodes = nullptr;
    const Bvh4Node* wn    = nullptr;
    uint32_t        gid = kInvalid, r = 0, nlim = 0, wlim = 0, first_leaf = 0, nf = 0, tf = 0;
    bool            any = false, active = false, pending = false, exhausted = false;
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
                    void*      hits = a.req[r].hits;
                    const bool full = (a.req[r].flags & kReqFull) != 0;
                    if (s.best != kInvalid)
                    {
                        const NodeView nd = load_binary_node(nodes, s.best);
                        if (full)
                            write_hit<true>(hits, gid, s.ray, s.ct, nd.l0, nd.h0, nd.l1, 0u, nd.child1, nd.child1);
                        else
                            write_hit<false>(hits, gid, s.ray, s.ct, nd.l0, nd.h0, nd.l1, 0u, nd.child1, nd.child1);
                    }
                    else if (full)
                        write_miss<true>(hits, gid);
                    else
                        write_miss<false>(hits, gid);
                    if (kStats)
                    {
                        atomicAdd(&a.words->rays, 1ull);
                        atomicAdd(&a.words->node_fetches, (unsigned long long)nf);
                        atomicAdd(&a.words->tri_fetches, (unsigned long long)tf);
                    }
                    pending = false;
                }
                const uint32_t my = base + __popc(idle & lt);
                if (n && my < count)
                {
                    r                      = batch_find(a.prefix, a.count, my);
                    gid                    = my - __ldg(a.prefix + r);
                    const BatchTraceReq& q  = a.req[r];
                    const uint32_t       fl = q.flags;
                    if (fl & kReqEmpty)
                    {
                        if (fl & kReqFull)
                            write_miss<true>(q.hits, gid);
                        else
                            write_miss<false>(q.hits, gid);
                    }
                    else
                    {
                        active     = true;
                        nf = tf    = 0;
                        nodes      = reinterpret_cast<const BvhNode*>(q.bvh);
                        wn         = reinterpret_cast<const Bvh4Node*>(q.bvh + (size_t)q.wide_off256 * 256);
                        nlim       = q.node_limit;
                        first_leaf = (nlim + 1u) / 2u - 1u;
                        wlim       = q.wide_limit;
                        any        = (fl & kReqAny) != 0;
                        b4_start<false>(s, load_ray(q.rays, gid));
                    }
                }
            }
        }
        const uint32_t amask = __ballot_sync(0xffffffffu, active);
        if (amask == 0 && exhausted && __ballot_sync(0xffffffffu, pending) == 0) break;
        // Leaf batching, as in the single-request 4-wide kernel: leaf steps
        // wait for a quarter of the active lanes.
        const bool at_leaf = active && (s.ref & kBvh4Leaf) != 0;
        const bool do_leaf = 4 * __popc(__ballot_sync(0xffffffffu, at_leaf)) >= __popc(amask);
        if (active && at_leaf == do_leaf &&
            b4_step<false, false, true, kQ8>(s, wn, nodes, wlim, first_leaf, nlim, st, a.words, nf, tf, any))
        {
            active  = false;
            pending = true;
        }
    }
}

template <bool kStats>
cudaError_t go(const BatchTraceArgs& a, cudaStream_t s)
{
    auto kern   = !a.use_bvh4 ? k_trace_batch<kStats>
                  : a.bvh4_q8 ? k_trace_batch_bvh4<kStats, true>
                              : k_trace_batch_bvh4<kStats, false>;
    int  per_sm = a.blocks_per_sm;
    if (per_sm <= 0)
    {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kPBlock, 0) != cudaSuccess) per_sm = 1;
        per_sm = per_sm > 0 ? per_sm : 1;
    }
    const PGrid g = persistent_grid(a.sm_count, per_sm, a.total, a.scratch_bytes, a.spill_off);
    cudaError_t e = cudaMemsetAsync(a.scratch, 0, kBatchHeader, s);
    if (e != cudaSuccess) return e;
    kern<<<g.blocks, kPBlock, 0, s>>>(a, g.gcap);
    return cudaGetLastError();
}
}  // namespace

BatchTraceLayout batch_trace_layout(uint32_t count, uint64_t total_rays)
{
    BatchTraceLayout L;
    L.req_off    = kBatchHeader;
    L.prefix_off = align_up(L.req_off + (size_t)count * sizeof(BatchTraceReq), kAlign);
    L.spill_off  = align_up(L.prefix_off + ((size_t)count + 1) * sizeof(uint32_t), kAlign);
    // The single-request scratch per ray (trace_scratch_bytes) minus its
    // header: the persistent grid takes its spill stacks from it.
    L.total = L.spill_off + (trace_scratch_bytes(total_rays > 0xffffffffull ? 0xffffffffu : (uint32_t)total_rays) -
                             kTraceScratchHeader);
    return L;
}

cudaError_t launch_trace_batch(const BatchTraceArgs& a, cudaStream_t s)
{
    if (a.total == 0) return cudaSuccess;
    return a.collect_stats ? go<true>(a, s) : go<false>(a, s);
}

}  // namespace rr
