// trace_bvh4.cu -- persistent lane-refill traversal over the 4-wide fp32
// nodes of an RR_CUDA_NODE_FORMAT_BVH4 buffer (no reference counterpart: the
// reference traverses its binary nodes only, vlk/kernels/isect.comp).
//
// A step fetches one reference of the lane's ray: a 4-wide node (128 bytes:
// four exact child boxes and their references) or a binary leaf node (the
// triangle).  A node's children are slab-tested with the reference's formula
// (vlk/kernels/common.h:150-164; the same arithmetic as the binary kernels);
// the hit ones are ordered by entry distance, the nearest is visited next
// and the others are pushed, farthest first.  A leaf gets the reference's
// triangle test (common.h:103-137) and is accepted iff t < closest t.  The
// closest hit is therefore the reference's except where two triangles are
// hit at exactly the same t (then the visit order decides), and any-hit
// hit/miss flags are the reference's.
//
// Compared with the binary kernels a 4-wide node covers about two binary
// levels: half as many dependent fetches, and the internal nodes are a third
// of the binary node array.  Scheduling is that of the persistent binary
// kernel (trace_persistent.cu): lanes refill from a ray counter as their ray
// finishes; the short stack lives in shared memory and spills to scratch.
#include "trace_bvh4.cuh"
#include "trace_stream.cuh"

namespace rr
{
namespace
{
using namespace stream_detail;
// kStream: the streamed variant for host-buffer tracing (trace_stream.cuh),
// with the same arrival waits and done counts as the persistent binary
// kernel's streamed variant.
// The short stack is dynamic shared memory of kPBlock x depth entries; the
// depth (12..32, default kPShort) is a launch parameter the autotuner picks.
// Residency: 8 blocks per SM (64 registers) over fp32 nodes; 9 (56
// registers, no spill) over quantised nodes, whose half-size fetches leave
// the L1 room for more rays in flight (measured 6 % faster; the fp32 nodes
// were 2 % slower at 9).  The precise test needs the 64 registers.
template <bool kAny, bool kFull, bool kStats, bool kStream, bool kPrecise, bool kQ8>
__global__ void __launch_bounds__(kPBlock, (kQ8 && !kPrecise) ? 9 : 8)
    k_trace_bvh4(TraceArgs a, uint32_t gcap, int depth)
{
    extern __shared__ uint32_t s_stack[];
    const uint32_t             tglob = blockIdx.x * blockDim.x + threadIdx.x;
    PStack                     st;
    st.s     = s_stack + threadIdx.x;
    st.g     = reinterpret_cast<uint32_t*>(a.scratch + kTraceScratchHeader) + (uint64_t)tglob * gcap;
    st.gcap  = gcap;
    st.depth = depth;
    uint32_t*       ray_ctr    = reinterpret_cast<uint32_t*>(a.scratch);
    const uint32_t  lane       = threadIdx.x & 31;
    const uint32_t  lt         = (1u << lane) - 1u;
    uint32_t        count      = a.ray_count;
    if (a.indirect) count = min(count, __ldg(a.indirect));
    const BvhNode*  nodes      = reinterpret_cast<const BvhNode*>(a.bvh);
    const Bvh4Node* wn         = a.bvh4_nodes;
    const uint32_t  first_leaf = a.tri_limit - 1;  // binary leaves [n-1, 2n-2]

    B4Ray    s;
    uint32_t gid = kInvalid, nf = 0, tf = 0;
    bool     active = false, pending = false, exhausted = false;
    __shared__ int        s_seen;
    __shared__ DoneCounts s_dc[kPBlock / 32];
    volatile DoneCounts&  dc = s_dc[threadIdx.x >> 5];
    if (kStream)
    {
        if (threadIdx.x == 0) s_seen = -1;
        if (lane == 0)
        {
            dc.cur_c = dc.cur_n = dc.prev_n = dc.fin = 0;
            dc.prev_c                               = kInvalid;
        }
        __syncthreads();
    }
    for (;;)
    {
        __syncwarp();
        const uint32_t idle = __ballot_sync(0xffffffffu, !active);
        if (idle && (__popc(idle) >= kPRefillMin || exhausted || idle == 0xffffffffu))
        {
            int            seen     = -1;  // kStream: highest chunk known to have arrived (warp-uniform)
            uint32_t       jump_end = 0;   // kStream: ClaimNote::jump_end (warp-uniform)
            const uint32_t n    = exhausted ? 0u : __popc(idle);
            uint32_t       base = 0;
            if (n)
            {
                const int leader = __ffs(idle) - 1;
                ClaimNote note{-1, kInvalid, 0u};
                if ((int)lane == leader)
                {
                    base = atomicAdd(ray_ctr, n);
                    // The streamed variant's arrival wait and claim counts
                    // (trace_stream.cuh), by the claiming lane alone.
                    if (kStream && base < count) note = claim_leader(a, base, min(base + n, count), &s_seen, dc);
                }
                base      = __shfl_sync(0xffffffffu, base, leader);
                exhausted = base + n >= count;
                if (kStream && base < count)
                {
                    seen                     = __shfl_sync(0xffffffffu, note.seen, leader);
                    jump_end                 = __shfl_sync(0xffffffffu, note.jump_end, leader);
                    const uint32_t late_part = __shfl_sync(0xffffffffu, note.late_part, leader);
                    if (late_part != kInvalid) late_held(a, active || pending, gid, late_part, lane);
                }
            }
            bool fresh = false;  // kStream: took a new ray at this refill
            if (!active)
            {
                if (pending)
                {
                    if (s.best != kInvalid)
                    {
                        const NodeView nd = load_binary_node(nodes, s.best);
                        if (kPrecise)
                            write_hit_precise<kFull>(a.hits, gid, s.ray, nd.l0, nd.h0, nd.l1, 0u, nd.child1,
                                                     nd.child1);
                        else
                            write_hit<kFull>(a.hits, gid, s.ray, s.ct, nd.l0, nd.h0, nd.l1, 0u, nd.child1,
                                             nd.child1);
                    }
                    else
                        write_miss<kFull>(a.hits, gid);
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
                    gid = my;
                    if (kStream)
                    {
                        fresh = true;
                        // Traced once its chunk is in; an empty geometry or a
                        // chunk that never arrived finishes as a miss at the
                        // next refill, where it is counted like any other.
                        if (!a.empty && (int)(gid >> a.stream_shift) <= seen)
                        {
                            active = true;
                            nf = tf = 0;
                            b4_start<kPrecise>(s, load_ray_cg(a.rays, gid));
                        }
                        else
                        {
                            s.best  = kInvalid;
                            pending = true;
                        }
                    }
                    else if (a.empty)
                        write_miss<kFull>(a.hits, gid);
                    else
                    {
                        active = true;
                        nf = tf = 0;
                        b4_start<kPrecise>(s, load_ray(a.rays, gid));
                    }
                }
            }
            if (kStream)
            {
                if (jump_end) jump_done(a, fresh, gid, jump_end, lane);
                if (exhausted) finalize_done(a, active || pending, gid, lane, dc);
            }
        }
        const uint32_t amask = __ballot_sync(0xffffffffu, active);
        if (amask == 0 && exhausted && __ballot_sync(0xffffffffu, pending) == 0) break;
        // Leaf batching: the lanes at a leaf take their step only with at
        // least a quarter of the active lanes (or when no lane is at an
        // inner node); otherwise they wait one iteration while the others
        // test nodes.  The warp then runs the leaf and the node paths in
        // separate iterations more often, instead of both in each.  Every
        // ray's own sequence of steps is unchanged, so hits are too.
        const bool     at_leaf = active && (s.ref & kBvh4Leaf) != 0;
        const bool     do_leaf = 4 * __popc(__ballot_sync(0xffffffffu, at_leaf)) >= __popc(amask);
        if (active && at_leaf == do_leaf &&
            b4_step<kAny, kPrecise, false, kQ8>(s, wn, nodes, a.wide_limit, first_leaf, a.node_limit, st, a.words, nf,
                                                tf))
        {
            active  = false;
            pending = true;
        }
    }
}

template <bool kAny, bool kFull, bool kStats, bool kStream, bool kPrecise, bool kQ8 = false>
cudaError_t go2(const TraceArgs& a, cudaStream_t s)
{
    auto         kern   = k_trace_bvh4<kAny, kFull, kStats, kStream, kPrecise, kQ8>;
    const int    depth  = a.short_stack > 0 ? a.short_stack : kPShort;
    const size_t smem   = (size_t)kPBlock * depth * sizeof(uint32_t);
    int          per_sm = a.blocks_per_sm;
    if (per_sm <= 0)
    {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kPBlock, smem) != cudaSuccess) per_sm = 1;
        per_sm = per_sm > 0 ? per_sm : 1;
    }
    const PGrid g = persistent_grid(a.sm_count, per_sm, a.ray_count, a.scratch_bytes, kTraceScratchHeader);
    cudaError_t e = cudaMemsetAsync(a.scratch, 0, kTraceScratchHeader, s);
    if (e != cudaSuccess) return e;
    kern<<<g.blocks, kPBlock, smem, s>>>(a, g.gcap, depth);
    return cudaGetLastError();
}

template <bool kAny, bool kFull, bool kStats, bool kStream>
cudaError_t go(const TraceArgs& a, cudaStream_t s)
{
    const bool precise = a.triangle_test == RR_CUDA_TRIANGLE_TEST_WATERTIGHT;
    if (a.bvh4_q8)
        return precise ? go2<kAny, kFull, kStats, kStream, true, true>(a, s)
                       : go2<kAny, kFull, kStats, kStream, false, true>(a, s);
    return precise ? go2<kAny, kFull, kStats, kStream, true>(a, s) : go2<kAny, kFull, kStats, kStream, false>(a, s);
}
}  // namespace

cudaError_t launch_trace_bvh4(const TraceArgs& a, cudaStream_t s)
{
    if (a.ray_count == 0) return cudaSuccess;
    const bool any = a.query == RR_INTERSECT_QUERY_ANY, full = a.output == RR_INTERSECT_QUERY_OUTPUT_FULL_HIT;
    if (a.stream_words)
    {
        if (any) return full ? go<true, true, false, true>(a, s) : go<true, false, false, true>(a, s);
        return full ? go<false, true, false, true>(a, s) : go<false, false, false, true>(a, s);
    }
    if (a.collect_stats)
    {
        if (any) return full ? go<true, true, true, false>(a, s) : go<true, false, true, false>(a, s);
        return full ? go<false, true, true, false>(a, s) : go<false, false, true, false>(a, s);
    }
    if (any) return full ? go<true, true, false, false>(a, s) : go<true, false, false, false>(a, s);
    return full ? go<false, true, false, false>(a, s) : go<false, false, false, false>(a, s);
}

}  // namespace rr
