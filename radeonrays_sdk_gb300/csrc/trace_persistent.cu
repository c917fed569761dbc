// trace_persistent.cu -- persistent lane-refill traversal over the reference's
// 64-byte binary nodes.
//
// The per-ray algorithm (trace_persistent.cuh, p_step) is the reference's
// (vlk/kernels/isect.comp:105-245), so the hits are bit-identical to the
// plain kernel and to the oracle, ties and any-hit choices included.
//
// What differs is the scheduling: a persistent grid whose lanes each advance
// their own ray one node per loop iteration and take the next ray from a
// counter as soon as their ray finishes (one warp-aggregated atomic per
// refill).  One thread per ray (the plain kernel) leaves most lanes of a warp
// idle while its longest ray finishes; refilling keeps them working.  The
// stack is a short stack in shared memory (interleaved across the block) that
// spills to a per-thread region of the caller's scratch buffer.
//
// Streamed variant (kStream, host-buffer tracing): one launch over all rays
// while the copy engine is still bringing them in.  Rays are taken in index
// order, so a warp only waits (bounded, once per chunk) for the arrival flag
// of the last chunk its new rays lie in, which the copy stream sets after
// that chunk's copy.  Each claimed ray is counted once in the done counter of
// its part (a copy-out unit of several chunks; release adds, batched per
// warp and part, published as the warp's claims move on and when the rays
// run out), and the copy-out stream waits for each counter before it copies
// that part's hits to the host.  A ray the warp still holds when it
// publishes the ray's part is late-listed; the late scatter after the kernel
// brings its hit to the host (trace_stream.cuh).  So every counter reaches
// its part's size by the time the kernel ends, whether its rays were traced,
// missed an empty geometry, or gave up waiting for their chunk.
#include "trace_persistent.cuh"
#include "trace_stream.cuh"

namespace rr
{
namespace
{
using namespace stream_detail;
template <bool kAny, bool kFull, bool kStats, bool kBox, bool kStream, bool kPrecise>
__global__ void __launch_bounds__(kPBlock, 8) k_trace_persistent(TraceArgs a, uint32_t gcap)
{
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
    const BvhNode* nodes = reinterpret_cast<const BvhNode*>(a.bvh);

    PRay     s;
    uint32_t gid = kInvalid, nf = 0;
    bool     active = false, pending = false, exhausted = false;
    // kStream: the block's highest chunk known to have arrived, and each
    // warp's done-count slots (shared memory).
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
        // Lanes whose ray finished write its hit and take a new ray together,
        // once at least kPRefillMin lanes are idle (or no ray is left).
        const uint32_t idle = __ballot_sync(0xffffffffu, !active);
        if (idle && (__popc(idle) >= kPRefillMin || exhausted || idle == 0xffffffffu))
        {
            int      seen     = -1;  // kStream: highest chunk known to have arrived (warp-uniform)
            uint32_t jump_end = 0;   // kStream: ClaimNote::jump_end (warp-uniform)
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
                    if (s.caddr != kInvalid)
                    {
                        const NodeView nd = load_binary_node(nodes, s.caddr);
                        if (kBox)
                            write_box_hit<kFull>(a.hits, gid, 0u, nd.child1, nd.child1);
                        else if (kPrecise)
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
                            nf     = 0;
                            p_start<kPrecise>(s, load_ray_cg(a.rays, gid));
                        }
                        else
                        {
                            s.caddr = kInvalid;
                            pending = true;
                        }
                    }
                    else if (a.empty)
                        write_miss<kFull>(a.hits, gid);
                    else
                    {
                        active = true;
                        nf     = 0;
                        p_start<kPrecise>(s, a.rays, gid);
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
        if (active && p_step<kAny, false, kBox, kPrecise>(s, nodes, a.node_limit, st, a.words, nf))
        {
            active  = false;
            pending = true;
        }
    }
}

template <bool kAny, bool kFull, bool kStats, bool kBox, bool kStream, bool kPrecise = false>
cudaError_t go2(const TraceArgs& a, cudaStream_t s)
{
    auto kern   = k_trace_persistent<kAny, kFull, kStats, kBox, kStream, kPrecise>;
    int  per_sm = a.blocks_per_sm;
    if (per_sm <= 0)
    {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kPBlock, 0) != cudaSuccess) per_sm = 1;
        per_sm = per_sm > 0 ? per_sm : 1;
    }
    const PGrid g = persistent_grid(a.sm_count, per_sm, a.ray_count, a.scratch_bytes, kTraceScratchHeader);
    cudaError_t e = cudaMemsetAsync(a.scratch, 0, kTraceScratchHeader, s);
    if (e != cudaSuccess) return e;
    kern<<<g.blocks, kPBlock, 0, s>>>(a, g.gcap);
    return cudaGetLastError();
}

// Triangle leaves: the reference's test, or the precise one; box leaves have
// no precise variant (their hit is the slab entry distance).
template <bool kAny, bool kFull, bool kStats, bool kStream>
cudaError_t go_tri(const TraceArgs& a, cudaStream_t s)
{
    if (a.triangle_test == RR_CUDA_TRIANGLE_TEST_WATERTIGHT)
        return go2<kAny, kFull, kStats, false, kStream, true>(a, s);
    return go2<kAny, kFull, kStats, false, kStream>(a, s);
}

template <bool kAny, bool kFull, bool kStats>
cudaError_t go(const TraceArgs& a, cudaStream_t s)
{
    return a.box_leaves ? go2<kAny, kFull, kStats, true, false>(a, s) : go_tri<kAny, kFull, kStats, false>(a, s);
}

template <bool kAny, bool kFull>
cudaError_t go_stream(const TraceArgs& a, cudaStream_t s)
{
    return a.box_leaves ? go2<kAny, kFull, false, true, true>(a, s) : go_tri<kAny, kFull, false, true>(a, s);
}

// The late scatter of a streamed trace (trace_stream.cuh): one record per
// listed ray, device hits to the host buffer.  Indices at or past cap are
// skipped (a listed ray index is always below the ray count).
template <typename Rec>
__global__ void k_late_scatter(const uint32_t* late_count, const uint32_t* late, uint32_t cap, const Rec* dev_hits,
                               Rec* host_hits)
{
    const uint32_t n = min(*late_count, cap);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const uint32_t g = __ldg(late + i);
        if (g < cap) host_hits[g] = dev_hits[g];
    }
}
}  // namespace

cudaError_t launch_late_scatter(const uint32_t* late_count, const uint32_t* late, uint32_t cap,
                                const uint8_t* dev_hits, uint8_t* host_hits, uint32_t rec_bytes, int sm_count,
                                cudaStream_t s)
{
    const int blocks = (sm_count > 0 ? sm_count : 1) * 2;
    if (rec_bytes == 16)
        k_late_scatter<uint4><<<blocks, 256, 0, s>>>(late_count, late, cap, reinterpret_cast<const uint4*>(dev_hits),
                                                     reinterpret_cast<uint4*>(host_hits));
    else
        k_late_scatter<uint32_t><<<blocks, 256, 0, s>>>(late_count, late, cap,
                                                        reinterpret_cast<const uint32_t*>(dev_hits),
                                                        reinterpret_cast<uint32_t*>(host_hits));
    return cudaGetLastError();
}

cudaError_t launch_trace_persistent(const TraceArgs& a, cudaStream_t s)
{
    if (a.ray_count == 0) return cudaSuccess;
    const bool any = a.query == RR_INTERSECT_QUERY_ANY, full = a.output == RR_INTERSECT_QUERY_OUTPUT_FULL_HIT;
    if (a.stream_words)
    {
        if (any) return full ? go_stream<true, true>(a, s) : go_stream<true, false>(a, s);
        return full ? go_stream<false, true>(a, s) : go_stream<false, false>(a, s);
    }
    if (a.collect_stats)
    {
        if (any) return full ? go<true, true, true>(a, s) : go<true, false, true>(a, s);
        return full ? go<false, true, true>(a, s) : go<false, false, true>(a, s);
    }
    if (any) return full ? go<true, true, false>(a, s) : go<true, false, false>(a, s);
    return full ? go<false, true, false>(a, s) : go<false, false, false>(a, s);
}

}  // namespace rr
