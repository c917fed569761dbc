// trace_stream.cuh -- device side of streamed host-buffer tracing, shared by
// the persistent kernels that have a streamed variant (trace_persistent.cu,
// trace_bvh4.cu): bounded waits for the rays' arrival flags, and the per-warp
// done counts that let the copy-out stream follow the kernel.
#pragma once
#include "trace_common.cuh"

namespace rr
{
namespace stream_detail
{
// Bounded wait for a chunk's arrival flag: about 2^21 polls of ~1 us (the
// context's wait limits can shorten it: rrCudaSetWaitLimits).  After
// one lane has given up (the copy never landed), every later wait fails at
// once, so a stuck copy costs one timeout, not one per ray.
//
// The polls are relaxed loads, not acquire loads: an acquire at gpu scope
// would drop the SM's L1 (and with it the cached upper tree levels) each
// time.  Ordering rests on three facts: the flag is written by the copy
// stream after the chunk's copy with a system-wide fence before it; the ray
// loads are control-dependent on the flag value (issued only after it
// returned); and they are L2 loads (ld.cg), so no stale L1 line can serve
// them.  Chunks arrive in order, so a warp that saw chunk c need not check
// any chunk <= c again.
constexpr uint32_t kArrivalPolls = 1u << 21;

// Highest chunk known to have arrived, starting the search at chunk `hi`
// (not yet known): flags are read four at a time (the words are 256-byte
// aligned), so one poll usually also covers the next few chunks, which the
// copy stream has landed by then.  Returns -1 if chunk `hi` never arrived.
__device__ __noinline__ static int wait_arrival(const TraceArgs& a, uint32_t hi)
{
    const uint32_t  g       = hi & ~3u;
    const uint4*    quad    = reinterpret_cast<const uint4*>(a.stream_words + g);
    const uint32_t* gave_up = a.stream_words + a.stream_chunks + a.stream_parts;
    const uint32_t  polls   = a.stream_polls ? a.stream_polls : kArrivalPolls;
    for (uint32_t k = 0; k < polls; ++k)
    {
        uint4 f;
        asm volatile("ld.relaxed.gpu.global.v4.u32 {%0, %1, %2, %3}, [%4];"
                     : "=r"(f.x), "=r"(f.y), "=r"(f.z), "=r"(f.w)
                     : "l"(quad)
                     : "memory");
        const uint32_t got[4] = {f.x, f.y, f.z, f.w};
        if (got[hi - g])
        {
            // Chunks arrive in order: the highest set flag of the quad (at
            // most the last chunk) bounds every chunk below it.
            int top = (int)hi;
            for (uint32_t j = hi - g + 1; j < 4 && g + j < a.stream_chunks; ++j)
                if (got[j]) top = (int)(g + j);
            return top;
        }
        uint32_t stop;
        asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(stop) : "l"(gave_up) : "memory");
        if (stop) return -1;
        __nanosleep(1000);
    }
    atomicExch(const_cast<uint32_t*>(gave_up), 1u);
    raise_error(a.words, RR_CUDA_DEVICE_ERROR_WAIT_TIMEOUT);
    return -1;
}

// Chunk c's done counter += v, ordered after every hit write of the warp's
// lanes that passed an earlier __syncwarp (release at gpu scope).  Out of
// line, like wait_arrival: rarely run, and kept out of the loop's code.
__device__ __noinline__ static void add_release(uint32_t* p, uint32_t v)
{
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Done counts of a warp, kept by claims: a warp counts the rays it claims in
// the part (copy-out unit, several arrival chunks) it is claiming from (cur)
// and in the one before it (prev), and publishes `prev` when its claims move
// on to a later part, both once the rays are exhausted.  A ray the warp
// still holds when it publishes the ray's part (in flight, or finished with
// its hit not yet written) is late-listed: its index goes to the late list,
// and the late scatter after the kernel (launch_late_scatter), which runs
// after every part's copy, brings its hit to the host.  Every other ray of
// the part finished earlier, and its hit was written before the loop's
// __syncwarp that precedes the release add.  So a part's counter reaches
// its size about two parts behind the claim front, however long its slowest
// rays take, and the last parts leave while the kernel drains.
// A release add waits until the SM's earlier stores are visible, which costs
// microseconds, so a warp issues one about once per part it works on.  The
// counts live in shared memory (one record per warp, written by one lane at
// a time: the refill's claiming lane, or lane 0 at exhaustion) so that no
// register stays live across the traversal step for them.
struct DoneCounts
{
    uint32_t cur_c, cur_n, prev_c, prev_n, fin;
};

// Appends the rays of the lanes in m (warp-uniform, non-zero) to the late
// list; `mine` is this lane's bit of m.
__device__ __forceinline__ void late_append(const TraceArgs& a, uint32_t m, bool mine, uint32_t gid, uint32_t lane)
{
    const int leader = __ffs(m) - 1;
    uint32_t  base   = 0;
    if ((int)lane == leader) base = atomicAdd(a.stream_words + a.stream_chunks + a.stream_parts + 1, (uint32_t)__popc(m));
    base                = __shfl_sync(0xffffffffu, base, leader);
    const uint32_t slot = base + __popc(m & ((1u << lane) - 1u));
    if (mine && slot < a.ray_count) a.stream_late[slot] = gid;
}

// What the lane that claimed a refill's rays tells its warp (claim_leader).
struct ClaimNote
{
    int      seen;       // highest chunk known to have arrived
    uint32_t late_part;  // part just published (its held rays are late-listed), or kInvalid
    uint32_t jump_end;   // new rays below this lie in neither open part (0: none)
};

// Run by the lane that claimed rays [base, end) at a refill, right after its
// atomic: waits (bounded, once per block and chunk) for the arrival of the
// claim's last chunk, then keeps the warp's claim counts.  A claim spans at
// most two parts (it is at most 32 rays; a part is at least 2^15).  When it
// reaches a part beyond cur, prev is published and the counts shift; the
// warp then late-lists the rays it holds in the published part
// (late_held: their hits, written later, reach the host through the late
// scatter).  The new rays are counted in cur, or in prev when they lie
// there; rays in neither (the claim skipped a whole part, so this warp will
// not publish theirs) are counted and late-listed at once (jump_done).
// One lane does all of it, so the refill pays for one divergent block.
__device__ __forceinline__ ClaimNote claim_leader(const TraceArgs& a, uint32_t base, uint32_t end, int* s_seen,
                                                  volatile DoneCounts& d)
{
    ClaimNote      c;
    const int      hc  = (int)((end - 1u) >> a.stream_shift);
    int            top = *reinterpret_cast<volatile int*>(s_seen);
    if (top < hc)
    {
        top = wait_arrival(a, (uint32_t)hc);
        if (top >= 0) atomicMax(s_seen, top);
    }
    c.seen              = top;
    const uint32_t ps   = a.stream_part_shift;
    const uint32_t hi   = (end - 1u) >> ps, lo = base >> ps;
    const uint32_t cur_c = d.cur_c;
    c.late_part          = kInvalid;
    if (hi > cur_c)
    {
        const uint32_t prev_c = d.prev_c, prev_n = d.prev_n;
        if (prev_n) add_release(a.stream_words + a.stream_chunks + prev_c, prev_n);
        c.late_part = prev_c;
        d.prev_c    = cur_c;
        d.prev_n    = d.cur_n;
        d.cur_c     = hi;
        d.cur_n     = 0;
    }
    const uint32_t hs      = hi << ps;
    const bool     in_prev = base < hs && lo == cur_c;  // cur_c is prev now
    c.jump_end             = base < hs && !in_prev ? hs : 0u;
    d.cur_n                = d.cur_n + (end - max(base, hs));
    if (in_prev) d.prev_n = d.prev_n + (hs - base);
    return c;
}

// All lanes, after a claim published part p (ClaimNote::late_part): the
// rays the warp still holds there (in flight, or finished with the hit not
// yet written: `holds`) go to the late list.
__device__ __forceinline__ void late_held(const TraceArgs& a, bool holds, uint32_t gid, uint32_t p, uint32_t lane)
{
    const bool     late = holds && (gid >> a.stream_part_shift) == p;
    const uint32_t lm   = __ballot_sync(0xffffffffu, late);
    if (lm) late_append(a, lm, late, gid, lane);
}

// The new rays below jump_end (claim_leader) are counted and late-listed at
// once; `fresh`: the lane took a new ray at this refill.  Warp-uniform call.
__device__ __forceinline__ void jump_done(const TraceArgs& a, bool fresh, uint32_t gid, uint32_t jump_end,
                                          uint32_t lane)
{
    const bool     late = fresh && gid < jump_end;
    const uint32_t lm   = __ballot_sync(0xffffffffu, late);
    if (!lm) return;
    late_append(a, lm, late, gid, lane);
    if ((int)lane == __ffs(lm) - 1)
        add_release(a.stream_words + a.stream_chunks + ((jump_end - 1u) >> a.stream_part_shift), (uint32_t)__popc(lm));
}

// The warp's claims are exhausted (warp-uniform call at each refill after
// that): once, late-list every ray it holds in prev or cur and publish both
// counts.  Later finishes need no bookkeeping.
__device__ __forceinline__ void finalize_done(const TraceArgs& a, bool holds, uint32_t gid, uint32_t lane,
                                              volatile DoneCounts& d)
{
    if (d.fin) return;
    const uint32_t rc   = gid >> a.stream_part_shift;
    const bool     late = holds && (rc == d.cur_c || rc == d.prev_c);
    const uint32_t lm   = __ballot_sync(0xffffffffu, late);
    if (lm) late_append(a, lm, late, gid, lane);
    __syncwarp();
    if (lane == 0)
    {
        if (d.cur_n) add_release(a.stream_words + a.stream_chunks + d.cur_c, d.cur_n);
        if (d.prev_n) add_release(a.stream_words + a.stream_chunks + d.prev_c, d.prev_n);
        d.cur_n = d.prev_n = 0;
        d.fin   = 1;
    }
    __syncwarp();
}

// A streamed ray's 32 bytes, read through L2 only: a neighbouring chunk may
// share a sector with it and must not be served stale from L1.
__device__ __forceinline__ Ray load_ray_cg(const uint8_t* rays, uint32_t i)
{
    const float4* p = reinterpret_cast<const float4*>(rays) + 2ull * i;
    const float4  x = __ldcg(p), y = __ldcg(p + 1);
    return Ray{f3(x.x, x.y, x.z), x.w, f3(y.x, y.y, y.z), y.w};
}

}  // namespace stream_detail
}  // namespace rr
