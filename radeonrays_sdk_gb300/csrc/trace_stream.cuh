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

// Done counts of a warp: rays finished in the part (copy-out unit, several
// arrival chunks) the warp is claiming from (cur) and in the one before it
// (prev), not yet added to the parts' done counters.  `prev` is published
// when the warp's claims move on to a later part, both at exit; a ray of any
// other part (a straggler) is added at once.  A release add waits until the
// SM's earlier stores are visible, which costs microseconds, so a warp
// issues one about once per part it works on, not at every refill.  The
// counts live in shared memory (one record per warp, written by lane 0 only)
// so that no register stays live across the traversal step for them.
struct DoneCounts
{
    uint32_t cur_c, cur_n, prev_c, prev_n;
};

// Rays finished at this refill (`fin`, part `c`); all 32 lanes call it,
// after their hits are written.
__device__ __forceinline__ void note_done(const TraceArgs& a, bool fin, uint32_t c, uint32_t lane,
                                          volatile DoneCounts& d)
{
    if (!__ballot_sync(0xffffffffu, fin)) return;
    const uint32_t cur_c = d.cur_c, prev_c = d.prev_c;
    const uint32_t in_cur  = __ballot_sync(0xffffffffu, fin && c == cur_c);
    const uint32_t in_prev = __ballot_sync(0xffffffffu, fin && c == prev_c && prev_c != cur_c);
    if (lane == 0)
    {
        d.cur_n  = d.cur_n + __popc(in_cur);
        d.prev_n = d.prev_n + __popc(in_prev);
    }
    if (fin && !(((in_cur | in_prev) >> lane) & 1u)) add_release(a.stream_words + a.stream_chunks + c, 1u);
    __syncwarp();
}

// The warp's claims reached part `hi` (warp-uniform): publish `prev` and
// shift.  The counted hits were written before the loop's __syncwarp.
__device__ __forceinline__ void advance_done(const TraceArgs& a, uint32_t hi, uint32_t lane, volatile DoneCounts& d)
{
    if (lane != 0 || hi <= d.cur_c) return;
    if (d.prev_n) add_release(a.stream_words + a.stream_chunks + d.prev_c, d.prev_n);
    d.prev_c = d.cur_c;
    d.prev_n = d.cur_n;
    d.cur_c  = hi;
    d.cur_n  = 0;
}

// Publish both open counts (lane 0); after a __syncwarp that follows the
// counted hits' writes.
__device__ __forceinline__ void publish_done(const TraceArgs& a, uint32_t lane, volatile DoneCounts& d)
{
    if (lane == 0)
    {
        if (d.cur_n) add_release(a.stream_words + a.stream_chunks + d.cur_c, d.cur_n);
        if (d.prev_n && d.prev_c != d.cur_c) add_release(a.stream_words + a.stream_chunks + d.prev_c, d.prev_n);
        d.cur_n = d.prev_n = 0;
    }
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
