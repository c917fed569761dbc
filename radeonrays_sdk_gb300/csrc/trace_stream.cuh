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
//
// With a late list (a.stream_late), a part is not held open by its slowest
// rays: when the warp publishes a part, a ray it still holds there (in
// flight, or finished with its hit not yet written) is counted at once and
// its index late-listed; the same happens to every ray the warp holds once
// the rays are exhausted.  The copy-out of a part then follows the claim
// front by about two parts instead of waiting for its longest ray, and the
// last parts leave while the kernel drains.  A late-listed ray's hit reaches
// the host through the late scatter after the kernel (launch_late_scatter),
// which runs after every part's copy.  `defer` holds the lanes whose current
// ray is late-listed (not counted again when it finishes); `fin` is set once
// the warp has published everything at exhaustion.
struct DoneCounts
{
    uint32_t cur_c, cur_n, prev_c, prev_n, defer, fin;
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

// Rays finished at this refill (`fin`, part `c`); all 32 lanes call it,
// after their hits are written.  A late-listed ray is not counted again.
__device__ __forceinline__ void note_done(const TraceArgs& a, bool fin, uint32_t c, uint32_t lane,
                                          volatile DoneCounts& d)
{
    const uint32_t fm = __ballot_sync(0xffffffffu, fin);
    if (!fm) return;
    const uint32_t cur_c = d.cur_c, prev_c = d.prev_c, dm = d.defer;
    const bool     cnt     = fin && !((dm >> lane) & 1u);
    const uint32_t in_cur  = __ballot_sync(0xffffffffu, cnt && c == cur_c);
    const uint32_t in_prev = __ballot_sync(0xffffffffu, cnt && c == prev_c && prev_c != cur_c);
    if (lane == 0)
    {
        d.cur_n  = d.cur_n + __popc(in_cur);
        d.prev_n = d.prev_n + __popc(in_prev);
        d.defer  = dm & ~fm;
    }
    if (cnt && !(((in_cur | in_prev) >> lane) & 1u)) add_release(a.stream_words + a.stream_chunks + c, 1u);
    __syncwarp();
}

// The warp's claims reached part `hi` (warp-uniform): publish `prev` and
// shift.  The counted hits were written before the loop's __syncwarp.
// `holds`: the lane has a ray not yet counted (gid); with a late list, such a
// ray in a part that is not open after the shift is counted now (with prev
// when it lies there) and late-listed.  Rays the warp holds lie in parts up
// to cur (claimed earlier), so that is every held ray outside cur.
__device__ __forceinline__ void advance_done(const TraceArgs& a, uint32_t hi, bool holds, uint32_t gid, uint32_t lane,
                                             volatile DoneCounts& d)
{
    const uint32_t cur_c = d.cur_c;
    if (hi <= cur_c) return;
    const uint32_t prev_c = d.prev_c;
    uint32_t       nlate  = 0, lm = 0;
    if (a.stream_late)
    {
        const uint32_t rc   = gid >> a.stream_part_shift;
        const bool     late = holds && !((d.defer >> lane) & 1u) && rc != cur_c;
        lm                  = __ballot_sync(0xffffffffu, late);
        if (lm)
        {
            late_append(a, lm, late, gid, lane);
            const bool to_prev = late && rc == prev_c && prev_c != cur_c;
            nlate              = __popc(__ballot_sync(0xffffffffu, to_prev));
            if (late && !to_prev) add_release(a.stream_words + a.stream_chunks + rc, 1u);
        }
    }
    __syncwarp();
    if (lane != 0) return;
    const uint32_t n = d.prev_n + nlate;
    if (n) add_release(a.stream_words + a.stream_chunks + prev_c, n);
    d.defer  = d.defer | lm;
    d.prev_c = cur_c;
    d.prev_n = d.cur_n;
    d.cur_c  = hi;
    d.cur_n  = 0;
}

// With a late list: the warp's claims are exhausted (warp-uniform call at
// each refill after that): once, count and late-list every ray the warp
// still holds and publish both open counts.  Later finishes are all
// late-listed rays, so nothing is left to publish at exit.
__device__ __forceinline__ void finalize_done(const TraceArgs& a, bool holds, uint32_t gid, uint32_t lane,
                                              volatile DoneCounts& d)
{
    if (d.fin) return;
    const uint32_t cur_c = d.cur_c, prev_c = d.prev_c;
    const uint32_t rc      = gid >> a.stream_part_shift;
    const bool     late    = holds && !((d.defer >> lane) & 1u);
    const bool     in_cur  = late && rc == cur_c;
    const bool     in_prev = late && rc == prev_c && prev_c != cur_c;
    const uint32_t lm      = __ballot_sync(0xffffffffu, late);
    const uint32_t nc      = __popc(__ballot_sync(0xffffffffu, in_cur));
    const uint32_t np      = __popc(__ballot_sync(0xffffffffu, in_prev));
    if (lm) late_append(a, lm, late, gid, lane);
    if (late && !in_cur && !in_prev) add_release(a.stream_words + a.stream_chunks + rc, 1u);
    __syncwarp();
    if (lane == 0)
    {
        if (d.cur_n + nc) add_release(a.stream_words + a.stream_chunks + cur_c, d.cur_n + nc);
        if (d.prev_n + np) add_release(a.stream_words + a.stream_chunks + prev_c, d.prev_n + np);
        d.cur_n = d.prev_n = 0;
        d.defer = d.defer | lm;
        d.fin   = 1;
    }
    __syncwarp();
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
