// trace_wide.cu -- "chosen" single-level traversal over 8-wide nodes with 8-bit
// child bounds.
//
// No reference counterpart (the reference traverses binary nodes,
// vlk/kernels/isect.comp); the hit contract is the reference's:
//   * closest hit: the same fp32 triangle test as isect.comp (bit-identical t),
//     strict `t < closest_t` accept, uv recomputed from the hit point, so the
//     hit primitive equals the plain path's except for exact equal-t ties
//     reached in a different order;
//   * any hit: the first accepted triangle in this kernel's visit order;
//   * misses write only inst_id.
// Child boxes decode to fp32 boxes that contain the exact child boxes (see
// wide.cu), and the slab test is the reference's, so no hit that the exact
// box admits is culled.
//
// Scheduling: a persistent grid (SM count x resident blocks).  Every lane owns
// one ray at a time and advances it one node per loop iteration
// (trace_wide.cuh, wide_step); when a lane's ray finishes, it writes the hit
// and takes the next ray from a counter in the scratch header in the same
// iteration (one warp-aggregated atomic per refill).  Incoherent rays finish
// at very different times, so refilling keeps the warp's lanes busy instead of
// idling until the warp's longest ray ends.  Every node is five 128-bit
// read-only loads, every triangle three.
#include "rr_internal.h"
#include "trace_wide.cuh"

namespace rr
{
namespace
{
template <bool kAny, bool kFull>
__device__ __forceinline__ void finish(const TraceArgs& a, uint32_t gid, const WideRay& s)
{
    if (s.best != kInvalid)
    {
        const float4*  tp   = reinterpret_cast<const float4*>(a.wide_tris + s.best);
        const float4   A = __ldg(tp), B = __ldg(tp + 1), C = __ldg(tp + 2);
        const uint32_t prim = __float_as_uint(A.w);
        write_hit<kFull>(a.hits, gid, s.ray, s.ct, f3(A.x, A.y, A.z), f3(B.x, B.y, B.z), f3(C.x, C.y, C.z), 0u, prim,
                         prim);
    }
    else
        write_miss<kFull>(a.hits, gid);
}

template <bool kAny, bool kFull, bool kStats>
__global__ void k_trace_wide(TraceArgs a, uint32_t gcap)
{
    extern __shared__ WideEntry s_stack[];
    const uint32_t tglob = blockIdx.x * blockDim.x + threadIdx.x;
    WideStack      st;
    st.s    = s_stack + threadIdx.x * kWideShortStack;
    st.g    = reinterpret_cast<WideEntry*>(a.scratch + kTraceScratchHeader) + (uint64_t)tglob * gcap;
    st.gcap = gcap;
    uint32_t*      ray_ctr = reinterpret_cast<uint32_t*>(a.scratch);
    const uint32_t lane    = threadIdx.x & 31;
    const uint32_t lt      = (1u << lane) - 1u;
    uint32_t       count   = a.ray_count;
    if (a.indirect) count = min(count, __ldg(a.indirect));

    WideRay  s;
    uint32_t gid = kInvalid, nf = 0, tf = 0;
    bool     active = false, exhausted = false;
    for (;;)
    {
        const uint32_t idle = __ballot_sync(0xffffffffu, !active);
        if (idle && !exhausted)
        {
            const uint32_t n      = __popc(idle);
            const int      leader = __ffs(idle) - 1;
            uint32_t       base   = 0;
            if ((int)lane == leader) base = atomicAdd(ray_ctr, n);
            base      = __shfl_sync(0xffffffffu, base, leader);
            exhausted = base + n >= count;
            if (!active)
            {
                const uint32_t my = base + __popc(idle & lt);
                if (my < count)
                {
                    gid    = my;
                    active = true;
                    nf = tf = 0;
                    wide_begin(s, load_ray(a.rays, gid), a.empty != 0);
                }
            }
        }
        if (__ballot_sync(0xffffffffu, active) == 0) break;
        if (active && wide_step<kAny>(s, a.wide_nodes, a.wide_tris, a.wide_limit, a.tri_limit, st, a.words, nf, tf))
        {
            finish<kAny, kFull>(a, gid, s);
            if (kStats)
            {
                atomicAdd(&a.words->rays, 1ull);
                atomicAdd(&a.words->node_fetches, (unsigned long long)nf);
                atomicAdd(&a.words->tri_fetches, (unsigned long long)tf);
            }
            active = false;
        }
    }
}

template <bool kAny, bool kFull, bool kStats>
cudaError_t go(const TraceArgs& a, cudaStream_t s)
{
    auto         kern  = k_trace_wide<kAny, kFull, kStats>;
    const int    block = a.block_size > 0 ? a.block_size : 128;
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
    kern<<<blocks, block, smem, s>>>(a, (uint32_t)gcap);
    return cudaGetLastError();
}
}  // namespace

cudaError_t launch_trace_wide(const TraceArgs& a, cudaStream_t s)
{
    if (a.ray_count == 0) return cudaSuccess;
    const bool any = a.query == RR_INTERSECT_QUERY_ANY, full = a.output == RR_INTERSECT_QUERY_OUTPUT_FULL_HIT;
    if (a.collect_stats)
    {
        if (any) return full ? go<true, true, true>(a, s) : go<true, false, true>(a, s);
        return full ? go<false, true, true>(a, s) : go<false, false, true>(a, s);
    }
    if (any) return full ? go<true, true, false>(a, s) : go<true, false, false>(a, s);
    return full ? go<false, true, false>(a, s) : go<false, false, false>(a, s);
}

}  // namespace rr
