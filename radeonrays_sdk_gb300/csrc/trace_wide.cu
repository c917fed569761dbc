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
constexpr uint32_t kRayOrderMin  = 1u << 20;  // batches from this size are sorted before traversal
constexpr uint64_t kWideSpillCap = 128;       // spill entries per thread (groups; depth <= tree depth)
constexpr uint32_t kRefillMin    = 8;         // idle lanes that trigger a refill (measured best of 1/4/8/16)

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

// Ray ordering key: direction octant (3 bits) above the 27-bit Morton code of
// the origin in the mesh box (9 bits per axis).  Rays that start close
// together and head the same way become neighbours in the traversal order,
// so a warp's lanes walk similar nodes and share cache lines.
__device__ __forceinline__ uint32_t spread9(uint32_t v)
{
    v &= 0x1ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}
__device__ __forceinline__ float unord_bound(uint32_t u)
{
    u ^= (((u >> 31) - 1u) | 0x80000000u);
    return __uint_as_float(u);
}

__global__ void __launch_bounds__(256) k_ray_keys(const uint8_t* __restrict__ rays, uint32_t n,
                                                  const uint32_t* __restrict__ bounds, uint32_t* __restrict__ keys)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4* p  = reinterpret_cast<const float4*>(rays) + 2ull * i;
    const float4  o  = __ldg(p), d = __ldg(p + 1);
    const float   lx = unord_bound(bounds[0]), ly = unord_bound(bounds[1]), lz = unord_bound(bounds[2]);
    const float   ex = unord_bound(bounds[4]) - lx, ey = unord_bound(bounds[5]) - ly, ez = unord_bound(bounds[6]) - lz;
    const float   s  = 511.0f;
    const uint32_t x = (uint32_t)fminf(fmaxf((o.x - lx) / ex * s, 0.f), s);
    const uint32_t y = (uint32_t)fminf(fmaxf((o.y - ly) / ey * s, 0.f), s);
    const uint32_t z = (uint32_t)fminf(fmaxf((o.z - lz) / ez * s, 0.f), s);
    const uint32_t oct = (d.x < 0.f ? 4u : 0u) | (d.y < 0.f ? 2u : 0u) | (d.z < 0.f ? 1u : 0u);
    keys[i] = (oct << 27) | (spread9(x) << 2) | (spread9(y) << 1) | spread9(z);
}

template <bool kAny, bool kFull, bool kStats>
__global__ void __launch_bounds__(kWideBlock, 8) k_trace_wide(TraceArgs a, uint32_t gcap, const uint32_t* __restrict__ order)
{
    extern __shared__ WideEntry s_stack[];
    const uint32_t tglob = blockIdx.x * blockDim.x + threadIdx.x;
    WideStack      st;
    st.s    = s_stack + threadIdx.x;
    st.g    = reinterpret_cast<WideEntry*>(a.scratch + kTraceScratchHeader) + (uint64_t)tglob * gcap;
    st.gcap = gcap;
    uint32_t*      ray_ctr = reinterpret_cast<uint32_t*>(a.scratch);
    const uint32_t lane    = threadIdx.x & 31;
    const uint32_t lt      = (1u << lane) - 1u;
    uint32_t       count   = a.ray_count;
    if (a.indirect) count = min(count, __ldg(a.indirect));

    WideRay  s;
    uint32_t gid = kInvalid, nf = 0, tf = 0;
    bool     active = false, pending = false, exhausted = false;
    for (;;)
    {
        __syncwarp();
        // Lanes whose ray finished write its hit and take a new ray together,
        // once at least kRefillMin lanes are idle (or no ray is left to trace).
        const uint32_t idle  = __ballot_sync(0xffffffffu, !active);
        const uint32_t amask0 = ~idle;
        if (idle && (__popc(idle) >= kRefillMin || exhausted || amask0 == 0))
        {
            uint32_t base = 0;
            const uint32_t n = exhausted ? 0u : __popc(idle);
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
                    finish<kAny, kFull>(a, gid, s);
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
                    gid    = order ? __ldg(order + my) : my;
                    active = true;
                    nf = tf = 0;
                    wide_begin(s, load_ray(a.rays, gid), a.empty != 0);
                }
            }
        }
        const uint32_t amask = __ballot_sync(0xffffffffu, active);
        if (amask == 0 && exhausted && __ballot_sync(0xffffffffu, pending) == 0) break;
        if (active &&
            wide_step<kAny>(s, a.wide_nodes, a.wide_tris, a.wide_limit, a.tri_limit, st, a.words, nf, tf, amask))
        {
            active  = false;
            pending = true;
        }
    }
}

template <bool kAny, bool kFull, bool kStats>
cudaError_t go(const TraceArgs& a, cudaStream_t s)
{
    auto         kern  = k_trace_wide<kAny, kFull, kStats>;
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
    const int blocks = (int)(threads / block);
    threads          = (uint64_t)blocks * block;

    // Scratch: header | per-thread spill stacks | (optional) ray-ordering sort.
    const uint64_t avail = a.scratch_bytes - kTraceScratchHeader;
    bool           sort  = a.bounds && !a.indirect && a.ray_count >= kRayOrderMin && a.ray_order == 2;
    size_t         sort_bytes = 0, s_keys = 0, s_keys_alt = 0, s_idx = 0, s_idx_alt = 0, s_sort = 0;
    uint32_t       tiles = 0, passes = 0;
    if (sort)
    {
        const size_t r = a.ray_count;
        s_keys_alt     = align_up(4 * r, kAlign);
        s_idx          = s_keys_alt + align_up(4 * r, kAlign);
        s_idx_alt      = s_idx + align_up(4 * r, kAlign);
        s_sort         = s_idx_alt + align_up(4 * r, kAlign);
        sort_bytes     = s_sort + radix_sort_scratch_bytes(a.ray_count, 30, &tiles, &passes);
        if (sort_bytes + threads * 64 * sizeof(WideEntry) > avail) sort = false;
    }
    uint64_t gcap = (avail - (sort ? sort_bytes : 0)) / (threads * sizeof(WideEntry));
    gcap          = gcap / kWideShortStack * kWideShortStack;
    if (gcap > kWideSpillCap) gcap = kWideSpillCap;
    cudaError_t e = cudaMemsetAsync(a.scratch, 0, kTraceScratchHeader, s);
    if (e != cudaSuccess) return e;
    const uint32_t* order = nullptr;
    if (sort)
    {
        uint8_t* base = a.scratch + kTraceScratchHeader + align_up(threads * gcap * sizeof(WideEntry), kAlign);
        uint32_t *keys = reinterpret_cast<uint32_t*>(base + s_keys), *keys_alt = reinterpret_cast<uint32_t*>(base + s_keys_alt);
        uint32_t *idx = reinterpret_cast<uint32_t*>(base + s_idx), *idx_alt = reinterpret_cast<uint32_t*>(base + s_idx_alt);
        k_ray_keys<<<(a.ray_count + 255) / 256, 256, 0, s>>>(a.rays, a.ray_count, a.bounds, keys);
        bool alt = false;
        e = launch_radix_sort(keys, keys_alt, idx, idx_alt, a.ray_count, 30, base + s_sort, tiles, a.words, s, &alt);
        if (e != cudaSuccess) return e;
        order = alt ? idx_alt : idx;
    }
    kern<<<blocks, block, smem, s>>>(a, (uint32_t)gcap, order);
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
