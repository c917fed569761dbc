// trace_persistent.cu -- persistent lane-refill traversal over the reference's
// 64-byte binary nodes.
//
// The per-ray algorithm is the reference's (vlk/kernels/isect.comp:105-245):
// the same slab and triangle arithmetic (trace_common.cuh), near child first
// (child 1 iff it is hit and child 0's entry distance is larger), a LIFO stack
// of deferred children, strict `t < closest_t` accept.  The visit order is
// therefore exactly the reference's and the hits are bit-identical to the
// plain kernel and to the oracle, ties and any-hit choices included.
//
// What differs is the scheduling: a persistent grid whose lanes each advance
// their own ray one node per loop iteration and take the next ray from a
// counter as soon as their ray finishes (one warp-aggregated atomic per
// refill).  One thread per ray (the plain kernel) leaves most lanes of a warp
// idle while its longest ray finishes; refilling keeps them working.  The
// stack is a short stack in shared memory (interleaved across the block) that
// spills to a per-thread region of the caller's scratch buffer.
#include "rr_internal.h"
#include "trace_common.cuh"

namespace rr
{
namespace
{
constexpr int      kPBlock    = 128;
constexpr int      kPShort    = 32;   // shared short-stack entries per thread
constexpr uint32_t kPSpillCap = 256;  // global spill entries per thread (binary LBVH depth <= 64)
constexpr uint32_t kPRefillMin = 8;   // idle lanes that trigger a refill

struct PRay
{
    Ray      ray;
    F3       inv, oxi;
    float    ct;
    uint32_t caddr;  // leaf of the closest hit
    uint32_t addr;   // node to fetch next
    uint32_t gsp;    // entries spilled to global
    uint32_t steps;
    int      sp;     // entries in the short stack
};

struct PStack
{
    uint32_t* s;  // this thread's first short-stack entry (shared), entries kPBlock apart
    uint32_t* g;  // global spill region
    uint32_t  gcap;
    __device__ __forceinline__ uint32_t& at(int k) const { return s[k * kPBlock]; }
};

// One iteration of the reference's traversal loop.  Returns true when the ray
// is finished (stack empty, or a hit accepted by an any-hit query).
template <bool kAny>
__device__ __forceinline__ bool p_step(PRay& s, const BvhNode* __restrict__ nodes, uint32_t node_limit,
                                       const PStack& st, DeviceWords* words, uint32_t& nf)
{
    if (++s.steps > kFetchCap || s.addr >= node_limit)
    {
        raise_error(words, RR_CUDA_DEVICE_ERROR_NODE_RANGE);
        s.caddr = kInvalid;
        return true;
    }
    const NodeView nd = load_binary_node(nodes, s.addr);
    ++nf;
    // Single exit: the internal-node and leaf paths rejoin before the pop.
    bool pop = true, done = false;
    if (nd.child0 != kInvalid)
    {
        float a0, a1, b0, b1;
        isect_box(nd.l0, nd.h0, s.inv, s.oxi, s.ct, s.ray.tmin, a0, a1);
        isect_box(nd.l1, nd.h1, s.inv, s.oxi, s.ct, s.ray.tmin, b0, b1);
        const bool tc0 = a0 <= a1, tc1 = b0 <= b1;
        const bool c1f = tc1 && (a0 > b0);
        if (tc0 || tc1)
        {
            const bool     first1   = c1f || !tc0;
            const uint32_t next     = first1 ? nd.child1 : nd.child0;
            const uint32_t deferred = first1 ? nd.child0 : nd.child1;
            if (tc0 && tc1)
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
                st.at(s.sp++) = deferred;
            }
            s.addr = next;
            pop    = false;
        }
    }
    else
    {
        const float t = isect_tri(s.ray, nd.l0, nd.h0, nd.l1, s.ct);
        if (t < s.ct)
        {
            s.ct    = t;
            s.caddr = s.addr;
            if (kAny) done = true;
        }
    }
    if (pop && !done)
    {
        if (s.sp == 0 && s.gsp == 0)
            done = true;
        else
        {
            if (s.sp == 0)
            {
                s.gsp -= kPShort;
                for (int k = 0; k < kPShort; ++k) st.at(k) = st.g[s.gsp + k];
                s.sp = kPShort;
            }
            s.addr = st.at(--s.sp);
        }
    }
    return done;
}

template <bool kAny, bool kFull, bool kStats>
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
    for (;;)
    {
        __syncwarp();
        // Lanes whose ray finished write its hit and take a new ray together,
        // once at least kPRefillMin lanes are idle (or no ray is left).
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
                        const NodeView nd = load_binary_node(nodes, s.caddr);
                        write_hit<kFull>(a.hits, gid, s.ray, s.ct, nd.l0, nd.h0, nd.l1, 0u, nd.child1, nd.child1);
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
                        active  = true;
                        nf      = 0;
                        s.ray   = load_ray(a.rays, gid);
                        s.inv   = safe_invdir(s.ray.d);
                        s.oxi   = f3(-s.ray.o.x * s.inv.x, -s.ray.o.y * s.inv.y, -s.ray.o.z * s.inv.z);
                        s.ct    = s.ray.tmax;
                        s.caddr = kInvalid;
                        s.addr  = 0;
                        s.gsp = s.steps = 0;
                        s.sp            = 0;
                    }
                }
            }
        }
        const uint32_t amask = __ballot_sync(0xffffffffu, active);
        if (amask == 0 && exhausted && __ballot_sync(0xffffffffu, pending) == 0) break;
        if (active && p_step<kAny>(s, nodes, a.node_limit, st, a.words, nf))
        {
            active  = false;
            pending = true;
        }
    }
}

template <bool kAny, bool kFull, bool kStats>
cudaError_t go(const TraceArgs& a, cudaStream_t s)
{
    auto kern   = k_trace_persistent<kAny, kFull, kStats>;
    int  per_sm = a.blocks_per_sm;
    if (per_sm <= 0)
    {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kPBlock, 0) != cudaSuccess) per_sm = 1;
        per_sm = per_sm > 0 ? per_sm : 1;
    }
    uint64_t       threads = (uint64_t)a.sm_count * per_sm * kPBlock;
    const uint64_t need    = ((uint64_t)a.ray_count + 31) / 32 * 32;
    if (threads > need) threads = (need + kPBlock - 1) / kPBlock * kPBlock;
    const int      blocks = (int)(threads / kPBlock);
    threads               = (uint64_t)blocks * kPBlock;
    uint64_t gcap = (a.scratch_bytes - kTraceScratchHeader) / (threads * sizeof(uint32_t));
    gcap          = gcap / kPShort * kPShort;
    if (gcap > kPSpillCap) gcap = kPSpillCap;
    cudaError_t e = cudaMemsetAsync(a.scratch, 0, kTraceScratchHeader, s);
    if (e != cudaSuccess) return e;
    kern<<<blocks, kPBlock, 0, s>>>(a, (uint32_t)gcap);
    return cudaGetLastError();
}
}  // namespace

cudaError_t launch_trace_persistent(const TraceArgs& a, cudaStream_t s)
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
