// trace_persistent.cuh -- per-lane state machine of the persistent binary
// traversal, shared by the single-batch kernel (trace_persistent.cu) and the
// multi-request kernel (trace_batch.cu).
//
// The per-ray algorithm is the reference's (vlk/kernels/isect.comp:105-245):
// the same slab and triangle arithmetic (trace_common.cuh), near child first
// (child 1 iff it is hit and child 0's entry distance is larger), a LIFO stack
// of deferred children, strict `t < closest_t` accept.  The visit order is
// therefore exactly the reference's and the hits are bit-identical to the
// plain kernel and to the oracle, ties and any-hit choices included.
#pragma once
#include "rr_internal.h"
#include "trace_common.cuh"
#include "trace_precise.cuh"

namespace rr
{
constexpr int      kPBlock     = 128;
// Shared short-stack entries per thread.  16 rather than 32: 8 KB per block
// leaves 64 KB more of each SM's L1 for node data (+2% on incoherent rays).
constexpr int      kPShort     = 16;
constexpr uint32_t kPSpillCap  = 256;  // global spill entries per thread (binary LBVH depth <= 64)
constexpr uint32_t kPRefillMin = 8;    // idle lanes that trigger a refill

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
    int       depth = kPShort;  // short-stack entries (the 4-wide kernels' helpers read it)
    __device__ __forceinline__ uint32_t& at(int k) const { return s[k * kPBlock]; }
};

// kPrecise: the precise triangle test's traversal (trace_precise.cuh): the
// exact reciprocal of the direction and slab distances (p - o) * inv.
template <bool kPrecise = false>
__device__ __forceinline__ void p_start(PRay& s, const Ray& r)
{
    s.ray   = r;
    s.inv   = kPrecise ? exact_invdir(s.ray.d) : safe_invdir(s.ray.d);
    s.oxi   = f3(-s.ray.o.x * s.inv.x, -s.ray.o.y * s.inv.y, -s.ray.o.z * s.inv.z);
    s.ct    = s.ray.tmax;
    s.caddr = kInvalid;
    s.addr  = 0;
    s.gsp = s.steps = 0;
    s.sp            = 0;
}
template <bool kPrecise = false>
__device__ __forceinline__ void p_start(PRay& s, const uint8_t* rays, uint32_t i)
{
    p_start<kPrecise>(s, load_ray(rays, i));
}

// One iteration of the reference's traversal loop.  Returns true when the ray
// is finished (stack empty, or a hit accepted by an any-hit query).  The
// query is kAny, or `any` when kRuntime (requests of both kinds mixed); the
// leaves are boxes (AABB-list geometry) when kBox, or `box` when kRuntime.
// kPrecise: the conservative box test and the precise triangle test
// (trace_precise.cuh) in the same visit order.
template <bool kAny, bool kRuntime = false, bool kBox = false, bool kPrecise = false>
__device__ __forceinline__ bool p_step(PRay& s, const BvhNode* __restrict__ nodes, uint32_t node_limit,
                                       const PStack& st, DeviceWords* words, uint32_t& nf, bool any = false,
                                       bool box = false)
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
        if (kPrecise)
        {
            isect_box_robust(nd.l0, nd.h0, s.inv, s.ray.o, s.ct, s.ray.tmin, a0, a1);
            isect_box_robust(nd.l1, nd.h1, s.inv, s.ray.o, s.ct, s.ray.tmin, b0, b1);
        }
        else
        {
            isect_box(nd.l0, nd.h0, s.inv, s.oxi, s.ct, s.ray.tmin, a0, a1);
            isect_box(nd.l1, nd.h1, s.inv, s.oxi, s.ct, s.ray.tmin, b0, b1);
        }
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
        const float t = (kBox || (kRuntime && box)) ? isect_leaf_box(s.ray, s.inv, s.oxi, nd.l0, nd.h0, s.ct)
                        : kPrecise                  ? isect_tri_precise(s.ray, nd.l0, nd.h0, nd.l1, s.ct)
                                                    : isect_tri(s.ray, nd.l0, nd.h0, nd.l1, s.ct);
        if (t < s.ct)
        {
            s.ct    = t;
            s.caddr = s.addr;
            if (kAny || (kRuntime && any)) done = true;
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

// Grid of a persistent launch: resident blocks on every SM, no more threads
// than rays (rounded to warps), and the spill entries per thread that fit the
// scratch after its header (a multiple of kPShort, at most kPSpillCap).
struct PGrid
{
    int      blocks;
    uint32_t gcap;
};
inline PGrid persistent_grid(int sm_count, int per_sm, uint64_t rays, size_t scratch_bytes, size_t header)
{
    uint64_t       threads = (uint64_t)sm_count * per_sm * kPBlock;
    const uint64_t need    = (rays + 31) / 32 * 32;
    if (threads > need) threads = (need + kPBlock - 1) / kPBlock * kPBlock;
    PGrid g;
    g.blocks = (int)(threads / kPBlock);
    threads  = (uint64_t)g.blocks * kPBlock;
    uint64_t gcap = scratch_bytes > header ? (scratch_bytes - header) / (threads * sizeof(uint32_t)) : 0;
    gcap          = gcap / kPShort * kPShort;
    if (gcap > kPSpillCap) gcap = kPSpillCap;
    g.gcap = (uint32_t)gcap;
    return g;
}

}  // namespace rr
