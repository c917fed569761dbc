// trace_binary.cu -- "plain" traversal: one thread per ray over the 64-byte
// binary nodes, in the reference's visit order (vlk/kernels/isect.comp:88-246).
//
// Kept from the reference on purpose (this kernel is the baseline the wide
// path is measured against): 128-thread blocks, a 16-entry shared-memory stack
// per ray that spills 15 entries at a time to a 64-entry per-ray stack in the
// caller's scratch buffer, near-child-first order (child 1 first iff it is
// hit and child 0's entry distance is larger), strict `t < closest_t` accept,
// barycentrics recomputed from the hit point.  Arithmetic is the oracle's
// (IEEE fp32, fma only in the slab test, no contraction: --fmad=false), so
// hits are bit-identical to the CPU restatement.
//
// Differences from the reference: a ray whose stack would leave its 64-entry
// scratch slot raises RR_CUDA_DEVICE_ERROR_STACK_OVERFLOW instead of writing
// into the next ray's slot; the indirect count is clamped to ray_count.
#include "rr_internal.h"
#include "trace_common.cuh"

namespace rr
{
namespace
{
constexpr int kBlock    = 128;
constexpr int kLdsStack = 16;
constexpr int kGlobalStack = 64;

template <bool kAny, bool kFull, bool kStats>
__global__ void __launch_bounds__(kBlock) k_trace_binary(TraceArgs a)
{
    __shared__ uint32_t lds[kBlock * kLdsStack];
    const uint32_t      gid   = blockIdx.x * kBlock + threadIdx.x;
    uint32_t            count = a.ray_count;
    if (a.indirect) count = min(count, __ldg(a.indirect));
    if (gid >= count) return;

    const BvhNode* nodes = reinterpret_cast<const BvhNode*>(a.bvh);
    Ray            ray   = load_ray(a.rays, gid);
    const F3       inv   = safe_invdir(ray.d);
    const F3       oxi   = f3(-ray.o.x * inv.x, -ray.o.y * inv.y, -ray.o.z * inv.z);
    float          ct    = ray.tmax;
    uint32_t       caddr = kInvalid;
    uint32_t       fetches = 0;

    uint32_t* gstack = reinterpret_cast<uint32_t*>(a.scratch + kTraceScratchHeader) + (uint64_t)gid * kGlobalStack;
    uint32_t  sptr   = 0;  // entries spilled (multiple of 16)
    const uint32_t bottom = threadIdx.x * kLdsStack;
    uint32_t       lsp    = bottom;
    lds[lsp++]            = kInvalid;
    uint32_t addr         = a.empty ? kInvalid : 0u;

    while (addr != kInvalid)
    {
        if (addr >= a.node_limit || fetches >= kFetchCap)
        {
            raise_error(a.words, RR_CUDA_DEVICE_ERROR_NODE_RANGE);
            caddr = kInvalid;
            break;
        }
        const NodeView nd = load_binary_node(nodes, addr);
        ++fetches;
        if (nd.child0 != kInvalid)
        {
            float a0, a1, b0, b1;
            isect_box(nd.l0, nd.h0, inv, oxi, ct, ray.tmin, a0, a1);
            isect_box(nd.l1, nd.h1, inv, oxi, ct, ray.tmin, b0, b1);
            const bool tc0 = a0 <= a1, tc1 = b0 <= b1;
            const bool c1f = tc1 && (a0 > b0);
            if (tc0 || tc1)
            {
                uint32_t deferred;
                if (c1f || !tc0)
                {
                    addr     = nd.child1;
                    deferred = nd.child0;
                }
                else
                {
                    addr     = nd.child0;
                    deferred = nd.child1;
                }
                if (tc0 && tc1)
                {
                    if (lsp - bottom >= kLdsStack)
                    {
                        if (sptr + kLdsStack > kGlobalStack)
                        {
                            atomicOr(&a.words->error_bits, (uint32_t)RR_CUDA_DEVICE_ERROR_STACK_OVERFLOW);
                            continue;  // drop the deferred child: result flagged invalid
                        }
                        for (int i = 1; i < kLdsStack; ++i) gstack[sptr + i] = lds[bottom + i];
                        sptr += kLdsStack;
                        lsp = bottom + 1;
                    }
                    lds[lsp++] = deferred;
                }
                continue;
            }
        }
        else
        {
            const float t = a.box_leaves ? isect_leaf_box(ray, inv, oxi, nd.l0, nd.h0, ct)
                                         : isect_tri(ray, nd.l0, nd.h0, nd.l1, ct);
            if (t < ct)
            {
                if (!kAny)
                {
                    ct    = t;
                    caddr = addr;
                }
                else
                {
                    if (a.box_leaves)
                        write_box_hit<kFull>(a.hits, gid, 0u, nd.child1, nd.child1);
                    else
                        write_hit<kFull>(a.hits, gid, ray, t, nd.l0, nd.h0, nd.l1, 0u, nd.child1, nd.child1);
                    if (kStats) add_stats(a.words, fetches, 0);
                    return;
                }
            }
        }
        addr = lds[--lsp];
        if (addr == kInvalid && sptr > 0)
        {
            sptr -= kLdsStack;
            for (int i = 1; i < kLdsStack; ++i) lds[bottom + i] = gstack[sptr + i];
            lsp  = bottom + kLdsStack - 1;
            addr = lds[lsp];
        }
    }

    if (caddr != kInvalid)
    {
        const NodeView nd = load_binary_node(nodes, caddr);
        if (a.box_leaves)
            write_box_hit<kFull>(a.hits, gid, 0u, nd.child1, nd.child1);
        else
            write_hit<kFull>(a.hits, gid, ray, ct, nd.l0, nd.h0, nd.l1, 0u, nd.child1, nd.child1);
    }
    else
        write_miss<kFull>(a.hits, gid);
    if (kStats) add_stats(a.words, fetches, 0);
}

template <bool kAny, bool kFull, bool kStats>
cudaError_t go(const TraceArgs& a, cudaStream_t s)
{
    const int blocks = (int)((a.ray_count + kBlock - 1) / kBlock);
    k_trace_binary<kAny, kFull, kStats><<<blocks, kBlock, 0, s>>>(a);
    return cudaGetLastError();
}
}  // namespace

cudaError_t launch_trace_binary(const TraceArgs& a, cudaStream_t s)
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

size_t trace_scratch_bytes(uint32_t ray_count)
{
    // 256 bytes per ray (the reference's figure, vlk/geometry_trace.cpp:169),
    // and never less than for 4096 rays so the persistent wide kernel always
    // has a deep spill region per thread.
    const size_t rays = ray_count < 4096u ? 4096u : ray_count;
    return kTraceScratchHeader + rays * kGlobalStack * sizeof(uint32_t);
}

}  // namespace rr
