// wide.cu -- collapse of the binary LBVH into 8-wide nodes with 8-bit child
// bounds, or into 4-wide nodes with exact fp32 child boxes (traversal
// formats of this build; no reference counterpart: the reference traverses
// its binary nodes only, vlk/kernels/isect.comp).
//
// Collapse: top-down and level-synchronous.  A work item is (binary node b,
// wide slot w).  The children of w start as b's two children; the internal
// child with the largest surface area is replaced by its two children until
// there are W (8 or 4) children or only triangles remain.  A 4-wide node
// keeps each child's exact box and refers to leaf children by their binary
// leaf node; the 8-wide format is described below.  Internal children become
// the next level's work items; triangle children are written to a contiguous
// 48-byte triangle array.  Every level is one launch whose item count is read
// on the device, so the whole build records into a stream without a host
// round trip.
//
// Quantisation: per node, origin p = union box minimum; per axis the smallest
// power of two 2^e with ceil((hi - p) / 2^e) <= 255.  Child bounds are
// qlo = floor(rd(lo - p) / 2^e), qhi = ceil(ru(hi - p) / 2^e), so the decoded
// box fma(q, 2^e, p) contains the exact fp32 child box (round-to-nearest is
// monotonic and the bounds are floats).  A traversal slab test on the decoded
// box therefore never rejects a ray that the exact box accepts.
#include <algorithm>
#include <cstdlib>

#include "rr_internal.h"

namespace rr
{
namespace
{
constexpr int kMaxLevels = 66;

struct CollapseCtl
{
    uint32_t wide_count;
    uint32_t tri_count;
    uint32_t pad[2];
    uint32_t level_count[kMaxLevels + 2];
};

struct Item
{
    uint32_t b, w;
};

struct Bx
{
    float lo[3], hi[3];
};

__device__ __forceinline__ Bx node_union(const BvhNode& nd)
{
    Bx r;
    if (nd.child0 != kInvalid)
    {
        r.lo[0] = fminf(nd.a0[0], nd.b0[0]);
        r.lo[1] = fminf(nd.a0[1], nd.b0[1]);
        r.lo[2] = fminf(nd.a0[2], nd.b0[2]);
        r.hi[0] = fmaxf(nd.a1[0], nd.b1[0]);
        r.hi[1] = fmaxf(nd.a1[1], nd.b1[1]);
        r.hi[2] = fmaxf(nd.a1[2], nd.b1[2]);
    }
    else
    {
        for (int k = 0; k < 3; ++k)
        {
            r.lo[k] = fminf(fminf(nd.a0[k], nd.a1[k]), nd.b0[k]);
            r.hi[k] = fmaxf(fmaxf(nd.a0[k], nd.a1[k]), nd.b0[k]);
        }
    }
    return r;
}

__device__ __forceinline__ float half_area(const Bx& b)
{
    float x = b.hi[0] - b.lo[0], y = b.hi[1] - b.lo[1], z = b.hi[2] - b.lo[2];
    return x * y + y * z + z * x;
}

__device__ __forceinline__ BvhNode load_node(const BvhNode* nodes, uint32_t i)
{
    const float4* p = reinterpret_cast<const float4*>(nodes + i);
    float4        a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2), d = __ldg(p + 3);
    BvhNode       n;
    n.a0[0] = a.x;
    n.a0[1] = a.y;
    n.a0[2] = a.z;
    n.child0 = __float_as_uint(a.w);
    n.a1[0] = b.x;
    n.a1[1] = b.y;
    n.a1[2] = b.z;
    n.child1 = __float_as_uint(b.w);
    n.b0[0] = c.x;
    n.b0[1] = c.y;
    n.b0[2] = c.z;
    n.parent = __float_as_uint(c.w);
    n.b1[0] = d.x;
    n.b1[1] = d.y;
    n.b1[2] = d.z;
    n.update = __float_as_uint(d.w);
    return n;
}

// Box of child slot 0 (a0 / a1) or 1 (b0 / b1) of a binary internal node: the
// refit wrote the exact union of the child's boxes (or its triangle's box)
// there, so the collapse reads child boxes from the parent and loads a node
// only to expand it.
__device__ __forceinline__ Bx child_box(const BvhNode& nd, int side)
{
    Bx r;
    for (int k = 0; k < 3; ++k)
    {
        r.lo[k] = side ? nd.b0[k] : nd.a0[k];
        r.hi[k] = side ? nd.b1[k] : nd.a1[k];
    }
    return r;
}

// Exponent e (biased) of the smallest power of two s with ceil(ext / s) <= 255.
__device__ __forceinline__ int pick_exp(float lo, float hi)
{
    float    ext = __fsub_ru(hi, lo);
    float    s   = __fdiv_ru(ext, 255.f);
    uint32_t u   = __float_as_uint(s);
    int      ex  = (int)((u >> 23) & 0xffu);
    if (ex == 0) ex = 1;  // zero or subnormal extent: 2^-126
    else if (u & 0x7fffffu) ex += 1;
    while (ex < 253)
    {
        float inv = __uint_as_float((uint32_t)(254 - ex) << 23);  // 2^(127-ex)
        if (ceilf(__fmul_ru(ext, inv)) <= 255.f) break;
        ++ex;
    }
    return ex;
}

// The quantised 4-wide node of child boxes cb[0..nc-1] (slots nc..3 empty):
// the frame of their union, bounds rounded outward.  The collapse and the
// update's requantisation (k_refit_bvh4) both write nodes through it.
__device__ __forceinline__ void quantize4(Bvh4QNode& o, const Bx* cb, int nc)
{
    Bx u = cb[0];
#pragma unroll
    for (int k = 1; k < 4; ++k)
        if (k < nc)
            for (int a = 0; a < 3; ++a)
            {
                u.lo[a] = fminf(u.lo[a], cb[k].lo[a]);
                u.hi[a] = fmaxf(u.hi[a], cb[k].hi[a]);
            }
    float iv[3];
    for (int a = 0; a < 3; ++a)
    {
        o.p[a]  = u.lo[a];
        int e   = pick_exp(u.lo[a], u.hi[a]);
        o.e[a]  = (uint8_t)e;
        iv[a]   = __uint_as_float((uint32_t)(254 - e) << 23);
    }
    o.pad0 = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k)
    {
        const bool used = k < nc;
        for (int a = 0; a < 3; ++a)
        {
            const float ql = used ? floorf(__fmul_rd(__fsub_rd(cb[k].lo[a], o.p[a]), iv[a])) : 0.f;
            const float qh = used ? ceilf(__fmul_ru(__fsub_ru(cb[k].hi[a], o.p[a]), iv[a])) : 0.f;
            o.q[a][k]     = (uint8_t)fminf(fmaxf(ql, 0.f), 255.f);
            o.q[3 + a][k] = (uint8_t)fminf(fmaxf(qh, 0.f), 255.f);
        }
    }
}

// Per-geometry views of a fused build's collapse state.
__device__ __forceinline__ CollapseCtl* ctl_of(const BuildItem& it)
{
    return reinterpret_cast<CollapseCtl*>(it.scratch + it.s_queue);
}
__device__ __forceinline__ Item* queue_of(const BuildItem& it, int level)
{
    Item* q0 = reinterpret_cast<Item*>(it.scratch + it.s_queue + 2 * kAlign);
    return (level & 1) ? q0 + it.n : q0;
}

// Warp-aggregated atomicAdd where the lanes form runs of equal counters:
// `peers` is the lane's run (lanes with the same counter, contiguous), v its
// addend.  All 32 lanes must call it; a run with valid == false adds nothing.
__device__ __forceinline__ uint32_t run_add(uint32_t* ctr, uint32_t v, uint32_t peers, bool valid)
{
    const int lane = threadIdx.x & 31;
    uint32_t  x    = v;
    for (int o = 1; o < 32; o <<= 1)
    {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    const int      first  = __ffs(peers) - 1;
    const int      last   = 31 - __clz(peers);
    const uint32_t before = __shfl_sync(0xffffffffu, x - v, first);
    const uint32_t total  = __shfl_sync(0xffffffffu, x, last) - before;
    uint32_t       base   = 0;
    if (lane == last && valid && total) base = atomicAdd(ctr, total);
    base = __shfl_sync(0xffffffffu, base, last);
    return base + (x - v) - before;
}

__global__ void k_collapse_init(BatchArgs b)
{
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= b.count) return;
    const BuildItem& it = b.items[g];
    const uint32_t   n  = it.n;
    if (n == 0) return;
    const BvhNode* nodes = reinterpret_cast<const BvhNode*>(it.result);
    CollapseCtl*   ctl   = ctl_of(it);
    Item*          q0    = queue_of(it, 0);
    WideNode*      wn    = reinterpret_cast<WideNode*>(it.result + it.wide_off);
    WideTri*       wt    = reinterpret_cast<WideTri*>(it.result + it.tris_off);
    for (int i = 0; i < kMaxLevels + 2; ++i) ctl->level_count[i] = 0;
    if (n == 1 && b.format == RR_CUDA_NODE_FORMAT_BVH4Q8)
    {
        // A one-triangle mesh: one quantised 4-wide node whose only child is
        // the leaf (slot 0 spans the node's whole quantisation frame).
        const Bx  bx = node_union(nodes[0]);
        Bvh4QNode o{};
        for (int a = 0; a < 3; ++a)
        {
            o.p[a]         = bx.lo[a];
            const int   e  = pick_exp(bx.lo[a], bx.hi[a]);
            const float iv = __uint_as_float((uint32_t)(254 - e) << 23);
            o.e[a]         = (uint8_t)e;
            o.q[a][0]      = 0;
            o.q[3 + a][0]  = (uint8_t)fminf(255.f, ceilf(__fmul_ru(__fsub_ru(bx.hi[a], bx.lo[a]), iv)));
        }
        for (int k = 0; k < 4; ++k) o.child[k] = k == 0 ? kBvh4Leaf : kInvalid;
        reinterpret_cast<Bvh4QNode*>(it.result + it.wide_off)[0] = o;
        ctl->wide_count = 1;
        ctl->tri_count  = 0;
        return;
    }
    if (n == 1 && b.format == RR_CUDA_NODE_FORMAT_BVH4)
    {
        // A one-triangle mesh: one 4-wide node whose only child is the leaf.
        const Bx  bx = node_union(nodes[0]);
        Bvh4Node  o{};
        for (int k = 0; k < 4; ++k)
        {
            for (int a = 0; a < 3; ++a)
            {
                o.lo[a][k] = k == 0 ? bx.lo[a] : 0.f;
                o.hi[a][k] = k == 0 ? bx.hi[a] : 0.f;
            }
            o.child[k] = k == 0 ? kBvh4Leaf : kInvalid;
        }
        reinterpret_cast<Bvh4Node*>(it.result + it.wide_off)[0] = o;
        ctl->wide_count = 1;
        ctl->tri_count  = 0;
        return;
    }
    if (n == 1)
    {
        // A one-triangle mesh: one wide node with a single triangle slot.
        BvhNode  lf = nodes[0];
        WideNode w{};
        Bx       bx = node_union(lf);
        for (int k = 0; k < 3; ++k)
        {
            w.p[k] = bx.lo[k];
            int e  = pick_exp(bx.lo[k], bx.hi[k]);
            w.e[k] = (uint8_t)e;
            float inv = __uint_as_float((uint32_t)(254 - e) << 23);
            w.qlo[k][0] = 0;
            w.qhi[k][0] = (uint8_t)min(255.f, ceilf(__fmul_ru(__fsub_ru(bx.hi[k], bx.lo[k]), inv)));
        }
        w.imask      = 0;
        w.child_base = 0;
        w.tri_base   = 0;
        w.meta[0]    = (uint8_t)((1u << 5) | 0u);
        wn[0]        = w;
        WideTri t;
        t.v0[0] = lf.a0[0];
        t.v0[1] = lf.a0[1];
        t.v0[2] = lf.a0[2];
        t.prim  = lf.child1;
        t.v1[0] = lf.a1[0];
        t.v1[1] = lf.a1[1];
        t.v1[2] = lf.a1[2];
        t.pad1  = 0;
        t.v2[0] = lf.b0[0];
        t.v2[1] = lf.b0[1];
        t.v2[2] = lf.b0[2];
        t.pad2  = 0;
        wt[0]   = t;
        ctl->wide_count = 1;
        ctl->tri_count  = 1;
        return;
    }
    q0[0]              = Item{0u, 0u};
    ctl->level_count[0] = 1;
    ctl->wide_count    = 1;
    ctl->tri_count     = 0;
}

// Exclusive prefix over geometries of this level's work items, by one block
// of kScanBlock threads.  The counts are read from L2 (the drain below runs
// this after its own atomics in the same launch).
constexpr int kScanBlock = 1024;
__device__ __forceinline__ void level_scan_block(const BatchArgs& b, int level)
{
    __shared__ uint32_t warp_sum[kScanBlock / 32];
    const uint32_t per = (b.count + kScanBlock - 1) / kScanBlock;
    const uint32_t g0  = threadIdx.x * per;
    uint32_t       sum = 0;
    for (uint32_t g = g0; g < g0 + per && g < b.count; ++g)
        if (b.items[g].n > 0) sum += __ldcg(&ctl_of(b.items[g])->level_count[level]);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t  x    = sum;
    for (int o = 1; o < 32; o <<= 1)
    {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sum[w] = x;
    __syncthreads();
    uint32_t add = 0;
    for (int k = 0; k < w; ++k) add += warp_sum[k];
    uint32_t run = x - sum + add;
    for (uint32_t g = g0; g < g0 + per && g < b.count; ++g)
    {
        b.level_prefix[g] = run;
        if (b.items[g].n > 0) run += __ldcg(&ctl_of(b.items[g])->level_count[level]);
    }
    if (threadIdx.x == kScanBlock - 1) b.level_prefix[b.count] = x + add;
}
__global__ void __launch_bounds__(kScanBlock) k_level_scan(BatchArgs b, int level) { level_scan_block(b, level); }

// Work items of a level in the batch: its total (a batch of one reads its
// count directly).
__device__ __forceinline__ uint32_t level_total(const BatchArgs& b, int level)
{
    return b.count == 1 ? *((volatile uint32_t*)&ctl_of(b.items[0])->level_count[level])
                        : *((volatile uint32_t*)&b.level_prefix[b.count]);
}

// Geometry of work item t: the last prefix entry <= t, read from L2.
__device__ __forceinline__ uint32_t batch_find_cg(const uint32_t* prefix, uint32_t count, uint32_t t)
{
    uint32_t lo = 0, hi = count;
    while (hi - lo > 1)
    {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldcg(prefix + mid) <= t)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

// One level of the collapse for every geometry, items first, first + stride,
// ...: work item `it` of the level belongs to the geometry found in the
// level prefix.  Warps stay whole (the item range is rounded up to 32).
// kQ8 (W == 4): the 4-wide nodes store 8-bit conservative bounds (Bvh4QNode).
// kCoherent: the queue and the prefix were written earlier in the same
// launch (the drain), so they are read from L2, never through the
// read-only path.
template <int W, bool kQ8, bool kCoherent>
__device__ __forceinline__ void collapse_pass(const BatchArgs& b, int level, DeviceWords* words, uint32_t total,
                                              uint32_t first, uint32_t stride)
{
    for (uint32_t it = first; it < ((total + 31u) & ~31u); it += stride)
    {
        const bool     active = it < total;
        const uint32_t g      = !active ? 0xffffffffu
                                        : (b.count == 1 ? 0u
                                           : kCoherent ? batch_find_cg(b.level_prefix, b.count, it)
                                                       : batch_find(b.level_prefix, b.count, it));
        const uint32_t peers  = __match_any_sync(0xffffffffu, g);
        const BuildItem* bi   = active ? b.items + g : b.items;
        const uint32_t local  = active ? it - (b.count == 1 ? 0u
                                                : kCoherent ? __ldcg(b.level_prefix + g)
                                                            : __ldg(b.level_prefix + g))
                                       : 0u;
        const BvhNode* __restrict__ nodes = reinterpret_cast<const BvhNode*>(bi->result);
        CollapseCtl*   ctl           = ctl_of(*bi);
        const Item* __restrict__ qin = queue_of(*bi, level);
        Item* __restrict__ qout      = queue_of(*bi, level + 1);
        WideNode*      wn            = reinterpret_cast<WideNode*>(bi->result + bi->wide_off);
        WideTri*       wt            = reinterpret_cast<WideTri*>(bi->result + bi->tris_off);
        const uint32_t wide_capacity = bi->wide_capacity, tri_capacity = bi->tri_capacity;
        // The children.  For W == 4 every loop over them is unrolled, so
        // each index is a compile-time constant and the arrays stay in
        // registers (a variable index would put them in local memory).  The
        // 8-wide node's slot assignment indexes them by variable anyway, so
        // W == 8 keeps the short loops to nc and the indexed updates.
        uint32_t ch[W];
        Bx       cb[W];
        bool     cint[W];
#pragma unroll
        for (int k = 0; k < W; ++k)
        {
            ch[k]   = 0;
            cint[k] = false;
            cb[k]   = Bx{{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
        }
        int  nc = 0;
        Item item{0, 0};
        if (active)
        {
            // Binary layout: internal nodes [0, n-2], leaves [n-1, 2n-2], so
            // a child's kind follows from its index; each expansion of the
            // largest internal child is one node load.
            const uint32_t first_leaf = bi->n - 1;
            if (kCoherent)
            {
                const uint2 q = __ldcg(reinterpret_cast<const uint2*>(qin) + local);
                item          = Item{q.x, q.y};
            }
            else
                item = qin[local];
            BvhNode root  = load_node(nodes, item.b);
            ch[0]         = root.child0;
            ch[1]         = root.child1;
            cb[0]         = child_box(root, 0);
            cb[1]         = child_box(root, 1);
            cint[0]       = ch[0] < first_leaf;
            cint[1]       = ch[1] < first_leaf;
            nc            = 2;
            while (nc < W)
            {
                int      best  = -1;
                float    ba    = -1.f;
                uint32_t cbest = 0;
                if constexpr (W == 4)
                {
#pragma unroll
                    for (int k = 0; k < W; ++k)
                        if (k < nc && cint[k])
                        {
                            const float a = half_area(cb[k]);
                            if (a > ba)
                            {
                                ba    = a;
                                best  = k;
                                cbest = ch[k];
                            }
                        }
                }
                else
                {
                    for (int k = 0; k < nc; ++k)
                        if (cint[k])
                        {
                            const float a = half_area(cb[k]);
                            if (a > ba)
                            {
                                ba   = a;
                                best = k;
                            }
                        }
                    if (best >= 0) cbest = ch[best];
                }
                if (best < 0) break;
                const BvhNode nd = load_node(nodes, cbest);
                if constexpr (W == 4)
                {
                    const Bx   b0 = child_box(nd, 0), b1 = child_box(nd, 1);
                    const bool i0 = nd.child0 < first_leaf, i1 = nd.child1 < first_leaf;
#pragma unroll
                    for (int k = 0; k < W; ++k)
                    {
                        if (k == best)
                        {
                            ch[k]   = nd.child0;
                            cb[k]   = b0;
                            cint[k] = i0;
                        }
                        if (k == nc)
                        {
                            ch[k]   = nd.child1;
                            cb[k]   = b1;
                            cint[k] = i1;
                        }
                    }
                }
                else
                {
                    ch[best]   = nd.child0;
                    cb[best]   = child_box(nd, 0);
                    cint[best] = nd.child0 < first_leaf;
                    ch[nc]     = nd.child1;
                    cb[nc]     = child_box(nd, 1);
                    cint[nc]   = nd.child1 < first_leaf;
                }
                ++nc;
            }
        }
        // Leaf slots hold one triangle each (the meta byte's count field
        // allows up to 3; one measured fastest); the 4-wide nodes have no
        // triangle array.
        uint32_t ccnt[W];
        uint32_t n_int = 0, n_leaf = 0;
#pragma unroll
        for (int k = 0; k < W; ++k)
        {
            ccnt[k] = (k < nc && !cint[k] && W == 8) ? 1u : 0u;
            if (k < nc && cint[k])
                ++n_int;
            else
                n_leaf += ccnt[k];
        }
        // Allocate (warp-aggregated over the full warp; inactive lanes add 0).
        __syncwarp();
        const uint32_t child_base = run_add(&ctl->wide_count, n_int, peers, active);
        const uint32_t tri_base   = run_add(&ctl->tri_count, n_leaf, peers, active);
        const uint32_t qpos       = run_add(&ctl->level_count[level + 1], n_int, peers, active);
        if (!active) continue;
        if (child_base + n_int > wide_capacity || tri_base + n_leaf > tri_capacity)
        {
            atomicOr(&words->error_bits, (uint32_t)RR_CUDA_DEVICE_ERROR_NODE_RANGE);
            continue;
        }
        if constexpr (W == 4 && kQ8)
        {
            // Quantised 4-wide node: the frame of the union of the child
            // boxes, bounds rounded outward as for the 8-wide node (below),
            // children numbered as in the fp32 4-wide node.  pad1[0] keeps
            // the node's binary node, for the update's requantisation.
            Bvh4QNode o;
            quantize4(o, cb, nc);
            o.pad1[0] = item.b;
            o.pad1[1] = 0;
            uint32_t ri = 0;
            for (int k = 0; k < 4; ++k)
            {
                if (k >= nc)
                    o.child[k] = kInvalid;
                else if (cint[k])
                {
                    o.child[k]      = child_base + ri;
                    qout[qpos + ri] = Item{ch[k], child_base + ri};
                    ++ri;
                }
                else
                    o.child[k] = kBvh4Leaf | ch[k];
            }
            reinterpret_cast<Bvh4QNode*>(bi->result + bi->wide_off)[item.w] = o;
            continue;
        }
        if constexpr (W == 4)
        {
            // 4-wide node: exact child boxes (read from the parents), internal
            // children numbered in slot order, leaf children by their binary
            // leaf node.
            Bvh4Node o;
            uint32_t ri = 0;
            for (int k = 0; k < 4; ++k)
            {
                const bool used = k < nc;
                for (int a = 0; a < 3; ++a)
                {
                    o.lo[a][k] = used ? cb[k].lo[a] : 0.f;
                    o.hi[a][k] = used ? cb[k].hi[a] : 0.f;
                }
                if (!used)
                    o.child[k] = kInvalid;
                else if (cint[k])
                {
                    o.child[k]      = child_base + ri;
                    qout[qpos + ri] = Item{ch[k], child_base + ri};
                    ++ri;
                }
                else
                    o.child[k] = kBvh4Leaf | ch[k];
                o.pad[k] = k == 0 ? item.b : 0u;  // pad[0]: the node's binary node (the update reads it)
            }
            reinterpret_cast<Bvh4Node*>(bi->result + bi->wide_off)[item.w] = o;
            continue;
        }
        if constexpr (W == 8)
        {
            // Quantisation frame.
            WideNode w;
            Bx       u = cb[0];
            for (int k = 1; k < nc; ++k)
                for (int a = 0; a < 3; ++a)
                {
                    u.lo[a] = fminf(u.lo[a], cb[k].lo[a]);
                    u.hi[a] = fmaxf(u.hi[a], cb[k].hi[a]);
                }
            float inv[3];
            for (int a = 0; a < 3; ++a)
            {
                w.p[a] = u.lo[a];
                int e  = pick_exp(u.lo[a], u.hi[a]);
                w.e[a] = (uint8_t)e;
                inv[a] = __uint_as_float((uint32_t)(254 - e) << 23);
            }
            w.child_base = child_base;
            w.tri_base   = tri_base;
            // Octant slot order: slot s holds a child on the + side of the node
            // centre along x if s & 4, y if s & 2, z if s & 1 (greedy assignment,
            // smallest cost first).  A ray with direction octant o visits slots
            // i ^ o for i = 0..7, which is then roughly front to back.
            int slot_child[8];
            {
                float dc[8][3];
                for (int k = 0; k < nc; ++k)
                    for (int a = 0; a < 3; ++a)
                        dc[k][a] = 0.5f * (cb[k].lo[a] + cb[k].hi[a]) - 0.5f * (u.lo[a] + u.hi[a]);
                for (int s2 = 0; s2 < 8; ++s2) slot_child[s2] = -1;
                uint32_t used = 0;
                for (int round = 0; round < nc; ++round)
                {
                    float bc = INFINITY;
                    int   bk = -1, bs = -1;
                    for (int k = 0; k < nc; ++k)
                    {
                        if (used >> k & 1u) continue;
                        for (int s2 = 0; s2 < 8; ++s2)
                        {
                            if (slot_child[s2] >= 0) continue;
                            const float cost = ((s2 & 4) ? -dc[k][0] : dc[k][0]) + ((s2 & 2) ? -dc[k][1] : dc[k][1]) +
                                               ((s2 & 1) ? -dc[k][2] : dc[k][2]);
                            if (cost < bc || bk < 0)
                            {
                                bc = cost;
                                bk = k;
                                bs = s2;
                            }
                        }
                    }
                    slot_child[bs] = bk;
                    used |= 1u << bk;
                }
            }
            uint8_t  imask = 0;
            uint32_t ri = 0, rl = 0;
            for (int slot = 0; slot < 8; ++slot)
            {
                const int k = slot_child[slot];
                if (k >= 0)
                {
                    for (int a = 0; a < 3; ++a)
                    {
                        float ql = floorf(__fmul_rd(__fsub_rd(cb[k].lo[a], w.p[a]), inv[a]));
                        float qh = ceilf(__fmul_ru(__fsub_ru(cb[k].hi[a], w.p[a]), inv[a]));
                        w.qlo[a][slot] = (uint8_t)fminf(fmaxf(ql, 0.f), 255.f);
                        w.qhi[a][slot] = (uint8_t)fminf(fmaxf(qh, 0.f), 255.f);
                    }
                    if (cint[k])
                    {
                        imask |= (uint8_t)(1u << slot);
                        w.meta[slot] = (uint8_t)(0x80u | ri);
                        qout[qpos + ri] = Item{ch[k], child_base + ri};
                        ++ri;
                    }
                    else
                    {
                        w.meta[slot] = (uint8_t)((ccnt[k] << 5) | rl);
                        for (uint32_t j = 0; j < ccnt[k]; ++j)
                        {
                            BvhNode lf = load_node(nodes, ch[k]);
                            WideTri t;
                            t.v0[0] = lf.a0[0];
                            t.v0[1] = lf.a0[1];
                            t.v0[2] = lf.a0[2];
                            t.prim  = lf.child1;
                            t.v1[0] = lf.a1[0];
                            t.v1[1] = lf.a1[1];
                            t.v1[2] = lf.a1[2];
                            t.pad1  = 0;
                            t.v2[0] = lf.b0[0];
                            t.v2[1] = lf.b0[1];
                            t.v2[2] = lf.b0[2];
                            t.pad2  = 0;
                            wt[tri_base + rl] = t;
                            ++rl;
                        }
                    }
                }
                else
                {
                    w.meta[slot] = 0;
                    for (int a = 0; a < 3; ++a)
                    {
                        w.qlo[a][slot] = 0;
                        w.qhi[a][slot] = 0;
                    }
                }
            }
            w.imask       = imask;
            wn[item.w]    = w;
        }
    }
}

template <int W, bool kQ8 = false>
__global__ void __launch_bounds__(128) k_collapse_level(BatchArgs b, int level, DeviceWords* words)
{
    collapse_pass<W, kQ8, false>(b, level, words, level_total(b, level), blockIdx.x * blockDim.x + threadIdx.x,
                                 gridDim.x * blockDim.x);
}

// The levels from `first_level` on, by one block, level after level (a
// barrier between them), until a level has no work items.  The host
// launches one k_collapse_level per level for as many levels as a tree of
// the batch's largest size normally has; a deeper tree (many equal Morton
// codes, for instance) ends here, correctly if slowly, instead of the host
// launching the maximum number of levels, most of them empty.
template <int W, bool kQ8 = false>
__global__ void __launch_bounds__(kScanBlock) k_collapse_drain(BatchArgs b, int first_level, DeviceWords* words)
{
    for (int level = first_level; level < kMaxLevels; ++level)
    {
        if (b.count > 1) level_scan_block(b, level);
        __syncthreads();
        const uint32_t total = level_total(b, level);  // the same for every thread: written before the barrier
        if (total == 0) break;
        collapse_pass<W, kQ8, true>(b, level, words, total, threadIdx.x, blockDim.x);
        __syncthreads();
    }
}

__global__ void k_collapse_finish(BatchArgs b, DeviceWords* words)
{
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= b.count) return;
    const BuildItem& it = b.items[g];
    if (it.n == 0) return;
    const CollapseCtl* ctl = ctl_of(it);
    Trailer*           tr  = reinterpret_cast<Trailer*>(it.result + it.trailer_off);
    if (ctl->level_count[kMaxLevels] != 0) atomicOr(&words->error_bits, (uint32_t)RR_CUDA_DEVICE_ERROR_COLLAPSE_DEPTH);
    tr->wide_count     = ctl->wide_count;
    tr->wide_tri_count = ctl->tri_count;
}

// The update of a buffer with 4-wide nodes (RR_BUILD_OPERATION_UPDATE, after
// the binary refit): the 4-wide topology stays, and every node takes its
// children's new boxes.  One thread per 4-wide node: a leaf child's box is its
// binary leaf's, an internal child's that of the binary node the child stands
// for (recorded in the child's pad word by the collapse).  Written like the
// collapse writes them (quantize4 for 8-bit bounds).  Indices out of range
// raise NODE_RANGE and leave the node as it was.
template <bool kQ8>
__global__ void __launch_bounds__(256) k_refit_bvh4(uint8_t* wide, const BvhNode* nodes, uint32_t n,
                                                     const Trailer* tr, uint32_t capacity, DeviceWords* words)
{
    const uint32_t count = min(tr->wide_count, capacity);
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < count; x += gridDim.x * blockDim.x)
    {
        uint32_t child[4];
        uint4    refs, pads;  // the node's reference and pad words, written back as they are
        if (kQ8)
        {
            const uint4* w = reinterpret_cast<const uint4*>(wide + (size_t)x * sizeof(Bvh4QNode));
            refs           = __ldcg(w + 1);
            pads           = __ldcg(w + 3);
        }
        else
        {
            const uint4* w = reinterpret_cast<const uint4*>(wide + (size_t)x * sizeof(Bvh4Node));
            refs           = __ldcg(w + 6);
            pads           = __ldcg(w + 7);
        }
        child[0] = refs.x, child[1] = refs.y, child[2] = refs.z, child[3] = refs.w;
        Bx   cb[4];
        int  nc = 0;
        bool ok = true;
#pragma unroll
        for (int k = 0; k < 4; ++k)
        {
            const uint32_t r = child[k];
            if (r == kInvalid) break;  // the collapse packs the children into the first slots
            uint32_t b;
            if (r & kBvh4Leaf)
                b = r & ~kBvh4Leaf;
            else if (r < count)
                b = kQ8 ? __ldcg(reinterpret_cast<const uint32_t*>(wide + (size_t)r * sizeof(Bvh4QNode) + 56))
                        : __ldcg(reinterpret_cast<const uint32_t*>(wide + (size_t)r * sizeof(Bvh4Node) + 112));
            else
                b = kInvalid;
            if (b >= 2 * n - 1)
            {
                ok = false;
                continue;
            }
            cb[nc++] = node_union(load_node(nodes, b));
        }
        if (!ok || nc == 0)
        {
            atomicOr(&words->error_bits, (uint32_t)RR_CUDA_DEVICE_ERROR_NODE_RANGE);
            continue;
        }
        if (kQ8)
        {
            // The whole node in four 16-byte stores (no partly written
            // sector): frame and planes new, references and pads as read.
            Bvh4QNode q;
            quantize4(q, cb, nc);
            const uint4* qs = reinterpret_cast<const uint4*>(&q);
            uint4*       w  = reinterpret_cast<uint4*>(wide + (size_t)x * sizeof(Bvh4QNode));
            uint4        w3 = qs[3];
            w3.z            = pads.z;
            w3.w            = pads.w;
            w[0]            = qs[0];
            w[1]            = refs;
            w[2]            = qs[2];
            w[3]            = w3;
        }
        else
        {
            Bvh4Node o;
#pragma unroll
            for (int k = 0; k < 4; ++k)
                for (int a = 0; a < 3; ++a)
                {
                    o.lo[a][k] = k < nc ? cb[k].lo[a] : 0.f;
                    o.hi[a][k] = k < nc ? cb[k].hi[a] : 0.f;
                }
            const uint4* os = reinterpret_cast<const uint4*>(&o);
            uint4*       w  = reinterpret_cast<uint4*>(wide + (size_t)x * sizeof(Bvh4Node));
#pragma unroll
            for (int j = 0; j < 6; ++j) w[j] = os[j];
            w[6] = refs;
            w[7] = pads;
        }
    }
}
}  // namespace

cudaError_t launch_collapse_batch(const BatchArgs& b, DeviceWords* words, int sm_count, cudaStream_t s)
{
    if (b.count == 0 || b.total_prims == 0) return cudaSuccess;
    static_assert(sizeof(CollapseCtl) <= 2 * kAlign, "collapse control block");
    const int per_geom = (int)((b.count + 127) / 128);
    k_collapse_init<<<per_geom, 128, 0, s>>>(b);
    if (b.max_n > 1)
    {
        // Work items of a level are bounded by count * 8^level and by the
        // number of triangles (every item is a distinct internal subtree).
        // Launched levels: ceil(log_W(largest n)) + 8 (a collapsed LBVH of n
        // triangles measured 4 to 16 levels deep for n up to 4.2 M: soups
        // and heightfields, fast and restructured); the drain takes any
        // deeper level.
        const uint32_t fan    = is_bvh4_format(b.format) ? 4u : 8u;
        int            levels = 8;
        for (uint64_t c = 1; c < b.max_n; c *= fan) ++levels;
        levels         = std::min(levels, kMaxLevels);
        // RR_CUDA_COLLAPSE_LEVELS=k (1 .. the count above) launches only k
        // level kernels and leaves the rest to the drain, so that tests run
        // the drain on ordinary trees.
        if (const char* e = std::getenv("RR_CUDA_COLLAPSE_LEVELS"))
        {
            const int k = std::atoi(e);
            if (k >= 1 && k < levels) levels = k;
        }
        uint64_t bound = b.count;
        for (int level = 0; level < levels; ++level)
        {
            if (b.count > 1) k_level_scan<<<1, kScanBlock, 0, s>>>(b, level);
            const uint64_t cap    = std::min<uint64_t>(bound, b.total_prims);
            const int      blocks = (int)std::max<uint64_t>(
                1, std::min<uint64_t>((cap + 127) / 128, (uint64_t)sm_count * 16));
            if (b.format == RR_CUDA_NODE_FORMAT_BVH4)
                k_collapse_level<4><<<blocks, 128, 0, s>>>(b, level, words);
            else if (b.format == RR_CUDA_NODE_FORMAT_BVH4Q8)
                k_collapse_level<4, true><<<blocks, 128, 0, s>>>(b, level, words);
            else
                k_collapse_level<8><<<blocks, 128, 0, s>>>(b, level, words);
            bound = std::min<uint64_t>(bound * fan, b.total_prims);
        }
        if (levels < kMaxLevels)
        {
            if (b.format == RR_CUDA_NODE_FORMAT_BVH4)
                k_collapse_drain<4><<<1, kScanBlock, 0, s>>>(b, levels, words);
            else if (b.format == RR_CUDA_NODE_FORMAT_BVH4Q8)
                k_collapse_drain<4, true><<<1, kScanBlock, 0, s>>>(b, levels, words);
            else
                k_collapse_drain<8><<<1, kScanBlock, 0, s>>>(b, levels, words);
        }
    }
    k_collapse_finish<<<per_geom, 128, 0, s>>>(b, words);
    return cudaGetLastError();
}

cudaError_t launch_refit_bvh4(uint8_t* result, const GeomLayout& L, DeviceWords* words, int sm_count, cudaStream_t s)
{
    if (L.n == 0 || !is_bvh4_format(L.format)) return cudaSuccess;
    const BvhNode* nodes = reinterpret_cast<const BvhNode*>(result);
    const Trailer* tr    = reinterpret_cast<const Trailer*>(result + L.trailer_off);
    const uint32_t cap   = (uint32_t)L.wide_capacity;
    const uint32_t grid  = (uint32_t)std::min<size_t>(((size_t)cap + 255) / 256, (size_t)sm_count * 16);
    if (L.format == RR_CUDA_NODE_FORMAT_BVH4Q8)
        k_refit_bvh4<true><<<grid, 256, 0, s>>>(result + L.wide_off, nodes, L.n, tr, cap, words);
    else
        k_refit_bvh4<false><<<grid, 256, 0, s>>>(result + L.wide_off, nodes, L.n, tr, cap, words);
    return cudaGetLastError();
}

}  // namespace rr

