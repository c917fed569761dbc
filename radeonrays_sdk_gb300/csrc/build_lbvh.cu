// build_lbvh.cu -- LBVH build of triangle meshes on sm_103a, one mesh or many
// meshes fused into one set of launches.
//
// Pipeline (reference: vlk/hlbvh_builder.cpp:159-351):
//   k_batch_init    trailers, bounds and histogram words of every geometry
//   k_batch_bounds  lbvh_calc_mesh_aabb.comp:121-179  exact min/max of all
//                   referenced vertices, order-preserving uint atomics
//   k_batch_morton  lbvh_calc_morton_codes_mesh.comp:78-130, plus the digit
//                   histograms of the sort (one read of the keys fewer)
//   radix sort      vlk/radix_sort.cpp (sort.cu, onesweep, per geometry)
//   k_batch_emit    lbvh_emit_hierarchy_mesh.comp:78-217 (Karras 2012)
//   k_batch_refit   lbvh_fit_aabb_mesh.comp:94-205 (atomic bottom-up climb)
//   wide collapse   (wide.cu) when the WIDE8 node format is requested
//
// Fused builds.  Every geometry keeps its own scratch and result buffer (the
// sizes rrGetGeometryBuildMemoryRequirements gives for it alone) and is
// described by a BuildItem in device memory.  The element range of every
// geometry is cut into sort tiles (radix_sort_tile_keys keys); a block of a
// tile-mapped kernel finds its geometry by a binary search over the tiles'
// exclusive prefix, so one launch covers all geometries however uneven they
// are, and a single mesh is the batch of one.  Results are those of separate
// builds: no value crosses from one geometry to another.
//
// Arithmetic follows the oracle's rules (IEEE fp32, no contraction: the file
// is compiled with --fmad=false), so codes, permutation, topology and boxes
// are bit-identical to the CPU restatement.
#include <algorithm>

#include "rr_internal.h"

namespace rr
{
cudaError_t launch_collapse_batch(const BatchArgs& b, DeviceWords* words, int sm_count, cudaStream_t s);

namespace
{
constexpr int kBlk   = 256;  // threads of the tile-mapped kernels
constexpr int kChunk = 256;  // elements per block of the emit / refit kernels
// Threads per block of the restructure climb: few climbs run long, and a
// block stays resident until its last warp ends, so small blocks leave room
// for more (64: 9.1 ms for the quality build of 4.2 M triangles, 256: 9.9).
constexpr int kRsBlk = 64;
// Threads per block of the refit climbs (build and update), for the same
// reason: 1.30 -> 1.24 ms for the fast build of 4.2 M triangles.
constexpr int kFitBlk = 64;

struct F3
{
    float x, y, z;
};
__device__ __forceinline__ F3 f3(float x, float y, float z) { return F3{x, y, z}; }
__device__ __forceinline__ F3 vmin(F3 a, F3 b) { return f3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }
__device__ __forceinline__ F3 vmax(F3 a, F3 b) { return f3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }

__device__ __forceinline__ uint32_t f2ord(float f)
{
    uint32_t u = __float_as_uint(f);
    return u ^ ((1u + ~(u >> 31)) | 0x80000000u);
}
__device__ __forceinline__ float ord2f(uint32_t u)
{
    u ^= (((u >> 31) - 1u) | 0x80000000u);
    return __uint_as_float(u);
}

__device__ __forceinline__ uint32_t tri_index(const BuildItem& m, uint64_t k)
{
    return m.index16 ? (uint32_t)__ldg((const uint16_t*)m.indices + k) : __ldg((const uint32_t*)m.indices + k);
}
__device__ __forceinline__ F3 vtx(const BuildItem& m, uint32_t i)
{
    const float* p = m.vertices + (uint64_t)i * m.stride_floats;
    return f3(__ldg(p), __ldg(p + 1), __ldg(p + 2));
}
// The three leaf vertices of primitive t: a triangle's vertices, or for an
// AABB list the box (min, max, max) read from its (min.xyzw, max.xyzw) pair.
__device__ __forceinline__ void tri_verts(const BuildItem& m, uint32_t t, F3& a, F3& b, F3& c)
{
    if (m.prim_kind == kPrimAabbs)
    {
        const float* p = m.vertices + (uint64_t)t * m.stride_floats;
        a              = f3(__ldg(p), __ldg(p + 1), __ldg(p + 2));
        b              = f3(__ldg(p + 4), __ldg(p + 5), __ldg(p + 6));
        c              = b;
        return;
    }
    uint32_t i0 = tri_index(m, 3ull * t), i1 = tri_index(m, 3ull * t + 1), i2 = tri_index(m, 3ull * t + 2);
    a = vtx(m, i0);
    b = vtx(m, i1);
    c = vtx(m, i2);
}

// The climb's arrival flag: exchange with acquire-release semantics at gpu
// scope.  The release half publishes this thread's stores below the node
// (its child's boxes) before the flag; the acquire half, for the second
// arriver, makes the partner's stores visible to the loads that follow.
// One ordered atomic replaces a fence on either side of a relaxed exchange.
__device__ __forceinline__ uint32_t climb_exch(uint32_t* flag)
{
    uint32_t old;
    asm volatile("atom.acq_rel.gpu.global.exch.b32 %0, [%1], %2;" : "=r"(old) : "l"(flag), "r"(1u) : "memory");
    return old;
}

__device__ __forceinline__ uint32_t expand_bits(uint32_t r)
{
    r = (r * 0x00010001u) & 0xFF0000FFu;
    r = (r * 0x00000101u) & 0x0F00F00Fu;
    r = (r * 0x00000011u) & 0xC30C30C3u;
    r = (r * 0x00000005u) & 0x49249249u;
    return r;
}
__device__ __forceinline__ uint64_t expand_bits21(uint64_t v)
{
    v &= 0x1fffffull;
    v = (v | (v << 32)) & 0x1f00000000ffffull;
    v = (v | (v << 16)) & 0x1f0000ff0000ffull;
    v = (v | (v << 8)) & 0x100f00f00f00f00full;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}
__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }

// clz as the reference shader defines it (32 - findMSB(v), findMSB(0) = -1).
__device__ __forceinline__ int clz_p1(uint32_t v) { return __clz(v) + 1; }
__device__ __forceinline__ int clz64_p1(uint64_t v) { return __clzll(v) + 1; }

template <int kBits>
struct Delta
{
    const void* codes;
    int64_t     n;
    __device__ __forceinline__ int operator()(int64_t i1, int64_t i2) const
    {
        int64_t l = min(i1, i2), r = max(i1, i2);
        if (l < 0 || r >= n) return 0;
        if (kBits == 63)
        {
            uint64_t a = __ldg((const unsigned long long*)codes + l), b = __ldg((const unsigned long long*)codes + r);
            return a != b ? clz64_p1(a ^ b) : 64 + clz_p1((uint32_t)(l ^ r));
        }
        uint32_t a = __ldg((const uint32_t*)codes + l), b = __ldg((const uint32_t*)codes + r);
        return a != b ? clz_p1(a ^ b) : 32 + clz_p1((uint32_t)(l ^ r));
    }
};

// Internal node i (< n - 1) of a Karras tree over n sorted codes.
template <int kBits>
__device__ __forceinline__ void emit_node(const void* __restrict__ codes, uint32_t n, uint32_t i, BvhNode* nodes)
{
    Delta<kBits> delta{codes, (int64_t)n};
    const int64_t ii = i;
    // FindSpan
    const int     dd   = delta(ii, ii + 1) - delta(ii, ii - 1);
    const int64_t d    = dd > 0 ? 1 : (dd < 0 ? -1 : 0);
    const int     dmin = delta(ii, ii - d);
    int64_t       lmax = 2;
    while (delta(ii, ii + lmax * d) > dmin) lmax *= 2;
    int64_t l = 0, t = lmax;
    do
    {
        t /= 2;
        if (delta(ii, ii + (l + t) * d) > dmin) l += t;
    } while (t > 1);
    const int64_t e    = ii + l * d;
    const int64_t lo_e = ii < e ? ii : e, hi_e = ii < e ? e : ii;
    const int64_t sx   = lo_e > 0 ? lo_e : 0;
    const int64_t sy   = hi_e < (int64_t)n - 1 ? hi_e : (int64_t)n - 1;
    // FindSplit
    int64_t   left = sx, right = sy;
    const int nid  = delta(left, right);
    do
    {
        int64_t ns = (right + left) / 2;
        if (delta(left, ns) > nid)
            left = ns;
        else
            right = ns;
    } while (right > left + 1);
    const int64_t  s  = left;
    const uint32_t al = (s == sx) ? (uint32_t)(n - 1 + s) : (uint32_t)s;
    const uint32_t ar = (s + 1 == sy) ? (uint32_t)(n - 1 + s + 1) : (uint32_t)(s + 1);
    nodes[i].child0   = al;
    nodes[i].child1   = ar;
    nodes[i].update   = 0;
    nodes[al].parent  = i;
    nodes[ar].parent  = i;
    if (i == 0) nodes[0].parent = kInvalid;
}

// Compact topology of a geometry build, in its scratch: the emit writes it
// and the refit reads it, then writes every node whole.  Children as one
// 8-byte word per internal node, parents as one 4-byte word per node, and the
// climb flags.  The emit's words are thus dense stores into arrays of 4 and
// 8-byte words instead of scattered 4-byte stores into 64-byte nodes (each
// of which made L2 fetch the node's sector before merging the word).
struct Topo
{
    uint2*    child;   // n - 1
    uint32_t* parent;  // 2n - 1
    uint32_t* flag;    // n - 1
};
__host__ __device__ __forceinline__ size_t topo_align(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }
__host__ __device__ __forceinline__ size_t topo_bytes(uint32_t n)
{
    if (n < 2) return 0;
    return topo_align(8ull * (n - 1)) + topo_align(4ull * (2ull * n - 1)) + topo_align(4ull * (n - 1));
}
__device__ __forceinline__ Topo topo_of(const BuildItem& it)
{
    uint8_t* base = it.scratch + it.s_topo;
    Topo     t;
    t.child  = reinterpret_cast<uint2*>(base);
    t.parent = reinterpret_cast<uint32_t*>(base + topo_align(8ull * (it.n - 1)));
    t.flag   = t.parent + topo_align(4ull * (2ull * it.n - 1)) / 4;
    return t;
}

// emit_node into the compact topology (flag cleared for the refit's climb).
template <int kBits>
__device__ __forceinline__ void emit_node_topo(const void* __restrict__ codes, uint32_t n, uint32_t i, const Topo& t)
{
    Delta<kBits> delta{codes, (int64_t)n};
    const int64_t ii = i;
    const int     dd   = delta(ii, ii + 1) - delta(ii, ii - 1);
    const int64_t d    = dd > 0 ? 1 : (dd < 0 ? -1 : 0);
    const int     dmin = delta(ii, ii - d);
    int64_t       lmax = 2;
    while (delta(ii, ii + lmax * d) > dmin) lmax *= 2;
    int64_t l = 0, tt = lmax;
    do
    {
        tt /= 2;
        if (delta(ii, ii + (l + tt) * d) > dmin) l += tt;
    } while (tt > 1);
    const int64_t e    = ii + l * d;
    const int64_t lo_e = ii < e ? ii : e, hi_e = ii < e ? e : ii;
    const int64_t sx   = lo_e > 0 ? lo_e : 0;
    const int64_t sy   = hi_e < (int64_t)n - 1 ? hi_e : (int64_t)n - 1;
    int64_t       left = sx, right = sy;
    const int     nid  = delta(left, right);
    do
    {
        int64_t ns = (right + left) / 2;
        if (delta(left, ns) > nid)
            left = ns;
        else
            right = ns;
    } while (right > left + 1);
    const int64_t  s  = left;
    const uint32_t al = (s == sx) ? (uint32_t)(n - 1 + s) : (uint32_t)s;
    const uint32_t ar = (s + 1 == sy) ? (uint32_t)(n - 1 + s + 1) : (uint32_t)(s + 1);
    t.child[i]   = make_uint2(al, ar);
    t.flag[i]    = 0;
    t.parent[al] = i;
    t.parent[ar] = i;
    if (i == 0) t.parent[0] = kInvalid;
}

// One sorted array (the instance tree of a scene build).
template <int kBits>
__global__ void __launch_bounds__(256) k_emit(const void* __restrict__ codes, uint32_t n, BvhNode* nodes)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i + 1 >= n) return;
    emit_node<kBits>(codes, n, i, nodes);
}


// Box of a child node as the fit shader computes it (lbvh_fit_aabb_mesh.comp:94-118).
// Loads are 16-byte L2-coherent vector loads (the node is four float4).
__device__ __forceinline__ void child_box(const BvhNode* nodes, uint32_t c, F3& lo, F3& hi)
{
    const float4* p4 = reinterpret_cast<const float4*>(nodes + c);
    const float4  w0 = __ldcg(p4), w1 = __ldcg(p4 + 1), w2 = __ldcg(p4 + 2);
    const F3      a = f3(w0.x, w0.y, w0.z), b = f3(w1.x, w1.y, w1.z), p = f3(w2.x, w2.y, w2.z);
    if (__float_as_uint(w0.w) != kInvalid)
    {
        const float4 w3 = __ldcg(p4 + 3);
        const F3     q  = f3(w3.x, w3.y, w3.z);
        lo              = vmin(a, p);
        hi              = vmax(b, q);
    }
    else
    {
        lo = vmin(vmin(a, b), p);
        hi = vmax(vmax(a, b), p);
    }
}

// Writes the two child boxes of internal node x as four 16-byte stores; the
// child, parent and climb-flag words are rewritten with the values given.
__device__ __forceinline__ void store_boxes4(BvhNode* nodes, uint32_t x, F3 lo0, F3 hi0, F3 lo1, F3 hi1, uint32_t c0,
                                             uint32_t c1, uint32_t parent, uint32_t flag)
{
    float4* o = reinterpret_cast<float4*>(nodes + x);
    __stcg(o + 0, make_float4(lo0.x, lo0.y, lo0.z, __uint_as_float(c0)));
    __stcg(o + 1, make_float4(hi0.x, hi0.y, hi0.z, __uint_as_float(c1)));
    __stcg(o + 2, make_float4(lo1.x, lo1.y, lo1.z, __uint_as_float(parent)));
    __stcg(o + 3, make_float4(hi1.x, hi1.y, hi1.z, __uint_as_float(flag)));
}

template <int kBits>
struct KeyCfg
{
    static constexpr uint32_t kTile   = kBits == 63 ? 2048u : 4096u;  // == radix_sort_tile_keys(kBits)
    static constexpr uint32_t kPasses = kBits == 63 ? 8u : 4u;
    static constexpr uint32_t kChunks = kTile / kChunk;              // emit / refit blocks per tile
};

__device__ __forceinline__ uint32_t* sort_words(const BuildItem& it)
{
    return reinterpret_cast<uint32_t*>(it.scratch + it.s_sort);
}

// Per geometry: trailer, bounds identities, digit histograms and run counters.
__global__ void __launch_bounds__(kBlk) k_batch_init(BatchArgs b)
{
    const uint32_t   g  = blockIdx.x;
    const BuildItem& it = b.items[g];
    if (g == 0)
        for (int k = threadIdx.x; k < kBatchCounters; k += blockDim.x) (&b.ctl->sort_tile[0])[k] = 0;
    if (threadIdx.x == 0)
    {
        Trailer t{};
        t.magic          = kMagic;
        t.version        = kVersion;
        t.kind           = kKindGeom;
        t.node_format    = b.format;
        t.leaf_count     = it.n;
        t.node_count     = it.n == 0 ? 0 : 2 * it.n - 1;
        t.wide_nodes_off = it.wide_off;
        t.wide_tris_off  = it.tris_off;
        t.wide_capacity  = it.wide_capacity;
        t.tri_capacity   = it.tri_capacity;
        t.morton_bits    = b.morton_bits;
        t.prim_kind      = it.prim_kind;
        *reinterpret_cast<Trailer*>(it.result + it.trailer_off) = t;
    }
    if (it.n == 0) return;
    uint32_t* bounds = reinterpret_cast<uint32_t*>(it.scratch + it.s_bounds);
    if (threadIdx.x < 8) bounds[threadIdx.x] = threadIdx.x < 4 ? 0xffffffffu : 0u;
    const uint32_t passes = b.morton_bits > 32 ? 8u : 4u;
    uint32_t*      ss     = sort_words(it);
    for (uint32_t k = threadIdx.x; k < passes * 256u + 64u; k += blockDim.x) ss[k] = 0;
}

struct TileRef
{
    uint32_t g;
    uint32_t tile;  // tile within the geometry
};
__device__ __forceinline__ TileRef tile_ref(const BatchArgs& b, uint32_t t)
{
    const uint32_t g = batch_find(b.tile_prefix, b.count, t);
    return TileRef{g, t - __ldg(b.tile_prefix + g)};
}

// Exact box of the referenced vertices of one tile's triangles; also zeroes
// the tile's look-back words of every sort pass.
template <int kBits>
__global__ void __launch_bounds__(kBlk) k_batch_bounds(BatchArgs b)
{
    using Cfg            = KeyCfg<kBits>;
    const TileRef    r   = tile_ref(b, blockIdx.x);
    const BuildItem& it  = b.items[r.g];
    const uint32_t   n   = it.n;
    const uint64_t   beg = (uint64_t)r.tile * Cfg::kTile;
    const uint64_t   end = min((uint64_t)n, beg + Cfg::kTile);
    uint32_t         lo[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, hi[3] = {0u, 0u, 0u};
#pragma unroll 4
    for (uint64_t t = beg + threadIdx.x; t < end; t += kBlk)
    {
        F3 a, bb, c;
        tri_verts(it, (uint32_t)t, a, bb, c);
        F3 l = vmin(vmin(a, bb), c), h = vmax(vmax(a, bb), c);
        lo[0] = min(lo[0], f2ord(l.x));
        lo[1] = min(lo[1], f2ord(l.y));
        lo[2] = min(lo[2], f2ord(l.z));
        hi[0] = max(hi[0], f2ord(h.x));
        hi[1] = max(hi[1], f2ord(h.y));
        hi[2] = max(hi[2], f2ord(h.z));
    }
    __shared__ uint32_t s[6][kBlk / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 3; ++k)
    {
        uint32_t x = __reduce_min_sync(0xffffffffu, lo[k]);
        uint32_t y = __reduce_max_sync(0xffffffffu, hi[k]);
        if (lane == 0)
        {
            s[k][w]     = x;
            s[k + 3][w] = y;
        }
    }
    uint32_t* lb = sort_words(it) + Cfg::kPasses * 256u + 64u;
#pragma unroll
    for (uint32_t p = 0; p < Cfg::kPasses; ++p) lb[((size_t)p * it.tiles + r.tile) * 256u + threadIdx.x] = 0;
    __syncthreads();
    if (threadIdx.x < 6)
    {
        const int k = threadIdx.x;
        uint32_t  v = s[k][0];
        for (int i = 1; i < kBlk / 32; ++i) v = k < 3 ? min(v, s[k][i]) : max(v, s[k][i]);
        uint32_t* bounds = reinterpret_cast<uint32_t*>(it.scratch + it.s_bounds);
        if (k < 3)
            atomicMin(&bounds[k], v);
        else
            atomicMax(&bounds[k + 1], v);
    }
}

// Morton codes of one tile's triangle box centres and the tile's digit
// histograms of every sort pass.
template <int kBits>
__global__ void __launch_bounds__(kBlk) k_batch_morton(BatchArgs b)
{
    using Cfg = KeyCfg<kBits>;
    __shared__ uint32_t h[Cfg::kPasses][256];
    for (uint32_t k = threadIdx.x; k < Cfg::kPasses * 256u; k += kBlk) (&h[0][0])[k] = 0;
    __syncthreads();
    const TileRef    r      = tile_ref(b, blockIdx.x);
    const BuildItem& it     = b.items[r.g];
    const uint32_t   n      = it.n;
    const uint32_t*  bounds = reinterpret_cast<const uint32_t*>(it.scratch + it.s_bounds);
    const F3         mlo    = f3(ord2f(bounds[0]), ord2f(bounds[1]), ord2f(bounds[2]));
    const F3         mhi    = f3(ord2f(bounds[4]), ord2f(bounds[5]), ord2f(bounds[6]));
    const F3         ext    = f3(mhi.x - mlo.x, mhi.y - mlo.y, mhi.z - mlo.z);
    const uint64_t   beg    = (uint64_t)r.tile * Cfg::kTile;
    const uint64_t   end    = min((uint64_t)n, beg + Cfg::kTile);
    void*            codes  = it.scratch + it.s_codes;
#pragma unroll 4
    for (uint64_t t = beg + threadIdx.x; t < end; t += kBlk)
    {
        F3 a, bb, c;
        tri_verts(it, (uint32_t)t, a, bb, c);
        F3 l = vmin(vmin(a, bb), c), hh = vmax(vmax(a, bb), c);
        F3 p = f3((0.5f * (l.x + hh.x) - mlo.x) / ext.x, (0.5f * (l.y + hh.y) - mlo.y) / ext.y,
                  (0.5f * (l.z + hh.z) - mlo.z) / ext.z);
        if (kBits == 63)
        {
            const float s = 2097152.0f;
            uint64_t    x = (uint64_t)clampf(p.x * s, 0.f, s - 1.f), y = (uint64_t)clampf(p.y * s, 0.f, s - 1.f),
                     z = (uint64_t)clampf(p.z * s, 0.f, s - 1.f);
            const uint64_t code = (expand_bits21(x) << 2) | (expand_bits21(y) << 1) | expand_bits21(z);
            ((uint64_t*)codes)[t] = code;
#pragma unroll
            for (uint32_t q = 0; q < Cfg::kPasses; ++q) atomicAdd(&h[q][(code >> (8 * q)) & 0xffu], 1u);
        }
        else
        {
            const float s = 1024.0f;
            uint32_t    x = (uint32_t)clampf(p.x * s, 0.f, s - 1.f), y = (uint32_t)clampf(p.y * s, 0.f, s - 1.f),
                     z = (uint32_t)clampf(p.z * s, 0.f, s - 1.f);
            const uint32_t code = (expand_bits(x) << 2) | (expand_bits(y) << 1) | expand_bits(z);
            ((uint32_t*)codes)[t] = code;
#pragma unroll
            for (uint32_t q = 0; q < Cfg::kPasses; ++q) atomicAdd(&h[q][(code >> (8 * q)) & 0xffu], 1u);
        }
    }
    __syncthreads();
    uint32_t* gh = sort_words(it);
    for (uint32_t k = threadIdx.x; k < Cfg::kPasses * 256u; k += kBlk)
    {
        const uint32_t v = (&h[0][0])[k];
        if (v) atomicAdd(gh + k, v);
    }
    if (r.tile == 0 && threadIdx.x < 8)
    {
        Trailer* tr                 = reinterpret_cast<Trailer*>(it.result + it.trailer_off);
        tr->bounds[threadIdx.x] = (threadIdx.x & 3) == 3 ? 0u : bounds[threadIdx.x];
    }
}

template <int kBits>
__global__ void __launch_bounds__(kBlk) k_batch_emit(BatchArgs b)
{
    using Cfg            = KeyCfg<kBits>;
    const uint32_t   t   = blockIdx.x / Cfg::kChunks;
    const TileRef    r   = tile_ref(b, t);
    const BuildItem& it  = b.items[r.g];
    const uint64_t   i64 = ((uint64_t)r.tile * Cfg::kChunks + blockIdx.x % Cfg::kChunks) * kChunk + threadIdx.x;
    if (i64 + 1 >= it.n) return;
    emit_node_topo<kBits>(it.scratch + it.s_codes, it.n, (uint32_t)i64, topo_of(it));
}

// ---- treelet restructure (quality build) -----------------------------------
// The reference's optional pass (restructure_hlbvh.cpp:133-278,
// restructure_bvh.comp; Karras & Aila 2013) restated deterministically: in
// post-order -- a bottom-up climb where the second child to arrive continues --
// every internal node X with at least `min_prims` triangles below it roots a
// treelet of up to 7 subtrees, grown by splitting the treelet leaf with the
// largest surface area (first on ties).  The topology of the treelet's
// internal nodes is replaced by the one that minimises the sum of node
// half-areas (dynamic programming over its 127 subsets, first minimum in
// enumeration order) when that is strictly cheaper, and the treelet's boxes
// are refitted.  Each node depends only on its own, finished subtree, so the
// result is independent of scheduling and equals the oracle's rro_restructure.
// Node slots are reused: the layout (root 0, internal [0, n-2], leaves
// [n-1, 2n-2]) and all other fields stay as built.
struct Bx3
{
    F3 lo, hi;
};
__device__ __forceinline__ float half_area3(const Bx3& b)
{
    const F3 e = f3(b.hi.x - b.lo.x, b.hi.y - b.lo.y, b.hi.z - b.lo.z);
    return (e.x * e.y + e.y * e.z) + e.z * e.x;
}
__device__ __forceinline__ Bx3 box_of(const BvhNode* nodes, uint32_t c)
{
    Bx3 b;
    child_box(nodes, c, b.lo, b.hi);
    return b;
}
__device__ __forceinline__ void store_child_boxes(BvhNode* nodes, uint32_t x)
{
    BvhNode*       nd = nodes + x;
    const uint32_t c0 = __ldcg(&nd->child0), c1 = __ldcg(&nd->child1), parent = __ldcg(&nd->parent);
    F3             lo0, hi0, lo1, hi1;
    child_box(nodes, c0, lo0, hi0);
    child_box(nodes, c1, lo1, hi1);
    // Every internal node under the node being restructured has been climbed
    // through in this pass, so its flag is 1.
    store_boxes4(nodes, x, lo0, hi0, lo1, hi1, c0, c1, parent, 1u);
}

// Shared tables of one warp's treelet optimisation.
struct TreeletDp
{
    float   area[128];
    float   cost[128];
    uint8_t part[128];
};

// Best split of subset s (first minimum in the order of decreasing p over the
// proper subsets p of s that hold s's lowest bit), scanning the partitions
// with index i = j, j + stride, ... in that order.
__device__ __forceinline__ void best_split(const TreeletDp& t, uint32_t s, uint32_t j, uint32_t stride, float& best,
                                           uint32_t& bp)
{
    const uint32_t low = s & (0u - s);
    best               = 0.f;
    bp                 = 0;
    uint32_t idx       = 0;
    for (uint32_t p = (s - 1) & s; p; p = (p - 1) & s)
    {
        if (!(p & low)) continue;
        if (idx++ % stride != j) continue;
        const float c = t.cost[p] + t.cost[s ^ p];
        if (bp == 0 || c < best)
        {
            best = c;
            bp   = p;
        }
    }
}

// An internal node as one 64-byte load: its children and their boxes (the
// copies its own slots hold, which the refit and every restructure keep equal
// to the child's own box), and its parent.
struct NodeLd
{
    uint32_t c0, c1, parent;
    Bx3      b0, b1;
};
__device__ __forceinline__ NodeLd load_node_cg(const BvhNode* nodes, uint32_t x)
{
    const float4* p4 = reinterpret_cast<const float4*>(nodes + x);
    const float4  w0 = __ldcg(p4), w1 = __ldcg(p4 + 1), w2 = __ldcg(p4 + 2), w3 = __ldcg(p4 + 3);
    NodeLd        d;
    d.c0     = __float_as_uint(w0.w);
    d.c1     = __float_as_uint(w1.w);
    d.parent = __float_as_uint(w2.w);
    d.b0     = Bx3{f3(w0.x, w0.y, w0.z), f3(w1.x, w1.y, w1.z)};
    d.b1     = Bx3{f3(w2.x, w2.y, w2.z), f3(w3.x, w3.y, w3.z)};
    return d;
}

// Restructure the treelet rooted at internal node x with the whole warp (all
// 32 lanes call it with the same x).  Same treelet, same tables, same tie rules
// as the sequential restatement (oracle rro_restructure), so the tree is
// identical: every lane forms the treelet (same loads); subset areas are
// spread over the lanes; subsets are costed by size, one lane per subset, and
// the largest subset (the whole treelet) by all lanes with a min reduction
// that keeps the first minimum in enumeration order; lane 0 rebuilds.
// Latency: forming the treelet costs one node load per expansion (the child
// boxes come from the parent's slots), and the rebuild writes each new node
// whole from boxes it unions in registers, bottom-up, exactly as the child's
// own node would give them (child_box).
__device__ void restructure_treelet_warp(BvhNode* nodes, uint32_t n, uint32_t x, TreeletDp& t, uint32_t lane)
{
    uint32_t leaf[7], inner[6];
    float    la[7], ia[6];
    Bx3      bx[7];
    int      nl = 2, ni = 1;
    const NodeLd r = load_node_cg(nodes, x);
    inner[0]       = x;
    leaf[0]        = r.c0;
    leaf[1]        = r.c1;
    bx[0]          = r.b0;
    bx[1]          = r.b1;
    la[0]          = half_area3(bx[0]);
    la[1]          = half_area3(bx[1]);
    while (nl < 7)
    {
        int   best = -1;
        float ba   = -1.f;
        for (int k = 0; k < nl; ++k)
            if (leaf[k] < n - 1 && la[k] > ba)
            {
                ba   = la[k];
                best = k;
            }
        if (best < 0) break;
        const uint32_t c = leaf[best];
        const NodeLd   d = load_node_cg(nodes, c);
        ia[ni]           = la[best];  // the area of c's box, which its parent's slot holds
        inner[ni++]      = c;
        leaf[best]       = d.c0;
        bx[best]         = d.b0;
        la[best]         = half_area3(d.b0);
        leaf[nl]         = d.c1;
        bx[nl]           = d.b1;
        la[nl]           = half_area3(d.b1);
        ++nl;
    }
    if (nl < 3) return;  // warp-uniform: every lane formed the same treelet
    const uint32_t full = (1u << nl) - 1;
    for (uint32_t s = lane + 1; s <= full; s += 32)
    {
        const int lo = __ffs(s) - 1;
        Bx3       u  = bx[lo];
        for (int k = lo + 1; k < nl; ++k)
            if (s >> k & 1u)
            {
                u.lo = vmin(u.lo, bx[k].lo);
                u.hi = vmax(u.hi, bx[k].hi);
            }
        t.area[s] = half_area3(u);
        if ((s & (s - 1)) == 0)
        {
            t.cost[s] = t.area[s];
            t.part[s] = 0;
        }
    }
    __syncwarp();
    for (int size = 2; size < nl; ++size)
    {
        for (uint32_t s = lane + 1; s <= full; s += 32)
        {
            if (__popc(s) != size) continue;
            float    best;
            uint32_t bp;
            best_split(t, s, 0, 1, best, bp);
            t.cost[s] = t.area[s] + best;
            t.part[s] = (uint8_t)bp;
        }
        __syncwarp();
    }
    {
        // The whole treelet: lanes split its partitions, then reduce.
        float    best;
        uint32_t bp;
        best_split(t, full, lane, 32, best, bp);
        for (int o = 16; o; o >>= 1)
        {
            const float    ob = __shfl_xor_sync(0xffffffffu, best, o);
            const uint32_t op = __shfl_xor_sync(0xffffffffu, bp, o);
            // Keep the first minimum in enumeration order: the smaller cost,
            // or on equal cost the larger p (p decreases along the order).
            if (op != 0 && (bp == 0 || ob < best || (ob == best && op > bp)))
            {
                best = ob;
                bp   = op;
            }
        }
        if (lane == 0)
        {
            t.cost[full] = t.area[full] + best;
            t.part[full] = (uint8_t)bp;
        }
    }
    __syncwarp();
    if (lane == 0)
    {
        float cur = t.area[full];
        for (int k = 1; k < ni; ++k) cur += ia[k];
        for (int k = 0; k < nl; ++k) cur += la[k];
        if (t.cost[full] < cur)
        {
            // New topology, top-down: node k of the rebuild takes slot
            // inner[k] (k = 0 is x), covers the treelet leaves in subset
            // sub[k], and has children c0/c1 (a slot, or a treelet leaf).
            // Slots go to the inner nodes in the order of a depth-first walk
            // with a stack (the order the oracle's rebuild assigns them).
            uint32_t sub[6], c0[6], c1[6], par[6];
            int      kid0[6], kid1[6];  // rebuild index of an inner child, -1 for a treelet leaf
            int      stk[6], sp = 0, no = 1;
            sub[0]    = full;
            par[0]    = r.parent;
            stk[sp++] = 0;
            while (sp > 0)
            {
                const int k = stk[--sp];
                const uint32_t sides[2] = {t.part[sub[k]], sub[k] ^ t.part[sub[k]]};
                for (int e = 0; e < 2; ++e)
                {
                    const uint32_t u = sides[e];
                    uint32_t       c;
                    int            kid = -1;
                    if ((u & (u - 1)) == 0)
                        c = leaf[__ffs(u) - 1];
                    else
                    {
                        kid       = no++;
                        c         = inner[kid];
                        sub[kid]  = u;
                        par[kid]  = inner[k];
                        stk[sp++] = kid;
                    }
                    (e ? c1 : c0)[k]     = c;
                    (e ? kid1 : kid0)[k] = kid;
                }
            }
            // Boxes bottom-up (children have larger rebuild indices), each
            // node written whole; treelet leaves take their new parent.
            Bx3 nb[6];
            for (int k = no - 1; k >= 0; --k)
            {
                const Bx3 l0 = kid0[k] < 0 ? bx[__ffs(t.part[sub[k]]) - 1] : nb[kid0[k]];
                const Bx3 l1 = kid1[k] < 0 ? bx[__ffs(sub[k] ^ t.part[sub[k]]) - 1] : nb[kid1[k]];
                nb[k]        = Bx3{vmin(l0.lo, l1.lo), vmax(l0.hi, l1.hi)};
                // Every internal node under the node being restructured has
                // been climbed through in this pass, so its flag is 1.
                store_boxes4(nodes, inner[k], l0.lo, l0.hi, l1.lo, l1.hi, c0[k], c1[k], par[k], 1u);
                if (kid0[k] < 0) __stcg(&nodes[c0[k]].parent, inner[k]);
                if (kid1[k] < 0) __stcg(&nodes[c1[k]].parent, inner[k]);
            }
            __threadfence();
        }
    }
    __syncwarp();
}

// One restructure pass of every geometry: leaf threads climb; the second to
// arrive at a node counts its triangles and restructures it if it has enough.
template <int kBits>
__global__ void __launch_bounds__(kRsBlk) k_batch_restructure(BatchArgs b, DeviceWords* words)
{
    using Cfg            = KeyCfg<kBits>;
    constexpr uint32_t kPer = Cfg::kTile / kRsBlk;  // blocks per sort tile
    const uint32_t   t   = blockIdx.x / kPer;
    const TileRef    r   = tile_ref(b, t);
    const BuildItem& it  = b.items[r.g];
    const uint64_t   k64 = ((uint64_t)r.tile * kPer + blockIdx.x % kPer) * kRsBlk + threadIdx.x;
    const uint32_t   n   = it.n;
    if (n < 3) return;  // block-uniform: a block covers one geometry
    __shared__ TreeletDp dp[kRsBlk / 32];
    TreeletDp&     tdp   = dp[threadIdx.x >> 5];
    const uint32_t lane  = threadIdx.x & 31;
    BvhNode*       nodes = reinterpret_cast<BvhNode*>(it.result);
    uint32_t*      cnt   = reinterpret_cast<uint32_t*>(it.scratch + it.s_codes);  // free after emit: 2n-1 counts
    // The warp climbs together: every round, each live lane takes one step
    // up; then the warp restructures, one after another, the treelets of the
    // lanes whose node qualified.
    bool     alive = k64 < n;
    uint32_t addr  = kInvalid;
    if (alive)
    {
        const uint32_t leaf = n - 1 + (uint32_t)k64;
        __stcg(&cnt[leaf], 1u);
        addr  = __ldcg(&nodes[leaf].parent);
        alive = addr != kInvalid;
    }
    for (int level = 0; __any_sync(0xffffffffu, alive); ++level)
    {
        bool need = false;
        if (alive)
        {
            if (addr >= n - 1 || level > 96)
            {
                atomicOr(&words->error_bits, (uint32_t)RR_CUDA_DEVICE_ERROR_NODE_RANGE);
                alive = false;
            }
            else
            {
                if (climb_exch(&nodes[addr].update) == 0u)
                    alive = false;
                else
                {
                    const uint32_t c0 = __ldcg(&nodes[addr].child0), c1 = __ldcg(&nodes[addr].child1);
                    if (c0 >= 2 * n - 1 || c1 >= 2 * n - 1)
                    {
                        atomicOr(&words->error_bits, (uint32_t)RR_CUDA_DEVICE_ERROR_NODE_RANGE);
                        alive = false;
                    }
                    else
                    {
                        const uint32_t c = __ldcg(&cnt[c0]) + __ldcg(&cnt[c1]);
                        __stcg(&cnt[addr], c);
                        need = c >= b.restructure_min;
                    }
                }
            }
        }
        for (uint32_t m = __ballot_sync(0xffffffffu, need); m; m &= m - 1)
        {
            const uint32_t x = __shfl_sync(0xffffffffu, addr, __ffs(m) - 1);
            restructure_treelet_warp(nodes, n, x, tdp, lane);
        }
        if (alive)
        {
            addr  = __ldcg(&nodes[addr].parent);
            alive = addr != kInvalid;
        }
    }
}

// Every node's climb flag back to 0 before a restructure pass.
__global__ void __launch_bounds__(kBlk) k_batch_reset_flags(BatchArgs b)
{
    for (uint32_t g = blockIdx.y; g < b.count; g += gridDim.y)
    {
        const BuildItem& it    = b.items[g];
        const uint64_t   m     = it.n >= 3 ? 2ull * it.n - 1 : 0;  // smaller trees are not restructured
        BvhNode*         nodes = reinterpret_cast<BvhNode*>(it.result);
        for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m;
             i += (uint64_t)gridDim.x * blockDim.x)
            nodes[i].update = 0;
    }
}

// Box of node s for its parent's slot, read without a dependent load: a
// node's kind follows from its index (binary layout: leaves [n-1, 2n-2]).
__device__ __forceinline__ void node_box(const BvhNode* nodes, uint32_t s, uint32_t n, F3& lo, F3& hi)
{
    const float4* p4 = reinterpret_cast<const float4*>(nodes + s);
    const float4  w0 = __ldcg(p4), w1 = __ldcg(p4 + 1), w2 = __ldcg(p4 + 2);
    const F3      a = f3(w0.x, w0.y, w0.z), b = f3(w1.x, w1.y, w1.z), p = f3(w2.x, w2.y, w2.z);
    if (s >= n - 1)
    {
        lo = vmin(vmin(a, b), p);
        hi = vmax(vmax(a, b), p);
    }
    else
    {
        const float4 w3 = __ldcg(p4 + 3);
        lo              = vmin(a, p);
        hi              = vmax(b, f3(w3.x, w3.y, w3.z));
    }
}

// Leaf k of a geometry takes triangle `prim`'s vertices, then climbs: the
// second child to arrive at a node (atomic flag) writes the node's two child
// boxes and goes on to its parent (lbvh_fit_aabb_mesh.comp:94-205).  The
// thread carries the box of the subtree it completed, so at a node it reads
// only the sibling's box; the node's child and parent words (written by the
// emit, unchanged by the climb) are read before the flag, so those loads
// overlap the atomic.  The boxes are the reference's: a node's box is the
// union of its two child boxes, slot 0 first.
// kTopo: a build -- the topology comes from the compact arrays (topo_of)
// and every node is written whole; otherwise an update of a built tree,
// whose nodes hold the topology and the climb flags.
template <bool kTopo>
__device__ __forceinline__ void fit_leaf(const BuildItem& it, BvhNode* nodes, uint32_t n, uint32_t k, uint32_t prim,
                                         DeviceWords* words)
{
    const uint32_t leaf = n - 1 + k;
    F3             a, bb, c;
    tri_verts(it, prim, a, bb, c);
    Topo topo{};
    if (kTopo && n > 1) topo = topo_of(it);
    uint32_t parent = (n == 1) ? kInvalid : (kTopo ? __ldcg(&topo.parent[leaf]) : __ldcg(&nodes[leaf].parent));
    float4*  dst    = reinterpret_cast<float4*>(nodes + leaf);
    __stcg(dst + 0, make_float4(a.x, a.y, a.z, __uint_as_float(kInvalid)));
    __stcg(dst + 1, make_float4(bb.x, bb.y, bb.z, __uint_as_float(prim)));
    __stcg(dst + 2, make_float4(c.x, c.y, c.z, __uint_as_float(parent)));
    __stcg(dst + 3, make_float4(0.f, 0.f, 0.f, __uint_as_float(0u)));
    F3       lo = vmin(vmin(a, bb), c), hi = vmax(vmax(a, bb), c);
    uint32_t x = leaf, addr = parent;
    // A Karras tree over 2^30 leaves with 32-bit index tie-breaks is at most
    // 64 levels deep; the bound and the range checks only guard against a
    // corrupted tree (they raise NODE_RANGE instead of faulting or spinning).
    for (int level = 0; addr != kInvalid; ++level)
    {
        if (addr >= n - 1 || level > 96)
        {
            atomicOr(&words->error_bits, (uint32_t)RR_CUDA_DEVICE_ERROR_NODE_RANGE);
            return;
        }
        BvhNode* nd = nodes + addr;
        uint32_t c0, c1, up;
        if (kTopo)
        {
            const uint2 ch = __ldcg(&topo.child[addr]);
            c0             = ch.x;
            c1             = ch.y;
            up             = __ldcg(&topo.parent[addr]);
        }
        else
        {
            c0 = __ldcg(&nd->child0);
            c1 = __ldcg(&nd->child1);
            up = __ldcg(&nd->parent);
        }
        if (climb_exch(kTopo ? &topo.flag[addr] : &nd->update) == 0u) return;
        if (c0 >= 2 * n - 1 || c1 >= 2 * n - 1 || (c0 != x && c1 != x))
        {
            atomicOr(&words->error_bits, (uint32_t)RR_CUDA_DEVICE_ERROR_NODE_RANGE);
            return;
        }
        // This thread arrived second: the flag is 1, the sibling's box is
        // complete, and no other thread writes this node any more.
        F3 slo, shi;
        node_box(nodes, c0 == x ? c1 : c0, n, slo, shi);
        const F3 lo0 = c0 == x ? lo : slo, hi0 = c0 == x ? hi : shi;
        const F3 lo1 = c0 == x ? slo : lo, hi1 = c0 == x ? shi : hi;
        store_boxes4(nodes, addr, lo0, hi0, lo1, hi1, c0, c1, up, 1u);
        lo   = vmin(lo0, lo1);
        hi   = vmax(hi0, hi1);
        x    = addr;
        addr = up;
    }
}

template <int kBits>
__global__ void __launch_bounds__(kFitBlk) k_batch_refit(BatchArgs b, DeviceWords* words)
{
    using Cfg            = KeyCfg<kBits>;
    constexpr uint32_t kPer = Cfg::kTile / kFitBlk;  // blocks per sort tile
    const uint32_t   t   = blockIdx.x / kPer;
    const TileRef    r   = tile_ref(b, t);
    const BuildItem& it  = b.items[r.g];
    const uint64_t   k64 = ((uint64_t)r.tile * kPer + blockIdx.x % kPer) * kFitBlk + threadIdx.x;
    const uint32_t   n   = it.n;
    if (k64 >= n) return;
    const uint32_t  k          = (uint32_t)k64;
    BvhNode*        nodes      = reinterpret_cast<BvhNode*>(it.result);
    const uint32_t* sorted_idx = reinterpret_cast<const uint32_t*>(it.scratch + it.s_idx);
    fit_leaf<true>(it, nodes, n, k, sorted_idx[k], words);
}

// RR_BUILD_OPERATION_UPDATE (lbvh_reset_update_flags.comp:58-80): every
// node's flag back to 0.  The reference dispatches this with one group only
// (vlk/update_hlbvh.cpp:150) and so leaves most flags at 1; here every node
// is reset.
__global__ void __launch_bounds__(kBlk) k_update_reset(BvhNode* nodes, uint32_t count)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) nodes[i].update = 0;
}

// lbvh_fit_aabb_mesh.comp:129-205 with UPDATE_KERNEL: the leaf keeps its
// primitive (child1) and takes the new vertices, then the usual climb.
__global__ void __launch_bounds__(kFitBlk) k_update_fit(BuildItem it, DeviceWords* words)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= it.n) return;
    BvhNode* nodes = reinterpret_cast<BvhNode*>(it.result);
    fit_leaf<false>(it, nodes, it.n, k, __ldcg(&nodes[it.n - 1 + k].child1), words);
}

__global__ void k_put_single(BuildItem* items, BuildItem it, uint32_t* tile_prefix, uint32_t tiles)
{
    if (threadIdx.x == 0)
    {
        items[0]       = it;
        tile_prefix[0] = 0;
        tile_prefix[1] = tiles;
    }
}

__global__ void k_init_trailer(Trailer* t, Trailer v) { *t = v; }

inline int grid_for(uint64_t n, int block) { return (int)std::max<uint64_t>(1, (n + block - 1) / block); }
template <int kBits>
cudaError_t run_batch(const BatchArgs& b, DeviceWords* words, int sm_count, cudaStream_t s)
{
    using Cfg = KeyCfg<kBits>;
    if (radix_sort_tile_keys(kBits) != Cfg::kTile) return cudaErrorInvalidConfiguration;
    k_batch_bounds<kBits><<<b.total_tiles, kBlk, 0, s>>>(b);
    k_batch_morton<kBits><<<b.total_tiles, kBlk, 0, s>>>(b);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if ((e = launch_radix_sort_batch(b, words, s)) != cudaSuccess) return e;
    const uint64_t blocks = (uint64_t)b.total_tiles * Cfg::kChunks;
    if (blocks > 0x7fffffffull) return cudaErrorInvalidConfiguration;
    k_batch_emit<kBits><<<(unsigned)blocks, kBlk, 0, s>>>(b);
    k_batch_refit<kBits><<<(unsigned)(b.total_tiles * (Cfg::kTile / kFitBlk)), kFitBlk, 0, s>>>(b, words);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (b.restructure_min)
    {
        const dim3 rgrid((unsigned)std::max<uint64_t>(1, std::min<uint64_t>((2ull * b.max_n + kBlk - 1) / kBlk,
                                                                            (uint64_t)sm_count * 8)),
                         std::min<uint32_t>(b.count, 65535u));
        for (uint32_t pass = 0; pass < b.restructure_passes; ++pass)
        {
            k_batch_reset_flags<<<rgrid, kBlk, 0, s>>>(b);
            k_batch_restructure<kBits><<<(unsigned)(b.total_tiles * (Cfg::kTile / kRsBlk)), kRsBlk, 0, s>>>(b, words);
        }
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if (has_wide_collapse(b.format)) return launch_collapse_batch(b, words, sm_count, s);
    return cudaSuccess;
}

}  // namespace

size_t batch_desc_bytes(uint32_t count)
{
    return align_up((size_t)count * sizeof(BuildItem), kAlign) + 2 * align_up(((size_t)count + 1) * 4, kAlign) +
           align_up(sizeof(BatchCtl), kAlign);
}

void batch_carve(uint8_t* block, uint32_t count, BuildItem** items, uint32_t** tile_prefix, uint32_t** level_prefix,
                 BatchCtl** ctl)
{
    size_t off    = 0;
    *items        = reinterpret_cast<BuildItem*>(block + off);
    off           = align_up((size_t)count * sizeof(BuildItem), kAlign);
    *tile_prefix  = reinterpret_cast<uint32_t*>(block + off);
    off          += align_up(((size_t)count + 1) * 4, kAlign);
    *level_prefix = reinterpret_cast<uint32_t*>(block + off);
    off          += align_up(((size_t)count + 1) * 4, kAlign);
    *ctl          = reinterpret_cast<BatchCtl*>(block + off);
}

GeomLayout geom_layout(uint32_t n, uint32_t format, uint32_t morton_bits)
{
    GeomLayout L{};
    L.n           = n;
    L.format      = format;
    L.morton_bits = morton_bits == 63 ? 63 : 30;
    const size_t nodes = n == 0 ? 0 : 2ull * n - 1;
    L.nodes_bytes = nodes * sizeof(BvhNode);
    L.trailer_off = align_up(L.nodes_bytes, kAlign);
    size_t off    = L.trailer_off + sizeof(Trailer);
    if (format == RR_CUDA_NODE_FORMAT_WIDE8 && n > 0)
    {
        L.wide_off      = align_up(off, kAlign);
        L.wide_capacity = std::max<size_t>(1, (size_t)n - 1);
        L.tris_off      = align_up(L.wide_off + L.wide_capacity * sizeof(WideNode), kAlign);
        L.tri_capacity  = n;
        off             = L.tris_off + L.tri_capacity * sizeof(WideTri);
    }
    else if (is_bvh4_format(format) && n > 0)
    {
        // Only a node whose children are all leaves has fewer than 4
        // children, so with F full nodes and B such nodes 3F + B <= n - 1 and
        // B <= n / 2, hence F + B <= (n - 1) / 3 + n / 3 + 1.
        L.wide_off      = align_up(off, kAlign);
        L.wide_capacity = ((size_t)n - 1) / 3 + (size_t)n / 3 + 1;
        L.tris_off      = 0;
        L.tri_capacity  = 0;
        off             = L.wide_off + L.wide_capacity *
                                       (format == RR_CUDA_NODE_FORMAT_BVH4Q8 ? sizeof(Bvh4QNode) : sizeof(Bvh4Node));
    }
    L.total = align_up(off, kAlign);
    // Scratch: batch descriptor of one | bounds | codes | codes_alt | idx |
    // idx_alt | sort | collapse queues.
    const size_t kb = L.morton_bits == 63 ? 8 : 4;
    L.s_desc        = 0;
    L.s_bounds      = align_up(batch_desc_bytes(1), kAlign);
    L.s_codes       = L.s_bounds + kAlign;
    L.s_codes_alt   = align_up(L.s_codes + kb * n, kAlign);
    L.s_idx         = align_up(L.s_codes_alt + kb * n, kAlign);
    L.s_idx_alt     = align_up(L.s_idx + 4ull * n, kAlign);
    L.s_sort        = align_up(L.s_idx_alt + 4ull * n, kAlign);
    L.s_sort_bytes  = radix_sort_scratch_bytes(n, (int)L.morton_bits, &L.sort_tiles, &L.sort_passes);
    L.s_queue       = align_up(L.s_sort + L.s_sort_bytes, kAlign);
    L.s_queue_bytes =
        (has_wide_collapse(format) && n > 0) ? 2 * kAlign + 2ull * 8ull * n : 0;
    L.s_topo        = align_up(L.s_queue + L.s_queue_bytes, kAlign);
    L.s_total       = align_up(L.s_topo + topo_bytes(n), kAlign);
    // An update re-collapses the wide nodes: descriptor of one + queues.
    L.u_queue = align_up(batch_desc_bytes(1), kAlign);
    L.u_total = L.s_queue_bytes ? align_up(L.u_queue + L.s_queue_bytes, kAlign) : 0;
    return L;
}

BuildItem make_build_item(const GeomLayout& L, const float* vertices, uint64_t stride_floats, const void* indices,
                          int index16, uint8_t* scratch, uint8_t* result, uint32_t prim_kind)
{
    BuildItem it{};
    it.vertices      = vertices;
    it.indices       = indices;
    it.scratch       = scratch;
    it.result        = result;
    it.stride_floats = stride_floats;
    it.s_bounds      = L.s_bounds;
    it.s_codes       = L.s_codes;
    it.s_codes_alt   = L.s_codes_alt;
    it.s_idx         = L.s_idx;
    it.s_idx_alt     = L.s_idx_alt;
    it.s_sort        = L.s_sort;
    it.s_queue       = L.s_queue;
    it.s_topo        = L.s_topo;
    it.trailer_off   = L.trailer_off;
    it.wide_off      = L.wide_off;
    it.tris_off      = L.tris_off;
    it.wide_capacity = (uint32_t)L.wide_capacity;
    it.tri_capacity  = (uint32_t)L.tri_capacity;
    it.n             = L.n;
    it.index16       = index16 ? 1u : 0u;
    it.tiles         = L.sort_tiles;
    it.prim_kind     = prim_kind;
    return it;
}

cudaError_t launch_emit(const void* sorted_codes, int bits, uint32_t n, BvhNode* nodes, cudaStream_t s)
{
    if (n < 2) return cudaSuccess;
    if (bits == 63)
        k_emit<63><<<grid_for(n - 1, 256), 256, 0, s>>>(sorted_codes, n, nodes);
    else
        k_emit<30><<<grid_for(n - 1, 256), 256, 0, s>>>(sorted_codes, n, nodes);
    return cudaGetLastError();
}

cudaError_t launch_build_batch(const BatchArgs& b, DeviceWords* words, int sm_count, cudaStream_t s)
{
    if (b.count == 0) return cudaSuccess;
    k_batch_init<<<b.count, kBlk, 0, s>>>(b);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || b.total_tiles == 0) return e;
    return b.morton_bits == 63 ? run_batch<63>(b, words, sm_count, s) : run_batch<30>(b, words, sm_count, s);
}

cudaError_t launch_update_mesh(const MeshArgs& m, const GeomLayout& L, uint8_t* scratch, uint8_t* result,
                               DeviceWords* words, int sm_count, cudaStream_t s)
{
    if (L.n == 0) return cudaSuccess;
    BuildItem it = make_build_item(L, m.vertices, m.stride_floats, m.indices, m.index16, scratch, result, m.prim_kind);
    it.s_queue   = L.u_queue;
    k_update_reset<<<grid_for(2ull * L.n - 1, kBlk), kBlk, 0, s>>>(reinterpret_cast<BvhNode*>(result), 2 * L.n - 1);
    k_update_fit<<<grid_for(L.n, kFitBlk), kFitBlk, 0, s>>>(it, words);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || !has_wide_collapse(L.format)) return e;
    // 4-wide nodes keep their topology and take the new boxes in one pass
    // (measured on the 4.2 M-triangle heightfield: 0.90 ms for the whole
    // update with the collapse run again); 8-wide nodes are collapsed again.
    if (is_bvh4_format(L.format)) return launch_refit_bvh4(result, L, words, sm_count, s);
    BuildItem* items = nullptr;
    uint32_t * tp = nullptr, *lp = nullptr;
    BatchCtl*  ctl = nullptr;
    batch_carve(scratch, 1, &items, &tp, &lp, &ctl);
    k_put_single<<<1, 32, 0, s>>>(items, it, tp, L.sort_tiles);
    BatchArgs b{};
    b.items        = items;
    b.tile_prefix  = tp;
    b.level_prefix = lp;
    b.ctl          = ctl;
    b.count        = 1;
    b.total_tiles  = L.sort_tiles;
    b.total_prims  = L.n;
    b.max_n        = L.n;
    b.format       = L.format;
    b.morton_bits  = L.morton_bits;
    return launch_collapse_batch(b, words, sm_count, s);
}

cudaError_t launch_build_mesh(const MeshArgs& m, const GeomLayout& L, uint8_t* scratch, uint8_t* result,
                              DeviceWords* words, int sm_count, cudaStream_t s)
{
    if (L.n == 0)
    {
        // No scratch is required for an empty mesh: write the trailer only.
        Trailer tr{};
        tr.magic       = kMagic;
        tr.version     = kVersion;
        tr.kind        = kKindGeom;
        tr.node_format = L.format;
        tr.morton_bits = L.morton_bits;
        tr.prim_kind   = m.prim_kind;
        k_init_trailer<<<1, 1, 0, s>>>(reinterpret_cast<Trailer*>(result + L.trailer_off), tr);
        return cudaGetLastError();
    }
    BuildItem* items = nullptr;
    uint32_t * tp = nullptr, *lp = nullptr;
    BatchCtl*  ctl = nullptr;
    batch_carve(scratch + L.s_desc, 1, &items, &tp, &lp, &ctl);
    k_put_single<<<1, 32, 0, s>>>(items, make_build_item(L, m.vertices, m.stride_floats, m.indices, m.index16, scratch,
                                                         result, m.prim_kind),
                                  tp, L.sort_tiles);
    BatchArgs b{};
    b.items        = items;
    b.tile_prefix  = tp;
    b.level_prefix = lp;
    b.ctl          = ctl;
    b.count        = 1;
    b.total_tiles  = L.sort_tiles;
    b.total_prims  = L.n;
    b.max_n        = L.n;
    b.format             = L.format;
    b.morton_bits        = L.morton_bits;
    b.restructure_min    = L.restructure_min;
    b.restructure_passes = L.restructure_passes;
    return launch_build_batch(b, words, sm_count, s);
}

}  // namespace rr
