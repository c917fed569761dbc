// build_lbvh.cu -- LBVH build of one triangle mesh on sm_103a.
//
// Pipeline (reference: vlk/hlbvh_builder.cpp:159-351):
//   k_mesh_bounds   lbvh_calc_mesh_aabb.comp:121-179  exact min/max of all
//                   referenced vertices, order-preserving uint atomics
//   k_morton        lbvh_calc_morton_codes_mesh.comp:78-130
//   radix sort      vlk/radix_sort.cpp (sort.cu, onesweep)
//   k_emit          lbvh_emit_hierarchy_mesh.comp:78-217 (Karras 2012)
//   k_refit         lbvh_fit_aabb_mesh.comp:94-205 (atomic bottom-up climb)
//   wide collapse   (wide.cu) when the WIDE8 node format is requested
//
// Arithmetic follows the oracle's rules (IEEE fp32, no contraction: the file
// is compiled with --fmad=false), so codes, permutation, topology and boxes
// are bit-identical to the CPU restatement.
#include <algorithm>

#include "rr_internal.h"

namespace rr
{
cudaError_t launch_collapse_wide(const GeomLayout& L, uint8_t* scratch, uint8_t* result, DeviceWords* words,
                                 int sm_count, cudaStream_t s);

namespace
{
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

__device__ __forceinline__ uint32_t tri_index(const MeshArgs& m, uint64_t k)
{
    return m.index16 ? (uint32_t)((const uint16_t*)m.indices)[k] : ((const uint32_t*)m.indices)[k];
}
__device__ __forceinline__ F3 vtx(const MeshArgs& m, uint32_t i)
{
    const float* p = m.vertices + (uint64_t)i * m.stride_floats;
    return f3(__ldg(p), __ldg(p + 1), __ldg(p + 2));
}
__device__ __forceinline__ void tri_verts(const MeshArgs& m, uint32_t t, F3& a, F3& b, F3& c)
{
    uint32_t i0 = tri_index(m, 3ull * t), i1 = tri_index(m, 3ull * t + 1), i2 = tri_index(m, 3ull * t + 2);
    a = vtx(m, i0);
    b = vtx(m, i1);
    c = vtx(m, i2);
}

// Exact mesh box over all referenced vertices.
__global__ void __launch_bounds__(256) k_mesh_bounds(MeshArgs m, uint32_t* bounds)
{
    uint32_t lo[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, hi[3] = {0u, 0u, 0u};
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < m.n; t += gridDim.x * blockDim.x)
    {
        F3 a, b, c;
        tri_verts(m, t, a, b, c);
        F3 l = vmin(vmin(a, b), c), h = vmax(vmax(a, b), c);
        lo[0] = min(lo[0], f2ord(l.x));
        lo[1] = min(lo[1], f2ord(l.y));
        lo[2] = min(lo[2], f2ord(l.z));
        hi[0] = max(hi[0], f2ord(h.x));
        hi[1] = max(hi[1], f2ord(h.y));
        hi[2] = max(hi[2], f2ord(h.z));
    }
    __shared__ uint32_t s[6][8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 3; ++k)
    {
        uint32_t a = __reduce_min_sync(0xffffffffu, lo[k]);
        uint32_t b = __reduce_max_sync(0xffffffffu, hi[k]);
        if (lane == 0)
        {
            s[k][w]     = a;
            s[k + 3][w] = b;
        }
    }
    __syncthreads();
    if (threadIdx.x < 6)
    {
        int      k = threadIdx.x;
        uint32_t v = s[k][0];
        for (int i = 1; i < (int)(blockDim.x >> 5); ++i) v = k < 3 ? min(v, s[k][i]) : max(v, s[k][i]);
        if (k < 3)
            atomicMin(&bounds[k], v);
        else
            atomicMax(&bounds[k + 1], v);
    }
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

template <int kBits>
__global__ void __launch_bounds__(256) k_morton(MeshArgs m, const uint32_t* __restrict__ bounds, void* codes)
{
    const F3 mlo = f3(ord2f(bounds[0]), ord2f(bounds[1]), ord2f(bounds[2]));
    const F3 mhi = f3(ord2f(bounds[4]), ord2f(bounds[5]), ord2f(bounds[6]));
    const F3 ext = f3(mhi.x - mlo.x, mhi.y - mlo.y, mhi.z - mlo.z);
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < m.n; t += gridDim.x * blockDim.x)
    {
        F3 a, b, c;
        tri_verts(m, t, a, b, c);
        F3 l = vmin(vmin(a, b), c), h = vmax(vmax(a, b), c);
        F3 p = f3((0.5f * (l.x + h.x) - mlo.x) / ext.x, (0.5f * (l.y + h.y) - mlo.y) / ext.y,
                  (0.5f * (l.z + h.z) - mlo.z) / ext.z);
        if (kBits == 63)
        {
            const float s = 2097152.0f;
            uint64_t    x = (uint64_t)clampf(p.x * s, 0.f, s - 1.f), y = (uint64_t)clampf(p.y * s, 0.f, s - 1.f),
                     z = (uint64_t)clampf(p.z * s, 0.f, s - 1.f);
            ((uint64_t*)codes)[t] = (expand_bits21(x) << 2) | (expand_bits21(y) << 1) | expand_bits21(z);
        }
        else
        {
            const float s = 1024.0f;
            uint32_t    x = (uint32_t)clampf(p.x * s, 0.f, s - 1.f), y = (uint32_t)clampf(p.y * s, 0.f, s - 1.f),
                     z = (uint32_t)clampf(p.z * s, 0.f, s - 1.f);
            ((uint32_t*)codes)[t] = (expand_bits(x) << 2) | (expand_bits(y) << 1) | expand_bits(z);
        }
    }
}

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

template <int kBits>
__global__ void __launch_bounds__(256) k_emit(const void* __restrict__ codes, uint32_t n, BvhNode* nodes)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i + 1 >= n) return;
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
    const int64_t e  = ii + l * d;
    const int64_t lo_e = ii < e ? ii : e, hi_e = ii < e ? e : ii;
    const int64_t sx = lo_e > 0 ? lo_e : 0;
    const int64_t sy = hi_e < (int64_t)n - 1 ? hi_e : (int64_t)n - 1;
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

__device__ __forceinline__ F3 ldcg3(const float* p) { return f3(__ldcg(p), __ldcg(p + 1), __ldcg(p + 2)); }

// Box of a child node as the fit shader computes it (lbvh_fit_aabb_mesh.comp:94-118).
__device__ __forceinline__ void child_box(const BvhNode* nodes, uint32_t c, F3& lo, F3& hi)
{
    const BvhNode* nd = nodes + c;
    if (__ldcg(&nd->child0) != kInvalid)
    {
        F3 a = ldcg3(nd->a0), b = ldcg3(nd->a1), p = ldcg3(nd->b0), q = ldcg3(nd->b1);
        lo   = vmin(a, p);
        hi   = vmax(b, q);
    }
    else
    {
        F3 a = ldcg3(nd->a0), b = ldcg3(nd->a1), p = ldcg3(nd->b0);
        lo   = vmin(vmin(a, b), p);
        hi   = vmax(vmax(a, b), p);
    }
}

__global__ void __launch_bounds__(256) k_refit(MeshArgs m, const uint32_t* __restrict__ sorted_idx, BvhNode* nodes,
                                               DeviceWords* words)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m.n) return;
    const uint32_t n    = m.n;
    const uint32_t leaf = n - 1 + k;
    const uint32_t prim = sorted_idx[k];
    F3             a, b, c;
    tri_verts(m, prim, a, b, c);
    uint32_t parent = (n == 1) ? kInvalid : __ldcg(&nodes[leaf].parent);
    float4*  dst    = reinterpret_cast<float4*>(nodes + leaf);
    __stcg(dst + 0, make_float4(a.x, a.y, a.z, __uint_as_float(kInvalid)));
    __stcg(dst + 1, make_float4(b.x, b.y, b.z, __uint_as_float(prim)));
    __stcg(dst + 2, make_float4(c.x, c.y, c.z, __uint_as_float(parent)));
    __stcg(dst + 3, make_float4(0.f, 0.f, 0.f, __uint_as_float(0u)));
    uint32_t addr = parent;
    // A Karras tree over 2^30 leaves with 32-bit index tie-breaks is at most
    // 64 levels deep; the bound and the range check only guard against a
    // corrupted tree (they raise NODE_RANGE instead of faulting or spinning).
    for (int level = 0; addr != kInvalid; ++level)
    {
        if (addr >= n - 1 || level > 96)
        {
            atomicOr(&words->error_bits, (uint32_t)RR_CUDA_DEVICE_ERROR_NODE_RANGE);
            return;
        }
        __threadfence();
        if (atomicExch(&nodes[addr].update, 1u) == 0u) return;
        __threadfence();
        BvhNode*       nd = nodes + addr;
        const uint32_t c0 = __ldcg(&nd->child0), c1 = __ldcg(&nd->child1);
        if (c0 >= 2 * n - 1 || c1 >= 2 * n - 1)
        {
            atomicOr(&words->error_bits, (uint32_t)RR_CUDA_DEVICE_ERROR_NODE_RANGE);
            return;
        }
        F3 lo0, hi0, lo1, hi1;
        child_box(nodes, c0, lo0, hi0);
        child_box(nodes, c1, lo1, hi1);
        __stcg(&nd->a0[0], lo0.x);
        __stcg(&nd->a0[1], lo0.y);
        __stcg(&nd->a0[2], lo0.z);
        __stcg(&nd->a1[0], hi0.x);
        __stcg(&nd->a1[1], hi0.y);
        __stcg(&nd->a1[2], hi0.z);
        __stcg(&nd->b0[0], lo1.x);
        __stcg(&nd->b0[1], lo1.y);
        __stcg(&nd->b0[2], lo1.z);
        __stcg(&nd->b1[0], hi1.x);
        __stcg(&nd->b1[1], hi1.y);
        __stcg(&nd->b1[2], hi1.z);
        addr = __ldcg(&nd->parent);
    }
}

__global__ void k_init_trailer(Trailer* t, Trailer v) { *t = v; }
__global__ void k_copy_bounds(const uint32_t* b, Trailer* t)
{
    if (threadIdx.x < 8) t->bounds[threadIdx.x] = (threadIdx.x & 3) == 3 ? 0u : b[threadIdx.x];
}

inline int grid_for(uint64_t n, int block) { return (int)std::max<uint64_t>(1, (n + block - 1) / block); }

}  // namespace

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
    L.total = align_up(off, kAlign);
    // Scratch: bounds | codes | codes_alt | idx | idx_alt | sort | collapse queues.
    const size_t kb = L.morton_bits == 63 ? 8 : 4;
    L.s_bounds      = 0;
    L.s_codes       = kAlign;
    L.s_codes_alt   = align_up(L.s_codes + kb * n, kAlign);
    L.s_idx         = align_up(L.s_codes_alt + kb * n, kAlign);
    L.s_idx_alt     = align_up(L.s_idx + 4ull * n, kAlign);
    L.s_sort        = align_up(L.s_idx_alt + 4ull * n, kAlign);
    L.s_sort_bytes  = radix_sort_scratch_bytes(n, (int)L.morton_bits, &L.sort_tiles, &L.sort_passes);
    L.s_queue       = align_up(L.s_sort + L.s_sort_bytes, kAlign);
    L.s_queue_bytes = (format == RR_CUDA_NODE_FORMAT_WIDE8 && n > 0) ? 2 * kAlign + 2ull * 8ull * n : 0;
    L.s_total       = align_up(L.s_queue + L.s_queue_bytes, kAlign);
    return L;
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

cudaError_t launch_build_mesh(const MeshArgs& m, const GeomLayout& L, uint8_t* scratch, uint8_t* result,
                              DeviceWords* words, int sm_count, cudaStream_t s)
{
    Trailer tr{};
    tr.magic          = kMagic;
    tr.version        = kVersion;
    tr.kind           = kKindGeom;
    tr.node_format    = L.format;
    tr.leaf_count     = L.n;
    tr.node_count     = L.n == 0 ? 0 : 2 * L.n - 1;
    tr.wide_nodes_off = L.wide_off;
    tr.wide_tris_off  = L.tris_off;
    tr.wide_capacity  = L.wide_capacity;
    tr.tri_capacity   = L.tri_capacity;
    tr.morton_bits    = L.morton_bits;
    Trailer* dtr      = reinterpret_cast<Trailer*>(result + L.trailer_off);
    k_init_trailer<<<1, 1, 0, s>>>(dtr, tr);
    if (L.n == 0) return cudaGetLastError();

    uint32_t*   bounds = reinterpret_cast<uint32_t*>(scratch + L.s_bounds);
    cudaError_t e      = cudaMemsetAsync(bounds, 0xff, 16, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(bounds + 4, 0, 16, s);
    if (e != cudaSuccess) return e;
    const int blocks = std::min(grid_for(L.n, 256), sm_count * 8);
    k_mesh_bounds<<<blocks, 256, 0, s>>>(m, bounds);
    k_copy_bounds<<<1, 32, 0, s>>>(bounds, dtr);
    void*     codes     = scratch + L.s_codes;
    void*     codes_alt = scratch + L.s_codes_alt;
    uint32_t* idx       = reinterpret_cast<uint32_t*>(scratch + L.s_idx);
    uint32_t* idx_alt   = reinterpret_cast<uint32_t*>(scratch + L.s_idx_alt);
    if (L.morton_bits == 63)
        k_morton<63><<<blocks, 256, 0, s>>>(m, bounds, codes);
    else
        k_morton<30><<<blocks, 256, 0, s>>>(m, bounds, codes);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    bool alt = false;
    e = launch_radix_sort(codes, codes_alt, idx, idx_alt, L.n, (int)L.morton_bits, scratch + L.s_sort, L.sort_tiles,
                          words, s, &alt);
    if (e != cudaSuccess) return e;
    const void*     sc   = alt ? codes_alt : codes;
    const uint32_t* sidx = alt ? idx_alt : idx;
    BvhNode*        nodes = reinterpret_cast<BvhNode*>(result);
    if ((e = launch_emit(sc, (int)L.morton_bits, L.n, nodes, s)) != cudaSuccess) return e;
    k_refit<<<grid_for(L.n, 256), 256, 0, s>>>(m, sidx, nodes, words);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (L.format == RR_CUDA_NODE_FORMAT_WIDE8) return launch_collapse_wide(L, scratch, result, words, sm_count, s);
    return cudaSuccess;
}

}  // namespace rr
