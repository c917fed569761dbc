// trace_wide.cuh -- traversal of one ray through an 8-wide BVH (device code
// shared by the single-level kernel, trace_wide.cu, and the two-level kernel,
// scene.cu).  Node format and conservativeness argument: wide.cu.
#pragma once
#include "trace_common.cuh"

namespace rr
{
constexpr int kWideShortStack = 16;

struct WideEntry
{
    uint32_t node;
    float    t0;
};

__device__ __forceinline__ uint32_t ord_f(float f)
{
    uint32_t u = __float_as_uint(f);
    return u ^ ((1u + ~(u >> 31)) | 0x80000000u);
}
__device__ __forceinline__ float unord_f(uint32_t v) { return __uint_as_float(v ^ (((v >> 31) - 1u) | 0x80000000u)); }
__device__ __forceinline__ float byte_f(uint32_t w, int byte) { return (float)((w >> (8 * byte)) & 0xffu); }

__device__ __forceinline__ void cmpx(unsigned long long& a, unsigned long long& b)
{
    const unsigned long long lo = a < b ? a : b, hi = a < b ? b : a;
    a = lo;
    b = hi;
}

// Per-thread traversal stack: a short stack in shared memory that spills
// kWideShortStack entries at a time to a per-thread global region.
struct WideStack
{
    WideEntry* s;        // kWideShortStack entries (shared)
    WideEntry* g;        // gcap entries (global scratch)
    uint32_t   gcap;
};

// Traverse the wide BVH (root = node 0) for `ray`.  Closest hit: shrinks `ct`
// and sets `best` (triangle index) for every accepted triangle.  Any hit
// (kAny): returns true at the first accepted triangle.  Returns false when the
// traversal completes.
template <bool kAny>
__device__ __forceinline__ bool wide_traverse(const Ray& ray, const F3 inv, const F3 oxi, const WideNode* __restrict__ wn,
                                              const WideTri* __restrict__ wt, float& ct, uint32_t& best,
                                              const WideStack& st, DeviceWords* words, uint32_t& nfetch,
                                              uint32_t& tfetch)
{
    int      sp   = 0;
    uint32_t gsp  = 0;
    uint32_t node = 0;
    for (;;)
    {
        if (node == kInvalid)
        {
            for (;;)
            {
                if (sp == 0)
                {
                    if (gsp == 0) return false;
                    gsp -= kWideShortStack;
                    for (int i = 0; i < kWideShortStack; ++i) st.s[i] = st.g[gsp + i];
                    sp = kWideShortStack;
                }
                const WideEntry e = st.s[--sp];
                if (e.t0 <= ct)
                {
                    node = e.node;
                    break;
                }
            }
        }

        const uint4* np = reinterpret_cast<const uint4*>(wn + node);
        const uint4  w0 = __ldg(np), w1 = __ldg(np + 1), w2 = __ldg(np + 2), w3 = __ldg(np + 3), w4 = __ldg(np + 4);
        ++nfetch;
        const F3       p  = f3(__uint_as_float(w0.x), __uint_as_float(w0.y), __uint_as_float(w0.z));
        const float    sx = __uint_as_float((w0.w & 0xffu) << 23);
        const float    sy = __uint_as_float(((w0.w >> 8) & 0xffu) << 23);
        const float    sz = __uint_as_float(((w0.w >> 16) & 0xffu) << 23);
        const uint32_t imask      = w0.w >> 24;
        const uint32_t child_base = w1.x, tri_base = w1.y;
        node                      = kInvalid;

        unsigned long long key[8];
#pragma unroll
        for (int k = 0; k < 8; ++k)
        {
            const uint32_t meta = ((k < 4 ? w1.z : w1.w) >> (8 * (k & 3))) & 0xffu;
            key[k]              = ~0ull;
            if (meta == 0) continue;
            const uint32_t qlx = k < 4 ? w2.x : w2.y, qly = k < 4 ? w2.z : w2.w, qlz = k < 4 ? w3.x : w3.y;
            const uint32_t qhx = k < 4 ? w3.z : w3.w, qhy = k < 4 ? w4.x : w4.y, qhz = k < 4 ? w4.z : w4.w;
            const int      b   = k & 3;
            const F3 lo = f3(fmaf(byte_f(qlx, b), sx, p.x), fmaf(byte_f(qly, b), sy, p.y), fmaf(byte_f(qlz, b), sz, p.z));
            const F3 hi = f3(fmaf(byte_f(qhx, b), sx, p.x), fmaf(byte_f(qhy, b), sy, p.y), fmaf(byte_f(qhz, b), sz, p.z));
            float    t0, t1;
            isect_box(lo, hi, inv, oxi, ct, ray.tmin, t0, t1);
            if (t0 > t1) continue;
            if (imask & (1u << k))
                key[k] = ((unsigned long long)ord_f(t0) << 32) | (child_base + (meta & 0x7fu));
            else
            {
                const uint32_t cnt = meta >> 5, off = meta & 31u;
                for (uint32_t j = 0; j < cnt; ++j)
                {
                    const uint32_t ti = tri_base + off + j;
                    const float4*  tp = reinterpret_cast<const float4*>(wt + ti);
                    const float4   A = __ldg(tp), B = __ldg(tp + 1), C = __ldg(tp + 2);
                    ++tfetch;
                    const float t = isect_tri(ray, f3(A.x, A.y, A.z), f3(B.x, B.y, B.z), f3(C.x, C.y, C.z), ct);
                    if (t < ct)
                    {
                        ct   = t;
                        best = ti;
                        if (kAny) return true;
                    }
                }
            }
        }

        // Nearest internal child next; the others pushed farthest-first.
        cmpx(key[0], key[1]); cmpx(key[2], key[3]); cmpx(key[4], key[5]); cmpx(key[6], key[7]);
        cmpx(key[0], key[2]); cmpx(key[1], key[3]); cmpx(key[4], key[6]); cmpx(key[5], key[7]);
        cmpx(key[1], key[2]); cmpx(key[5], key[6]); cmpx(key[0], key[4]); cmpx(key[3], key[7]);
        cmpx(key[1], key[5]); cmpx(key[2], key[6]);
        cmpx(key[1], key[4]); cmpx(key[3], key[6]);
        cmpx(key[2], key[4]); cmpx(key[3], key[5]);
        cmpx(key[3], key[4]);
#pragma unroll
        for (int k = 7; k >= 1; --k)
        {
            if (key[k] == ~0ull) continue;
            if (sp == kWideShortStack)
            {
                if (gsp + kWideShortStack > st.gcap)
                {
                    atomicOr(&words->error_bits, (uint32_t)RR_CUDA_DEVICE_ERROR_STACK_OVERFLOW);
                    continue;
                }
                for (int i = 0; i < kWideShortStack; ++i) st.g[gsp + i] = st.s[i];
                gsp += kWideShortStack;
                sp = 0;
            }
            st.s[sp++] = WideEntry{(uint32_t)key[k], unord_f((uint32_t)(key[k] >> 32))};
        }
        if (key[0] != ~0ull) node = (uint32_t)key[0];
    }
}

// Persistent-grid sizing shared by the wide kernels: threads never exceed the
// 32-ray batches; every thread gets an equal share of the scratch for spills.
struct WideLaunch
{
    int      blocks;
    int      block;
    uint32_t gcap;
};

}  // namespace rr
