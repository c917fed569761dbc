// sort.cu -- stable LSD key/value radix sort for the LBVH build (onesweep).
//
// Replaces the reference's 4-bit multi-pass sort (vlk/radix_sort.cpp:157-338,
// kernels radix_sort_group_histograms.comp + scan_exclusive_add*.comp +
// radix_sort_scatter_keys.comp).  The contract kept is the result: a stable
// permutation of (key, original index) pairs ordered by key.
//
// Scheme (Adinets & Merrill, "Onesweep", 2022):
//   1. one read of all keys builds the 256-bin digit histogram of every pass;
//   2. the histograms are turned into per-pass exclusive digit offsets;
//   3. one kernel per 8-bit digit pass: each block takes a tile id from an
//      atomic counter, ranks its keys stably with warp match/ballot
//      primitives, publishes its per-digit counts, looks back over earlier
//      tiles (decoupled look-back) for its per-digit prefix, and scatters
//      through shared memory.
// Every look-back wait is bounded; on exhaustion the kernel raises
// RR_CUDA_DEVICE_ERROR_WAIT_TIMEOUT and carries on (no hang, result invalid).
#include <algorithm>
#include <utility>

#include "rr_internal.h"

namespace rr
{
namespace
{
constexpr int      kRadixBits = 8;
constexpr int      kRadix     = 256;
constexpr int      kBlock     = 256;
constexpr int      kWarps     = kBlock / 32;
constexpr uint32_t kFlagAgg   = 1u << 30;
constexpr uint32_t kFlagInc   = 2u << 30;
constexpr uint32_t kValMask   = (1u << 30) - 1;
constexpr uint32_t kSpinLimit = 1u << 22;

template <class K>
struct Cfg;
template <>
struct Cfg<uint32_t>
{
    static constexpr int kKpt = 16;
};
template <>
struct Cfg<uint64_t>
{
    static constexpr int kKpt = 8;
};

struct SortScratch
{
    uint32_t* hist;      // passes * 256: counts, then exclusive offsets
    uint32_t* counters;  // passes tile counters
    uint32_t* lookback;  // passes * tiles * 256 status words
};

inline SortScratch carve(uint8_t* base, uint32_t passes, uint32_t tiles)
{
    SortScratch s;
    s.hist     = reinterpret_cast<uint32_t*>(base);
    s.counters = s.hist + passes * kRadix;
    s.lookback = s.counters + 64;
    (void)tiles;
    return s;
}

template <class K>
__global__ void __launch_bounds__(kBlock) k_global_hist(const K* __restrict__ keys, uint32_t n, int passes,
                                                         uint32_t* __restrict__ hist)
{
    __shared__ uint32_t h[8][kRadix];
    for (int i = threadIdx.x; i < passes * kRadix; i += blockDim.x) (&h[0][0])[i] = 0;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        K k = keys[i];
        for (int p = 0; p < passes; ++p) atomicAdd(&h[p][(k >> (p * kRadixBits)) & 0xff], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * kRadix; i += blockDim.x)
    {
        uint32_t v = (&h[0][0])[i];
        if (v) atomicAdd(&hist[i], v);
    }
}

// One block per pass: exclusive scan of the 256 digit counts.
__global__ void __launch_bounds__(kRadix) k_scan_hist(uint32_t* hist)
{
    __shared__ uint32_t warp_sum[kRadix / 32];
    uint32_t*           h    = hist + blockIdx.x * kRadix;
    uint32_t            v    = h[threadIdx.x];
    uint32_t            lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t            x    = v;
    for (int o = 1; o < 32; o <<= 1)
    {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) warp_sum[w] = x;
    __syncthreads();
    uint32_t add = 0;
    for (uint32_t k = 0; k < w; ++k) add += warp_sum[k];
    h[threadIdx.x] = x - v + add;
}

template <class K, bool kFirst>
__global__ void __launch_bounds__(kBlock) k_onesweep(const K* __restrict__ kin,
                                                     const uint32_t* __restrict__ vin,
                                                     K* __restrict__ kout,
                                                     uint32_t* __restrict__ vout,
                                                     uint32_t n,
                                                     int      shift,
                                                     const uint32_t* __restrict__ digit_offsets,
                                                     uint32_t* tile_counter,
                                                     uint32_t* lookback,
                                                     DeviceWords* words)
{
    constexpr int kKpt  = Cfg<K>::kKpt;
    constexpr int kTile = kBlock * kKpt;
    __shared__ uint32_t s_tile;
    __shared__ uint32_t warp_hist[kWarps][kRadix];  // counts -> exclusive offsets across warps
    __shared__ uint32_t tile_start[kRadix];         // local start of each digit in the tile
    __shared__ uint32_t global_base[kRadix];        // global start of this tile's run of each digit
    __shared__ uint32_t warp_tot[kWarps];
    __shared__ __align__(16) K        s_keys[kTile];
    __shared__ uint32_t s_vals[kTile];

    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(tile_counter, 1u);
    for (int i = lane; i < kRadix; i += 32) warp_hist[w][i] = 0;
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint64_t base = (uint64_t)tile * kTile + (uint64_t)w * 32 * kKpt;

    K        key[kKpt];
    uint32_t rank[kKpt];
    uint32_t dig[kKpt];
#pragma unroll
    for (int r = 0; r < kKpt; ++r)
    {
        uint64_t i = base + r * 32 + lane;
        key[r]     = i < n ? kin[i] : K(0);
    }
    const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < kKpt; ++r)
    {
        uint64_t i     = base + r * 32 + lane;
        bool     valid = i < n;
        uint32_t d     = (uint32_t)(key[r] >> shift) & 0xffu;
        dig[r]         = d;
        uint32_t peers = __match_any_sync(0xffffffffu, valid ? d : 0x100u);
        uint32_t before = warp_hist[w][d];
        __syncwarp();
        if (valid)
        {
            rank[r] = before + __popc(peers & lt);
            if ((peers & lt) == 0) warp_hist[w][d] = before + __popc(peers);
        }
        __syncwarp();
    }
    __syncthreads();

    // Per-digit totals and exclusive offsets across warps (thread = digit).
    uint32_t tot = 0;
    {
        const int d = tid;
#pragma unroll
        for (int k = 0; k < kWarps; ++k)
        {
            uint32_t c      = warp_hist[k][d];
            warp_hist[k][d] = tot;
            tot += c;
        }
        // Publish this tile's count (tile 0 publishes its inclusive prefix).
        uint32_t* mine = lookback + (uint64_t)tile * kRadix + d;
        if (tile == 0)
            atomicExch(mine, kFlagInc | tot);
        else
            atomicExch(mine, kFlagAgg | tot);
    }
    // Local exclusive scan of the tile's digit totals.
    {
        uint32_t x = tot;
        for (int o = 1; o < 32; o <<= 1)
        {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_tot[w] = x;
        __syncthreads();
        uint32_t add = 0;
        for (int k = 0; k < w; ++k) add += warp_tot[k];
        tile_start[tid] = x - tot + add;
    }
    // Decoupled look-back for this digit.
    {
        const int d    = tid;
        uint32_t  excl = 0;
        if (tile > 0)
        {
            int64_t j = (int64_t)tile - 1;
            while (j >= 0)
            {
                const volatile uint32_t* p = lookback + (uint64_t)j * kRadix + d;
                uint32_t                 v = *p;
                uint32_t                 spins = 0;
                while ((v & ~kValMask) == 0)
                {
                    if (++spins > kSpinLimit)
                    {
                        atomicOr(&words->error_bits, (uint32_t)RR_CUDA_DEVICE_ERROR_WAIT_TIMEOUT);
                        v = kFlagInc;
                        break;
                    }
                    if (spins > 64) __nanosleep(32);
                    v = *p;
                }
                excl += v & kValMask;
                if ((v & ~kValMask) == kFlagInc) break;
                --j;
            }
            atomicExch(lookback + (uint64_t)tile * kRadix + d, kFlagInc | (excl + tot));
        }
        global_base[d] = digit_offsets[d] + excl;
    }
    __syncthreads();

    // Local reorder through shared memory, then coalesced global writes.
#pragma unroll
    for (int r = 0; r < kKpt; ++r)
    {
        uint64_t i = base + r * 32 + lane;
        if (i < n)
        {
            uint32_t lp = tile_start[dig[r]] + warp_hist[w][dig[r]] + rank[r];
            s_keys[lp]  = key[r];
            s_vals[lp]  = kFirst ? (uint32_t)i : vin[i];
        }
    }
    __syncthreads();
    const uint64_t left   = (uint64_t)n - (uint64_t)tile * kTile;
    const uint32_t tile_n = (uint32_t)(left < (uint64_t)kTile ? left : (uint64_t)kTile);
    for (uint32_t lp = tid; lp < tile_n; lp += kBlock)
    {
        K        k = s_keys[lp];
        uint32_t d = (uint32_t)(k >> shift) & 0xffu;
        uint32_t g = global_base[d] + (lp - tile_start[d]);
        kout[g]    = k;
        vout[g]    = s_vals[lp];
    }
}

__global__ void k_iota(uint32_t* v, uint32_t n)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = i;
}

}  // namespace

size_t radix_sort_scratch_bytes(uint32_t n, int key_bits, uint32_t* tiles_out, uint32_t* passes_out)
{
    const int      kpt    = key_bits > 32 ? Cfg<uint64_t>::kKpt : Cfg<uint32_t>::kKpt;
    const uint32_t tile   = kBlock * kpt;
    const uint32_t tiles  = n == 0 ? 0 : (n + tile - 1) / tile;
    const uint32_t passes = (uint32_t)((key_bits + kRadixBits - 1) / kRadixBits);
    if (tiles_out) *tiles_out = tiles;
    if (passes_out) *passes_out = passes;
    return align_up(((size_t)passes * kRadix + 64 + (size_t)passes * tiles * kRadix) * sizeof(uint32_t), kAlign);
}

cudaError_t launch_radix_sort(void* codes, void* codes_alt, uint32_t* idx, uint32_t* idx_alt, uint32_t n,
                              int key_bits, uint8_t* sort_scratch, uint32_t tiles, DeviceWords* words,
                              cudaStream_t s, bool* sorted_in_alt)
{
    *sorted_in_alt = false;
    if (n == 0) return cudaSuccess;
    if (n == 1)
    {
        k_iota<<<1, 32, 0, s>>>(idx, 1);
        return cudaGetLastError();
    }
    uint32_t    tiles_chk = 0, passes = 0;
    size_t      bytes     = radix_sort_scratch_bytes(n, key_bits, &tiles_chk, &passes);
    SortScratch sc        = carve(sort_scratch, passes, tiles);
    cudaError_t e         = cudaMemsetAsync(sort_scratch, 0, bytes, s);
    if (e != cudaSuccess) return e;
    const bool wide = key_bits > 32;
    int        hist_blocks = (int)std::min<uint32_t>(1024u, (n + kBlock * 8 - 1) / (kBlock * 8));
    if (wide)
        k_global_hist<uint64_t><<<hist_blocks, kBlock, 0, s>>>((const uint64_t*)codes, n, (int)passes, sc.hist);
    else
        k_global_hist<uint32_t><<<hist_blocks, kBlock, 0, s>>>((const uint32_t*)codes, n, (int)passes, sc.hist);
    k_scan_hist<<<passes, kRadix, 0, s>>>(sc.hist);
    void*     kin = codes;
    void*     kout = codes_alt;
    uint32_t* vin = idx;
    uint32_t* vout = idx_alt;
    for (uint32_t p = 0; p < passes; ++p)
    {
        uint32_t* lb = sc.lookback + (size_t)p * tiles * kRadix;
        if (wide)
        {
            if (p == 0)
                k_onesweep<uint64_t, true><<<tiles, kBlock, 0, s>>>((const uint64_t*)kin, vin, (uint64_t*)kout, vout,
                                                                     n, p * kRadixBits, sc.hist + p * kRadix,
                                                                     sc.counters + p, lb, words);
            else
                k_onesweep<uint64_t, false><<<tiles, kBlock, 0, s>>>((const uint64_t*)kin, vin, (uint64_t*)kout,
                                                                      vout, n, p * kRadixBits, sc.hist + p * kRadix,
                                                                      sc.counters + p, lb, words);
        }
        else
        {
            if (p == 0)
                k_onesweep<uint32_t, true><<<tiles, kBlock, 0, s>>>((const uint32_t*)kin, vin, (uint32_t*)kout, vout,
                                                                     n, p * kRadixBits, sc.hist + p * kRadix,
                                                                     sc.counters + p, lb, words);
            else
                k_onesweep<uint32_t, false><<<tiles, kBlock, 0, s>>>((const uint32_t*)kin, vin, (uint32_t*)kout,
                                                                      vout, n, p * kRadixBits, sc.hist + p * kRadix,
                                                                      sc.counters + p, lb, words);
        }
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
    *sorted_in_alt = (passes & 1) != 0;
    return cudaSuccess;
}

}  // namespace rr
