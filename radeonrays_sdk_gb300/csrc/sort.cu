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
// Every look-back wait is bounded (DeviceWords::lookback_polls, default
// kLookbackPolls).  A block whose wait runs out raises
// RR_CUDA_DEVICE_ERROR_WAIT_TIMEOUT and finds its digit prefix the slow way:
// it counts the digits of every key of the earlier tiles itself.  No hang,
// and the sort stays exact.
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
constexpr uint32_t kLookbackPolls = 1u << 22;

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

// What one onesweep block works on: the key run of one sort (a whole array, or
// one geometry of a fused build) and its tile within that run.
template <class K>
struct SegView
{
    const K*        kin;
    const uint32_t* vin;
    K*              kout;
    uint32_t*       vout;
    uint32_t        n;
    const uint32_t* digit_offsets;  // this pass's exclusive digit offsets
    uint32_t*       lookback;       // this pass's status words, 256 per tile
    uint32_t        tile;           // tile index within the run
};

// One array (the TLAS build).
template <class K>
struct SegSingle
{
    const K*        kin;
    const uint32_t* vin;
    K*              kout;
    uint32_t*       vout;
    uint32_t        n;
    const uint32_t* digit_offsets;
    uint32_t*       lookback;
    __device__ __forceinline__ SegView<K> view(uint32_t t) const
    {
        return SegView<K>{kin, vin, kout, vout, n, digit_offsets, lookback, t};
    }
};

// Every geometry of a fused build; pass p reads the (codes, idx) pair that
// pass p - 1 wrote (even passes read s_codes / s_idx).
template <class K>
struct SegBatch
{
    const BuildItem* items;
    const uint32_t*  tile_prefix;
    uint32_t         count;
    uint32_t         pass;
    uint32_t         passes;
    __device__ __forceinline__ SegView<K> view(uint32_t t) const
    {
        const uint32_t   g  = batch_find(tile_prefix, count, t);
        const BuildItem& it = items[g];
        uint8_t*         sc = it.scratch;
        const bool       odd = (pass & 1u) != 0;
        uint32_t*        ss  = reinterpret_cast<uint32_t*>(sc + it.s_sort);
        SegView<K>       v;
        v.kin           = reinterpret_cast<const K*>(sc + (odd ? it.s_codes_alt : it.s_codes));
        v.kout          = reinterpret_cast<K*>(sc + (odd ? it.s_codes : it.s_codes_alt));
        v.vin           = reinterpret_cast<const uint32_t*>(sc + (odd ? it.s_idx_alt : it.s_idx));
        v.vout          = reinterpret_cast<uint32_t*>(sc + (odd ? it.s_idx : it.s_idx_alt));
        v.n             = it.n;
        v.digit_offsets = ss + pass * kRadix;
        v.lookback      = ss + passes * kRadix + 64 + (size_t)pass * it.tiles * kRadix;
        v.tile          = t - __ldg(tile_prefix + g);
        return v;
    }
};

template <class K, bool kFirst, class Seg>
__global__ void __launch_bounds__(kBlock) k_onesweep(Seg seg, int shift, uint32_t* tile_counter, DeviceWords* words)
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
    // Tiles are claimed in order, so every earlier tile of the same run is
    // already resident or done: the look-back below always makes progress.
    const SegView<K>      sv            = seg.view(s_tile);
    const K* __restrict__ kin           = sv.kin;
    const uint32_t*       vin           = sv.vin;
    K* __restrict__       kout          = sv.kout;
    uint32_t* __restrict__ vout         = sv.vout;
    const uint32_t        n             = sv.n;
    const uint32_t*       digit_offsets = sv.digit_offsets;
    uint32_t*             lookback      = sv.lookback;
    const uint32_t        tile          = sv.tile;
    const uint64_t base = (uint64_t)tile * kTile + (uint64_t)w * 32 * kKpt;
    // Wait limit of the look-back, and the test hook of the bounded wait (a
    // tile that never publishes its counts, so that later tiles run out).
    const uint32_t polls = words->lookback_polls ? words->lookback_polls : kLookbackPolls;
    const bool     held  = words->hold_tile == tile + 1u;

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
        // A held tile (test of the bounded wait) publishes nothing.
        uint32_t* mine = lookback + (uint64_t)tile * kRadix + d;
        if (held)
        {
        }
        else if (tile == 0)
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
        const int d         = tid;
        uint32_t  excl      = 0;
        bool      timed_out = false;
        if (tile > 0)
        {
            int64_t j = (int64_t)tile - 1;
            while (j >= 0 && !timed_out)
            {
                const volatile uint32_t* p = lookback + (uint64_t)j * kRadix + d;
                uint32_t                 v = *p;
                uint32_t                 spins = 0;
                while ((v & ~kValMask) == 0)
                {
                    if (++spins > polls)
                    {
                        timed_out = true;
                        break;
                    }
                    if (spins > 64) __nanosleep(32);
                    v = *p;
                }
                if (timed_out) break;
                excl += v & kValMask;
                if ((v & ~kValMask) == kFlagInc) break;
                --j;
            }
            if (!timed_out && !held) atomicExch(lookback + (uint64_t)tile * kRadix + d, kFlagInc | (excl + tot));
        }
        // A wait that ran out (an earlier tile never published): the block
        // counts the digits of every key before this tile (global_base is a
        // free 256-bin histogram here) and the timed-out digits take their
        // prefix from it.  Exact, only slow.
        if (__syncthreads_or(timed_out))
        {
            global_base[d] = 0;
            __syncthreads();
            const uint64_t before = (uint64_t)tile * kTile;
            for (uint64_t i = (uint64_t)tid; i < before; i += kBlock)
                atomicAdd(&global_base[(uint32_t)(kin[i] >> shift) & 0xffu], 1u);
            __syncthreads();
            if (timed_out)
            {
                excl = global_base[d];
                atomicOr(&words->error_bits, (uint32_t)RR_CUDA_DEVICE_ERROR_WAIT_TIMEOUT);
                if (!held) atomicExch(lookback + (uint64_t)tile * kRadix + d, kFlagInc | (excl + tot));
            }
            __syncthreads();  // every digit read its count before global_base is rewritten
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

// Exclusive digit offsets of every (geometry, pass) of a fused build: block
// g * passes + p scans geometry g's pass-p histogram in place.
__global__ void __launch_bounds__(kRadix) k_scan_hist_batch(const BuildItem* __restrict__ items, uint32_t passes)
{
    __shared__ uint32_t warp_sum[kRadix / 32];
    const uint32_t      g = blockIdx.x / passes, p = blockIdx.x % passes;
    const BuildItem&    it = items[g];
    if (it.n == 0) return;
    uint32_t* h    = reinterpret_cast<uint32_t*>(it.scratch + it.s_sort) + p * kRadix;
    uint32_t  v    = h[threadIdx.x];
    uint32_t  lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t  x    = v;
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

template <class K>
cudaError_t batch_passes(const BatchArgs& b, uint32_t passes, DeviceWords* words, cudaStream_t s)
{
    for (uint32_t p = 0; p < passes; ++p)
    {
        SegBatch<K> seg{b.items, b.tile_prefix, b.count, p, passes};
        if (p == 0)
            k_onesweep<K, true><<<b.total_tiles, kBlock, 0, s>>>(seg, (int)(p * kRadixBits), &b.ctl->sort_tile[p],
                                                                  words);
        else
            k_onesweep<K, false><<<b.total_tiles, kBlock, 0, s>>>(seg, (int)(p * kRadixBits), &b.ctl->sort_tile[p],
                                                                   words);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

template <class K>
cudaError_t single_passes(void* codes, void* codes_alt, uint32_t* idx, uint32_t* idx_alt, uint32_t n,
                          uint32_t passes, uint32_t tiles, const SortScratch& sc, DeviceWords* words, cudaStream_t s)
{
    void*     kin  = codes;
    void*     kout = codes_alt;
    uint32_t* vin  = idx;
    uint32_t* vout = idx_alt;
    for (uint32_t p = 0; p < passes; ++p)
    {
        SegSingle<K> seg{(const K*)kin, vin, (K*)kout, vout, n, sc.hist + p * kRadix,
                         sc.lookback + (size_t)p * tiles * kRadix};
        if (p == 0)
            k_onesweep<K, true><<<tiles, kBlock, 0, s>>>(seg, (int)(p * kRadixBits), sc.counters + p, words);
        else
            k_onesweep<K, false><<<tiles, kBlock, 0, s>>>(seg, (int)(p * kRadixBits), sc.counters + p, words);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
    return cudaSuccess;
}

}  // namespace

uint32_t radix_sort_tile_keys(int key_bits)
{
    return (uint32_t)kBlock * (uint32_t)(key_bits > 32 ? Cfg<uint64_t>::kKpt : Cfg<uint32_t>::kKpt);
}

size_t radix_sort_scratch_bytes(uint32_t n, int key_bits, uint32_t* tiles_out, uint32_t* passes_out)
{
    const uint32_t tile   = radix_sort_tile_keys(key_bits);
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
    e = wide ? single_passes<uint64_t>(codes, codes_alt, idx, idx_alt, n, passes, tiles, sc, words, s)
             : single_passes<uint32_t>(codes, codes_alt, idx, idx_alt, n, passes, tiles, sc, words, s);
    if (e != cudaSuccess) return e;
    *sorted_in_alt = (passes & 1) != 0;
    return cudaSuccess;
}

cudaError_t launch_radix_sort_batch(const BatchArgs& b, DeviceWords* words, cudaStream_t s)
{
    if (b.total_tiles == 0) return cudaSuccess;
    const uint32_t passes = b.morton_bits > 32 ? 8u : 4u;
    k_scan_hist_batch<<<b.count * passes, kRadix, 0, s>>>(b.items, passes);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return b.morton_bits > 32 ? batch_passes<uint64_t>(b, passes, words, s) : batch_passes<uint32_t>(b, passes, words, s);
}

}  // namespace rr
