// noalloc.cu -- rrCudaIntersectNoAlloc: the plain (binary-node) traversal
// kernel run with its scratch in a fixed device array owned by librr.so, so
// the call itself allocates nothing.
//
// Who needs it: callers that must not call cudaMalloc at the point where
// they trace rays -- for example a serving loop with a hard latency budget
// (cudaMalloc can block and synchronise the device) or a host application
// whose device memory is entirely owned by another allocator or pool (an
// extra cudaMalloc would fail or break that pool's accounting).  They still
// pass their own rays, BVH and hit buffers; only the traversal scratch (the
// per-ray spill stack and the device error word) comes from here.
//
// The device error word of these calls lives in the array too (no context
// holds it): rrCudaGetNoAllocDeviceErrors reads and clears it.
//
// The array is a file-scope static __device__ variable: every GPU that loads
// librr.so holds kNoAllocScratchBytes for it until the process exits.  Host
// code may not use the array's name as a device address; the first call on
// each device looks up its device address with cudaGetSymbolAddress (with
// that device current) and caches it, so that first call should come before
// any stream capture.  Every call shares the one array: calls that overlap on
// the GPU (different streams without ordering) race on it.
#include <cstdio>
#include <mutex>

#include "rr_internal.h"

namespace rr
{
namespace
{
// Traversal scratch for up to kNoAllocMaxRays rays (256 bytes per ray, the
// reference's figure) plus the error/counter words in front of it.
constexpr uint32_t kNoAllocMaxRays     = 131072;
constexpr size_t   kNoAllocWordsBytes  = 256;
constexpr size_t   kNoAllocScratchBytes = kNoAllocWordsBytes + 256 + (size_t)kNoAllocMaxRays * 256;

static __device__ __align__(256) uint8_t g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex    g_setup_mu;
uint8_t*      g_setup_ptr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (set-up once per
// device; the device must be current).
cudaError_t scratch_address(uint8_t** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_setup_ptr[dev])
    {
        void* p = nullptr;
        e       = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_setup_ptr[dev] = reinterpret_cast<uint8_t*>(p);
    }
    *out = g_setup_ptr[dev];
    return cudaSuccess;
}
}  // namespace
}  // namespace rr

using namespace rr;

extern "C" RR_API RRError rrCudaIntersectNoAlloc(const void* geometry, uint32_t triangle_count, RRIntersectQuery query,
                                                 const void* rays, uint32_t ray_count,
                                                 RRIntersectQueryOutput query_output, void* hits, void* cuda_stream)
{
    if (!geometry || !rays || !hits) return RR_ERROR_INVALID_PARAMETER;
    if (query != RR_INTERSECT_QUERY_CLOSEST && query != RR_INTERSECT_QUERY_ANY) return RR_ERROR_INVALID_PARAMETER;
    if (query_output != RR_INTERSECT_QUERY_OUTPUT_FULL_HIT && query_output != RR_INTERSECT_QUERY_OUTPUT_INSTANCE_ID)
        return RR_ERROR_INVALID_PARAMETER;
    if (triangle_count > 0x7fffffffu) return RR_ERROR_INVALID_PARAMETER;  // 2N - 1 binary nodes must fit 32 bits
    if (ray_count > kNoAllocMaxRays)
    {
        std::fprintf(stderr,
                     "[rr error] rrCudaIntersectNoAlloc: %u rays exceed the fixed scratch capacity of %u rays; "
                     "split the batch or use rrCmdIntersect with your own scratch buffer\n",
                     ray_count, kNoAllocMaxRays);
        return RR_ERROR_INVALID_PARAMETER;
    }
    if (ray_count == 0) return RR_SUCCESS;
    uint8_t*    base = nullptr;
    cudaError_t e    = scratch_address(&base);
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        return RR_ERROR_INTERNAL;
    }
    cudaStream_t s = reinterpret_cast<cudaStream_t>(cuda_stream);
    // The error word is sticky (zero when the library loads, read and cleared
    // by rrCudaGetNoAllocDeviceErrors); the plain kernel keeps no other state
    // between calls: its spill stacks are written before they are read.
    TraceArgs a{};
    a.bvh           = reinterpret_cast<const uint8_t*>(geometry);
    a.rays          = reinterpret_cast<const uint8_t*>(rays);
    a.ray_count     = ray_count;
    a.hits          = hits;
    a.scratch       = base + kNoAllocWordsBytes;
    a.scratch_bytes = kNoAllocScratchBytes - kNoAllocWordsBytes;
    a.query         = query;
    a.output        = query_output;
    a.empty         = triangle_count == 0;
    a.node_limit    = triangle_count == 0 ? 0u : 2u * triangle_count - 1u;
    a.words         = reinterpret_cast<DeviceWords*>(base);
    static_assert(sizeof(DeviceWords) <= kNoAllocWordsBytes, "words fit in front of the scratch");
    e = launch_trace_binary(a, s);
    if (e != cudaSuccess) return RR_ERROR_INTERNAL;
    return RR_SUCCESS;
}

extern "C" RR_API RRError rrCudaGetNoAllocDeviceErrors(void* cuda_stream, uint32_t* error_bits)
{
    if (!error_bits) return RR_ERROR_INVALID_PARAMETER;
    uint8_t*    base = nullptr;
    cudaError_t e    = scratch_address(&base);
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        return RR_ERROR_INTERNAL;
    }
    cudaStream_t s    = reinterpret_cast<cudaStream_t>(cuda_stream);
    uint32_t*    word = &reinterpret_cast<DeviceWords*>(base)->error_bits;
    uint32_t     v    = 0;
    // Ordered after the calls on this stream; the clear is ordered after the read.
    if (cudaMemcpyAsync(&v, word, sizeof(v), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemsetAsync(word, 0, sizeof(v), s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess)
    {
        cudaGetLastError();
        return RR_ERROR_INTERNAL;
    }
    *error_bits = v;
    return RR_SUCCESS;
}
