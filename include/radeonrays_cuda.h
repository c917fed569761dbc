/*
 * radeonrays_cuda.h -- CUDA interop and GB300 extensions of the RadeonRays C API.
 *
 * The reference ships Vulkan and D3D12 interop headers
 * (src/core/include/radeonrays_vlk.h, radeonrays_dx.h).  This header is their
 * CUDA counterpart: it wraps raw device pointers and CUDA streams as RadeonRays
 * handles, keeps the API-neutral buffer helpers (rrAllocateDeviceBuffer,
 * rrMapDevicePtr, rrUnmapDevicePtr) and adds the few controls the GB300 build
 * needs (node format of a build, traversal kernel selection, device error
 * word, traversal counters).
 *
 * All entry points are plain C: pointers, sizes and 32-bit enums only.  CUDA
 * handles (cudaStream_t) are passed as void*.
 */
#ifndef RADEONRAYS_CUDA_H
#define RADEONRAYS_CUDA_H

#include "radeonrays.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- node formats of a geometry build ---------------------------------- */
typedef enum
{
    /* Binary 64-byte nodes in the reference layout only ("plain" path). */
    RR_CUDA_NODE_FORMAT_BINARY = 0,
    /* Binary nodes plus 8-wide nodes with 8-bit conservatively quantised child
     * bounds and a 48-byte triangle array. */
    RR_CUDA_NODE_FORMAT_WIDE8 = 1,
    /* Binary nodes plus 4-wide 128-byte nodes with exact fp32 child boxes
     * whose leaf children are the binary leaf nodes. */
    RR_CUDA_NODE_FORMAT_BVH4 = 2,
    /* The node width rrCudaAutotuneNodeFormat picked for meshes of the same
     * size class (triangle-count octave) on this GPU, from this context or
     * the RR_CUDA_TUNE_CACHE file; BVH4Q8 when none was picked.  Memory
     * requirements with AUTO are sized for any of the wide formats.  A fused build
     * (rrCudaCmdBuildGeometries) takes its largest mesh's width. */
    RR_CUDA_NODE_FORMAT_AUTO = 3,
    /* Binary nodes plus 4-wide 64-byte nodes whose child bounds are 8-bit
     * offsets from a per-node fp32 origin in per-axis power-of-two steps,
     * rounded outward, so every quantised box contains the exact one; leaf
     * children are the binary leaf nodes, and the traversal re-tests each
     * leaf triangle's exact box with the reference's slab arithmetic before
     * its triangle test.  Half the bytes of a BVH4 node per fetch.  The
     * default. */
    RR_CUDA_NODE_FORMAT_BVH4Q8 = 4
} RRCudaNodeFormat;

/* Passed through RRBuildOptions::backend_specific_info.  A null
 * backend_specific_info selects the defaults (BVH4Q8, 30-bit Morton codes). */
typedef struct
{
    uint32_t struct_size;   /* sizeof(RRCudaBuildOptions) */
    uint32_t node_format;   /* RRCudaNodeFormat */
    uint32_t morton_bits;   /* 30 (reference) or 63; 0 = 30 */
    uint32_t reserved;
} RRCudaBuildOptions;

/* ---- traversal kernel selection ---------------------------------------- */
typedef enum
{
    /* The default: on a triangle geometry buffer with 4-wide nodes
     * (RR_CUDA_NODE_FORMAT_BVH4Q8, the default build format, or _BVH4) the
     * 4-wide kernel (RR_CUDA_TRAVERSAL_BVH4); on every other buffer (scenes
     * included) the persistent binary kernel, whose hits are bit-identical
     * to RR_CUDA_TRAVERSAL_BINARY.  rrCudaAutotuneTraversal replaces it with the
     * fastest kernel for a workload. */
    RR_CUDA_TRAVERSAL_AUTO = 0,
    /* One thread per ray, 64-byte binary nodes, reference visit order. */
    RR_CUDA_TRAVERSAL_BINARY = 1,
    /* Persistent warp-scheduled kernel over 8-wide quantised nodes. */
    RR_CUDA_TRAVERSAL_WIDE = 2,
    /* Persistent warp-scheduled kernel over the binary nodes, reference visit
     * order (hits bit-identical to RR_CUDA_TRAVERSAL_BINARY). */
    RR_CUDA_TRAVERSAL_BINARY_PERSISTENT = 3,
    /* Persistent warp-scheduled kernel over the 4-wide nodes of an
     * RR_CUDA_NODE_FORMAT_BVH4 (fp32 boxes) or RR_CUDA_NODE_FORMAT_BVH4Q8
     * (8-bit boxes) buffer, nearest child first. */
    RR_CUDA_TRAVERSAL_BVH4 = 4
} RRCudaTraversal;

/* Ray-triangle test of the traversal kernels. */
typedef enum
{
    /* The reference's test (vlk/kernels/common.h:103-137, Moller-Trumbore,
     * with the reference's slab test and barycentrics): hits bit-identical to
     * the reference's traversal.  The default. */
    RR_CUDA_TRIANGLE_TEST_REFERENCE = 0,
    /* Watertight and accurate, in fp32 (no counterpart in the reference): the
     * watertight hit decision of Woop, Benthin and Wald (JCGT 2013) with the
     * edge functions' signs computed exactly, t and the barycentrics from
     * exact differences and compensated ("double-float") products (t within
     * about 1 ulp of the exact intersection of the fp32 ray and triangle),
     * and a conservative box test (Ize, JCGT 2013) that never culls a box the
     * ray touches.  Supported by RR_CUDA_TRAVERSAL_AUTO,
     * RR_CUDA_TRAVERSAL_BINARY_PERSISTENT and RR_CUDA_TRAVERSAL_BVH4 on
     * triangle geometries (not on scene buffers, AABB lists or the
     * multi-request launch); over RR_CUDA_NODE_FORMAT_BVH4Q8 nodes the
     * 4-wide kernel decodes the 8-bit bounds rounded outward before the
     * conservative box test. */
    RR_CUDA_TRIANGLE_TEST_WATERTIGHT = 1
} RRCudaTriangleTest;

typedef struct
{
    uint32_t struct_size;     /* sizeof(RRCudaTraversalOptions) */
    uint32_t traversal;       /* RRCudaTraversal */
    uint32_t block_size;      /* threads per block, 0 = tuned default */
    uint32_t blocks_per_sm;   /* persistent kernel occupancy, 0 = tuned default */
    uint32_t collect_stats;   /* 1 = count node and triangle fetches */
    uint32_t ray_order;       /* wide kernel: 0 = default, 1 = trace in the given order, 2 = sort rays by
                                 direction octant and origin first (batches of 2^20 rays or more) */
    uint32_t short_stack;     /* RR_CUDA_TRAVERSAL_BVH4 single-level kernel: shared-memory stack entries
                                 per ray, 0 = default (16), else 12..32 (deeper entries spill to scratch) */
    uint32_t triangle_test;   /* RRCudaTriangleTest, 0 = the reference's */
} RRCudaTraversalOptions;

/* Fetch counters accumulated while collect_stats is 1. */
typedef struct
{
    uint64_t rays;
    uint64_t node_fetches;     /* binary nodes (64 B) or wide nodes (80 B) */
    uint64_t triangle_fetches; /* wide-path triangles (48 B); 0 on the binary path */
    uint64_t node_bytes;       /* bytes of one node fetch */
    uint64_t triangle_bytes;   /* bytes of one triangle fetch */
} RRCudaTraversalStats;

/* Bits of the sticky device error word (rrCudaGetDeviceErrors). */
typedef enum
{
    RR_CUDA_DEVICE_ERROR_STACK_OVERFLOW   = 1, /* a ray needed more stack than its scratch slot */
    RR_CUDA_DEVICE_ERROR_BAD_BUFFER       = 2, /* the BVH buffer header did not match */
    RR_CUDA_DEVICE_ERROR_COLLAPSE_DEPTH   = 4, /* wide collapse ran out of levels */
    RR_CUDA_DEVICE_ERROR_NODE_RANGE       = 8, /* a node index left the node array */
    RR_CUDA_DEVICE_ERROR_WAIT_TIMEOUT     = 16 /* a bounded device wait ran out (rrCudaSetWaitLimits says which
                                                  results stay valid) */
} RRCudaDeviceError;

/* Wrap a CUDA device pointer (plus byte offset) as an RRDevicePtr.  The caller
 * keeps ownership of the memory; rrReleaseDevicePtr frees only the handle.
 * Replaces rrGetDevicePtrFromVkBuffer (reference radeonrays_vlk.h:38). */
RR_API RRError rrGetDevicePtrFromCudaPtr(RRContext context, void* cuda_ptr, size_t offset, RRDevicePtr* device_ptr);

/* Device address (base + offset) behind an RRDevicePtr. */
RR_API RRError rrGetCudaPtrFromDevicePtr(RRContext context, RRDevicePtr device_ptr, void** cuda_ptr);

/* Wrap a cudaStream_t: rrCmd* calls on the returned stream enqueue at once on
 * that CUDA stream (no rrSumbitCommandStream needed).  Release it with
 * rrReleaseExternalCommandStream.
 * Replaces rrGetCommandStreamFromVkCommandBuffer (reference radeonrays_vlk.h:64). */
RR_API RRError rrGetCommandStreamFromCudaStream(RRContext context, void* cuda_stream, RRCommandStream* command_stream);

/* Allocate a buffer the host can map (CUDA managed memory).
 * reference radeonrays_vlk.h:77 */
RR_API RRError rrAllocateDeviceBuffer(RRContext context, size_t size, RRDevicePtr* device_ptr);
/* reference radeonrays_vlk.h:86.  Only buffers from rrAllocateDeviceBuffer map. */
RR_API RRError rrMapDevicePtr(RRContext context, RRDevicePtr device_ptr, void** mapping_ptr);
/* reference radeonrays_vlk.h:95 */
RR_API RRError rrUnmapDevicePtr(RRContext context, RRDevicePtr device_ptr, void** mapping_ptr);

/* Select the traversal kernel and its launch shape for later rrCmdIntersect
 * calls on this context (no reference counterpart: the reference has one
 * kernel per variant). */
RR_API RRError rrCudaSetTraversalOptions(RRContext context, const RRCudaTraversalOptions* options);
RR_API RRError rrCudaGetTraversalOptions(RRContext context, RRCudaTraversalOptions* options);

/* Read and clear the context's sticky device error word (RRCudaDeviceError
 * bits).  Synchronises the context's internal stream. */
RR_API RRError rrCudaGetDeviceErrors(RRContext context, uint32_t* error_bits);

/* Read and clear the traversal counters (collect_stats = 1). */
RR_API RRError rrCudaGetTraversalStats(RRContext context, RRCudaTraversalStats* stats);

/* Milliseconds rrWaitEvent polls before it gives up with RR_ERROR_INTERNAL
 * (default 600000).  The reference waits forever (vlk/device.cpp:249-272). */
RR_API RRError rrCudaSetWaitTimeout(RRContext context, uint32_t milliseconds);

/* Limits of the bounded device waits, and hooks that make them run out in
 * tests (no reference counterpart: the reference's waits are host-side and
 * unbounded, vlk/device.cpp:249-272).  Every device-side wait of this build
 * gives up after its limit, raises RR_CUDA_DEVICE_ERROR_WAIT_TIMEOUT in the
 * context's error word (rrCudaGetDeviceErrors) and carries on:
 *   the onesweep look-back of the LBVH sort (a tile waiting for an earlier
 *     tile's digit counts) then counts the earlier tiles' keys itself, so the
 *     sort stays exact;
 *   the streamed host-buffer trace (a warp waiting for its rays' arrival
 *     flag) finishes those rays as misses (inst_id = ~0), and the hits are
 *     invalid.
 * A zero limit selects the default.  The test_* fields never occur in normal
 * use: they withhold a signal so that a test can watch a wait run out. */
typedef struct
{
    uint32_t struct_size;             /* sizeof(RRCudaWaitLimits) */
    uint32_t lookback_polls;          /* look-back polls per earlier tile, 0 = 2^22 */
    uint32_t arrival_polls;           /* arrival-flag polls of about 1 us each, 0 = 2^21 */
    uint32_t test_hold_sort_tile;     /* this sort tile never publishes its counts; RR_INAVLID_VALUE = none */
    uint32_t test_drop_arrival_chunk; /* this chunk's arrival flag is never raised; RR_INAVLID_VALUE = none */
} RRCudaWaitLimits;

/* Set the context's wait limits (and test hooks) for later work; it waits
 * for the work already submitted on the context's internal stream. */
RR_API RRError rrCudaSetWaitLimits(RRContext context, const RRCudaWaitLimits* limits);

/* Pick the fastest traversal for a workload and make it this context's
 * traversal option (no reference counterpart: the reference has one kernel
 * per query variant).  Times every applicable kernel -- plain binary, binary
 * persistent, and by the buffer's format 4-wide (BVH4) or 8-wide with the
 * rays in the given order and, for batches of 2^20 rays or more, with the
 * rays sorted (WIDE8) -- on the caller's rays (their count is the sample
 * size), three runs each on the context's stream, and keeps the fastest.
 * Then the winner's launch shape: 4 and 6 resident blocks per SM against
 * the occupancy maximum (persistent kernels), and for the single-level
 * 4-wide kernel short stacks of 12 and 24 entries against 16; a variant
 * replaces the default only when it is at least 1 % faster.
 * Results are cached per (GPU, buffer kind, node format and size, query,
 * output, ray-count octave) in the context and, when the environment
 * variable RR_CUDA_TUNE_CACHE names a file, in that file across processes.
 * Synchronous; hits and scratch (rrGetTraceMemoryRequirements(ray_count))
 * are overwritten.  `chosen` (optional) receives the selection. */
RR_API RRError rrCudaAutotuneTraversal(RRContext               context,
                                       RRDevicePtr             scene_buffer,
                                       RRIntersectQuery        query,
                                       RRDevicePtr             rays,
                                       uint32_t                ray_count,
                                       RRIntersectQueryOutput  query_output,
                                       RRDevicePtr             hits,
                                       RRDevicePtr             scratch,
                                       RRCudaTraversalOptions* chosen);

/* Pick the node format for a mesh and a ray workload (no reference
 * counterpart: the reference has one binary node format).  Builds the mesh
 * (build_input, with build_options' quality flag) into temporary buffers in
 * the 4-wide fp32 (BVH4), 4-wide 8-bit (BVH4Q8) and 8-wide 8-bit (WIDE8)
 * formats -- the only
 * call of this library that allocates device memory for itself -- runs the
 * traversal autotuner on each with the caller's rays (timed afresh), and
 * keeps the faster.  The choice is remembered for the mesh's size class
 * (triangle-count octave) on this GPU, in the context and in the
 * RR_CUDA_TUNE_CACHE file when set, and later builds with
 * RR_CUDA_NODE_FORMAT_AUTO use it; the context's traversal option becomes
 * the winner's.  Synchronous; `hits` and `scratch` as for
 * rrCudaAutotuneTraversal.  Triangle meshes with the reference's triangle
 * test only. */
RR_API RRError rrCudaAutotuneNodeFormat(RRContext                   context,
                                        const RRGeometryBuildInput* build_input,
                                        const RRBuildOptions*       build_options,
                                        RRIntersectQuery            query,
                                        RRDevicePtr                 rays,
                                        uint32_t                    ray_count,
                                        RRIntersectQueryOutput      query_output,
                                        RRDevicePtr                 hits,
                                        RRDevicePtr                 scratch,
                                        uint32_t*                   node_format);

/* Make a geometry result buffer that was not built on this context -- read
 * back from a file, copied from another process or context -- known to it, so
 * that rrCmdIntersect, rrCmdBuildScene and updates treat it like one built
 * here (no counterpart in the reference, whose buffers never leave their
 * context).  Reads the buffer's 256-byte trailer with a blocking copy and
 * checks magic, version, kind and counts against `triangle_count`; a mismatch
 * returns RR_ERROR_INVALID_PARAMETER (a buffer written by an earlier version
 * of the library, whose 4-wide nodes do not record their binary nodes for
 * updates, is refused: build it again).  Geometry buffers are position-independent
 * (indices, not pointers), so their bytes can be stored and loaded as they
 * are; scene buffers hold BLAS addresses and are rebuilt instead. */
RR_API RRError rrCudaRegisterGeometry(RRContext context, RRDevicePtr geometry_buffer, uint32_t triangle_count);

/* Build `count` geometries in one fused set of launches (no counterpart in
 * the reference API, which records one rrCmdBuildGeometry per geometry,
 * radeonrays.h:322-328).  Geometry i reads build_inputs[i] and uses
 * temporary_buffers[i] and geometry_buffers[i], sized by
 * rrGetGeometryBuildMemoryRequirements for build_inputs[i] alone; all share
 * build_options.  The results are those of count separate rrCmdBuildGeometry
 * calls.  Buffers of different geometries must not overlap
 * (RR_ERROR_INVALID_PARAMETER).  The launch count does not depend on count:
 * every kernel of the build covers all geometries.
 *
 * Consecutive rrCmdBuildGeometry calls recorded into one internal command
 * stream (rrAllocateCommandStream) with the same options and disjoint buffers
 * are fused the same way at submission (environment variable
 * RR_CUDA_FUSE_BUILDS=0 turns that off); on an external stream every call
 * runs at once. */
RR_API RRError rrCudaCmdBuildGeometries(RRContext                   context,
                                        uint32_t                    count,
                                        const RRGeometryBuildInput* build_inputs,
                                        const RRBuildOptions*       build_options,
                                        const RRDevicePtr*          temporary_buffers,
                                        const RRDevicePtr*          geometry_buffers,
                                        RRCommandStream             command_stream);

/* Intersect rays that live in host memory (no counterpart in the reference
 * API, whose rrCmdIntersect takes device buffers, radeonrays.h:391-400).
 * Two plans, with the same hits:
 *   streamed (2^16 rays or more with the persistent binary or the 4-wide
 *     traversal, and host_hits page-locked or registered):
 *     one kernel launch over all rays; the rays are copied in chunks of
 *     `chunk_rays` (rounded down to a power of two; 0 = 2^17) on a context
 *     stream that raises a flag per chunk, the kernel traces each chunk once
 *     its flag is up, and a second context stream copies the hits out in
 *     parts of eight chunks as the kernel's warps publish each part (stream
 *     memory operations: cuStreamWriteValue32 / cuStreamWaitValue32); the
 *     hits of rays still in flight when their part was published are then
 *     written to host_hits by a small kernel after the trace;
 *   chunked (otherwise, inside a stream capture, or RR_CUDA_STREAM_RAYS=0):
 *     chunks of `chunk_rays` (0 = 2^21), each copied in, traced and copied
 *     out on one of three context streams.
 * Either way the host transfers overlap the traversal.
 *   host_rays   RRRay[ray_count] in host memory (page-locked for overlap)
 *   host_hits   RRHit[ray_count] (or uint32_t for INSTANCE_ID) in host memory
 *   rays, hits  device buffers of ray_count records (staging)
 *   scratch     rrGetTraceMemoryRequirements(ray_count) bytes
 * The traversal kernel is the context's (rrCudaSetTraversalOptions); the hits
 * are those of rrCmdIntersect on the same rays.  The work joins back into the
 * command stream's CUDA stream, so an event after it covers the copies. */
RR_API RRError rrCudaCmdIntersectHostBuffers(RRContext              context,
                                             RRDevicePtr            scene_buffer,
                                             RRIntersectQuery       query,
                                             const void*            host_rays,
                                             uint32_t               ray_count,
                                             RRIntersectQueryOutput query_output,
                                             void*                  host_hits,
                                             RRDevicePtr            rays,
                                             RRDevicePtr            hits,
                                             RRDevicePtr            scratch,
                                             uint32_t               chunk_rays,
                                             RRCommandStream        command_stream);

/* ---- many intersection requests in one launch ---------------------------
 * No counterpart in the reference API (one rrCmdIntersect dispatches one
 * query over one buffer, radeonrays.h:391-400).  A serving loop packs the
 * requests it admits into one call: every request's rays are traced by one
 * persistent launch whose lanes take rays from all requests.  When the
 * context's traversal option is RR_CUDA_TRAVERSAL_AUTO or _BVH4 and every
 * request with rays has a triangle geometry with 4-wide nodes of one form
 * (all RR_CUDA_NODE_FORMAT_BVH4Q8, the default, or all _BVH4) or no
 * triangles, each request is traced exactly like rrCmdIntersect with
 * RR_CUDA_TRAVERSAL_BVH4; otherwise
 * exactly like rrCmdIntersect with RR_CUDA_TRAVERSAL_BINARY (the reference's
 * visit order).  Either way a request's hits do not depend on what it is
 * packed with.  The precise triangle test is not applied here. */
typedef struct
{
    RRDevicePtr            geometry;   /* geometry result buffer (rrCmdBuildGeometry); scenes are not accepted */
    RRIntersectQuery       query;
    RRIntersectQueryOutput output;
    RRDevicePtr            rays;       /* RRRay[ray_count] */
    uint32_t               ray_count;
    RRDevicePtr            hits;       /* RRHit[ray_count], or uint32_t[ray_count] for INSTANCE_ID output */
} RRCudaIntersectRequest;

/* Scratch bytes of rrCudaCmdIntersectBatch for `request_count` requests with
 * `total_ray_count` rays in all. */
RR_API RRError rrCudaGetIntersectBatchMemoryRequirements(RRContext context,
                                                         uint32_t  request_count,
                                                         uint32_t  total_ray_count,
                                                         size_t*   scratch_size);

/* Record (or, on an external stream, enqueue) one launch over all requests.
 * The total ray count must be below 2^32.  A scene buffer as `geometry`
 * returns RR_ERROR_NOT_IMPLEMENTED. */
RR_API RRError rrCudaCmdIntersectBatch(RRContext                     context,
                                       uint32_t                      request_count,
                                       const RRCudaIntersectRequest* requests,
                                       RRDevicePtr                   scratch,
                                       RRCommandStream               command_stream);

/* The same launch for requests whose rays and hits live in host memory (page-
 * locked for asynchronous copies): every request's rays are copied into
 * `rays` (a device buffer of the total ray count), the hit buffer `hits`
 * (16 bytes per ray of the total) is filled with 0xFF, one persistent launch
 * traces all requests, and every request's hits are copied back to its host
 * buffer (16 or 4 bytes per ray), all on the command stream in that order.
 * Record fields a miss leaves untouched read back as 0xFFFFFFFF.  One call per
 * launch replaces one copy and one handle per request in a serving loop. */
typedef struct
{
    RRDevicePtr            geometry;
    RRIntersectQuery       query;
    RRIntersectQueryOutput output;
    const void*            host_rays;  /* RRRay[ray_count] */
    uint32_t               ray_count;
    void*                  host_hits;  /* RRHit[ray_count] or uint32_t[ray_count] */
} RRCudaHostIntersectRequest;

RR_API RRError rrCudaCmdIntersectBatchHost(RRContext                         context,
                                           uint32_t                          request_count,
                                           const RRCudaHostIntersectRequest* requests,
                                           RRDevicePtr                       rays,
                                           RRDevicePtr                       hits,
                                           RRDevicePtr                       scratch,
                                           RRCommandStream                   command_stream);

/* Intersect without allocating anything and without a caller scratch buffer.
 * No counterpart in the reference API.
 *
 * For callers that cannot call cudaMalloc at the point where they trace rays:
 * a serving loop with a hard latency budget (cudaMalloc may block and
 * synchronise the device), or a host whose device memory is owned by another
 * allocator or pool (an extra cudaMalloc would fail or break its accounting).
 * The caller passes its own BVH, rays and hit buffer (device pointers) and a
 * cudaStream_t as void* (0 = default stream); no RRContext is needed.
 *
 * Runs the plain binary-node traversal (the rrCmdIntersect plain kernel, same
 * hits) over `geometry`, a geometry result buffer of a TRIANGLE mesh written
 * by rrCmdBuildGeometry (binary nodes at offset 0; AABB-list geometries and
 * scene buffers are not supported).  `triangle_count` is the mesh's triangle
 * count: node indices outside its 2 * triangle_count - 1 binary nodes stop the
 * ray and raise RR_CUDA_DEVICE_ERROR_NODE_RANGE; 0 is an empty geometry, where
 * every ray misses.  Its traversal scratch is a fixed device array of about
 * 32 MiB inside librr.so, which every GPU that loads the library keeps until
 * the process exits; a call takes at most 131072 rays (more returns
 * RR_ERROR_INVALID_PARAMETER).  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress): make that first call before
 * any stream capture.  All calls share the one array, so calls that overlap on
 * the GPU race with each other.
 *
 * Device-side errors (RRCudaDeviceError bits: a stack overflow, a node index
 * out of range) mean the hits of the call are invalid although it returned
 * RR_SUCCESS; read them with rrCudaGetNoAllocDeviceErrors. */
RR_API RRError rrCudaIntersectNoAlloc(const void*            geometry,
                                      uint32_t               triangle_count,
                                      RRIntersectQuery       query,
                                      const void*            rays,
                                      uint32_t               ray_count,
                                      RRIntersectQueryOutput query_output,
                                      void*                  hits,
                                      void*                  cuda_stream);

/* Read and clear the device error word of rrCudaIntersectNoAlloc on the
 * current device (RRCudaDeviceError bits; no counterpart in the reference
 * API).  The word lives in the same fixed array: it is zero when the library
 * loads, every rrCudaIntersectNoAlloc call ORs its errors into it, and this
 * call reads it after the work already enqueued on `cuda_stream` (synchronises
 * that stream), then clears it.  Like the calls it reports on, it shares the
 * one word: a call that overlaps on the GPU with another stream's calls sees
 * their bits too.  Allocates nothing. */
RR_API RRError rrCudaGetNoAllocDeviceErrors(void* cuda_stream, uint32_t* error_bits);

#ifdef __cplusplus
}
#endif

#endif /* RADEONRAYS_CUDA_H */
