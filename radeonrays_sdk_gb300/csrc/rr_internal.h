// rr_internal.h -- data layouts and kernel entry points shared by the host
// runtime (api.cu) and the CUDA kernels of the GB300 RadeonRays build.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "../../include/radeonrays.h"
#include "../../include/radeonrays_cuda.h"

namespace rr
{
constexpr uint32_t kInvalid     = 0xffffffffu;  // vlk/kernels/common.h:20 RR_INVALID_ADDR
constexpr uint32_t kSentinel    = 0xfffffffeu;  // vlk/kernels/isect_2l.comp:28
constexpr uint32_t kMagic       = 0x52524742u;  // "RRGB": trailer tag of a result buffer
constexpr uint32_t kVersion     = 2;  // 2: 4-wide nodes record their binary node (the update reads it)
constexpr uint32_t kKindGeom    = 1;
constexpr uint32_t kKindScene   = 2;
constexpr size_t   kAlign       = 256;
constexpr uint32_t kMaxInstancesRef = 2048;  // vlk/intersector.cpp:38 (accepted; larger counts also work)

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Primitive kinds of a geometry build.  An AABB-list leaf stores its box as
// the three vertex slots (min, max, max): bounds, Morton centre and refit then
// treat it exactly like a triangle with those vertices.
constexpr uint32_t kPrimTriangles = 0;
constexpr uint32_t kPrimAabbs     = 1;

// 64-byte binary node in the reference layout (vlk/kernels/bvh2.h:25-35).
// Internal nodes [0, N-2], leaves [N-1, 2N-2]; a leaf has child0 = invalid,
// child1 = primitive id and its triangle's vertices in the first three vec3.
struct __align__(16) BvhNode
{
    float    a0[3];  // aabb0_min_or_v0
    uint32_t child0;
    float    a1[3];  // aabb0_max_or_v1
    uint32_t child1;
    float    b0[3];  // aabb1_min_or_v2
    uint32_t parent;
    float    b1[3];  // aabb1_max_or_v3
    uint32_t update;
};
static_assert(sizeof(BvhNode) == 64, "node layout");

// 8-wide node with 8-bit child bounds (80 bytes, five 16-byte words).
// Child box of slot i on axis a: [fma(qlo, 2^e, p), fma(qhi, 2^e, p)], rounded
// outward at build time so it contains the exact child box.
struct __align__(16) WideNode
{
    float    p[3];       // quantisation origin
    uint8_t  e[3];       // biased exponents: scale = 2^(e - 127)
    uint8_t  imask;      // bit i: slot i is an internal child
    uint32_t child_base; // index of the first internal child (children are contiguous)
    uint32_t tri_base;   // index of the first triangle of this node's leaf slots
    uint8_t  meta[8];    // internal: child offset; leaf: (count << 5) | tri offset; empty: 0
    uint8_t  qlo[3][8];  // [axis][slot]
    uint8_t  qhi[3][8];
};
static_assert(sizeof(WideNode) == 80, "wide node layout");

// Triangle of the wide path: three float4 with the primitive id in v0.w.
struct __align__(16) WideTri
{
    float v0[3];
    uint32_t prim;
    float v1[3];
    uint32_t pad1;
    float v2[3];
    uint32_t pad2;
};
static_assert(sizeof(WideTri) == 48, "triangle layout");

// 4-wide node with exact fp32 child boxes (128 bytes, eight 16-byte words):
// the boxes as structure of arrays, then the child references.  A reference
// is a 4-wide node index, kBvh4Leaf | a binary leaf node index (that node
// holds the triangle), or kInvalid for an empty slot.
struct __align__(16) Bvh4Node
{
    float    lo[3][4];  // [axis][slot]
    float    hi[3][4];
    uint32_t child[4];
    uint32_t pad[4];
};
static_assert(sizeof(Bvh4Node) == 128, "4-wide node layout");
constexpr uint32_t kBvh4Leaf = 0x80000000u;

// 4-wide node with 8-bit conservative child bounds (64 bytes, four 16-byte
// words): per-node origin p and per-axis scale 2^(e - 127); child box of
// slot k on axis a = [p + q[a][k] * s, p + q[3 + a][k] * s], rounded
// outward at build time so that it contains the exact child box.  The child
// references are those of Bvh4Node.
struct __align__(16) Bvh4QNode
{
    float    p[3];
    uint8_t  e[3];
    uint8_t  pad0;
    uint32_t child[4];
    uint8_t  q[6][4];   // planes lo x, y, z, hi x, y, z; [plane][slot]
    uint32_t pad1[2];
};
static_assert(sizeof(Bvh4QNode) == 64, "quantised 4-wide node layout");

// Formats whose buffer carries 4-wide nodes (fp32 or 8-bit bounds).
inline __host__ __device__ bool is_bvh4_format(uint32_t f)
{
    return f == RR_CUDA_NODE_FORMAT_BVH4 || f == RR_CUDA_NODE_FORMAT_BVH4Q8;
}
// Formats with a wide collapse after the binary build.
inline __host__ __device__ bool has_wide_collapse(uint32_t f)
{
    return f == RR_CUDA_NODE_FORMAT_WIDE8 || is_bvh4_format(f);
}

// Trailer written after the binary node array of every result buffer; it
// makes the buffer self-describing (kind, counts, section offsets).
struct __align__(16) Trailer
{
    uint32_t magic;
    uint32_t version;
    uint32_t kind;          // kKindGeom / kKindScene
    uint32_t node_format;   // RRCudaNodeFormat
    uint32_t leaf_count;    // triangles (geometry) or instances (scene)
    uint32_t node_count;    // binary nodes
    uint32_t wide_count;    // wide nodes written (device)
    uint32_t wide_tri_count;// wide triangles written (device)
    uint64_t wide_nodes_off;
    uint64_t wide_tris_off;
    uint64_t wide_capacity;
    uint64_t tri_capacity;
    uint32_t bounds[8];     // mesh/scene box in the order-preserving uint encoding
    uint32_t morton_bits;
    uint32_t prim_kind;     // geometry: kPrimTriangles / kPrimAabbs
    uint32_t pad[2];
    uint64_t xforms_off;    // scene: transforms [inverse, forward] per instance
    uint64_t inst_off;      // scene: InstanceDesc per instance
    uint64_t reserved[16];
};
static_assert(sizeof(Trailer) == 256, "trailer layout");

// Per-instance record of a scene buffer: where the instance's BLAS lives.
struct __align__(16) InstanceDesc
{
    uint64_t blas;       // device address of the BLAS result buffer (binary nodes at offset 0)
    uint64_t wide_nodes; // device address of its wide nodes, 0 if it has none
    uint64_t wide_tris;  // device address of its wide triangles
    uint32_t leaf_count;
    uint32_t flags;
};
static_assert(sizeof(InstanceDesc) == 32, "instance layout");

// Result-buffer layout of a geometry build with N triangles.
struct GeomLayout
{
    uint32_t n;
    uint32_t format;
    uint32_t morton_bits;
    size_t   nodes_bytes;
    size_t   trailer_off;
    size_t   wide_off;
    size_t   wide_capacity;
    size_t   tris_off;
    size_t   tri_capacity;
    size_t   total;
    // scratch
    size_t   s_desc, s_bounds, s_codes, s_codes_alt, s_idx, s_idx_alt, s_sort, s_sort_bytes, s_queue, s_queue_bytes,
        s_topo, s_total;
    // update scratch (RR_BUILD_OPERATION_UPDATE): descriptor | collapse queues
    size_t   u_queue, u_total;
    uint32_t sort_tiles, sort_passes;
    // quality build: treelet restructure of nodes with >= restructure_min
    // triangles (0: fast build), restructure_passes times
    uint32_t restructure_min, restructure_passes;
};
constexpr uint32_t kRestructureMinPrims = 64;  // vlk/restructure_hlbvh.cpp:34
constexpr uint32_t kRestructurePasses   = 3;   // vlk/restructure_hlbvh.cpp:35
GeomLayout geom_layout(uint32_t n, uint32_t format, uint32_t morton_bits);

struct DeviceWords;

// One geometry of a (possibly fused) build, resident on the device.  Offsets
// are the geometry's GeomLayout offsets into its own scratch / result buffer.
struct __align__(16) BuildItem
{
    const float* vertices;
    const void*  indices;
    uint8_t*     scratch;
    uint8_t*     result;
    uint64_t     stride_floats;
    uint64_t     s_bounds, s_codes, s_codes_alt, s_idx, s_idx_alt, s_sort, s_queue;
    uint64_t     s_topo;    // compact topology of the build (emit -> refit): children, parents, climb flags
    uint64_t     trailer_off, wide_off, tris_off;
    uint32_t     wide_capacity, tri_capacity;
    uint32_t     n;
    uint32_t     index16;
    uint32_t     tiles;     // sort tiles of this geometry
    uint32_t     prim_kind; // kPrimTriangles / kPrimAabbs
};

// Batch-wide control words (device).
constexpr int kBatchCounters = 64;
struct BatchCtl
{
    uint32_t sort_tile[16];  // tile claim counter of every onesweep pass
    uint32_t pad[kBatchCounters - 16];
};

// A fused build of `count` geometries with the same node format and key
// width.  `items`, `tile_prefix` (count + 1 exclusive prefix of the sort
// tiles), `level_prefix` (count + 1, collapse work per level) and `ctl` are
// device memory.
struct BatchArgs
{
    const BuildItem* items;
    const uint32_t*  tile_prefix;
    uint32_t*        level_prefix;
    BatchCtl*        ctl;
    uint32_t         count;
    uint32_t         total_tiles;   // sum of items[i].tiles
    uint64_t         total_prims;   // sum of items[i].n
    uint32_t         max_n;         // largest items[i].n
    uint32_t         format;
    uint32_t         morton_bits;
    uint32_t         restructure_min;  // 0: fast build; else treelet restructure of nodes with >= this many triangles
    uint32_t         restructure_passes;
};
size_t batch_desc_bytes(uint32_t count);
// Geometry owning tile t: the largest g < count with prefix[g] <= t (prefix
// has count + 1 entries, prefix[count] > t).  Empty geometries are skipped.
__device__ __forceinline__ uint32_t batch_find(const uint32_t* __restrict__ prefix, uint32_t count, uint32_t t)
{
    uint32_t lo = 0, hi = count;
    while (hi - lo > 1)
    {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(prefix + mid) <= t)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}
// Carve `count` items + prefixes + control words from a device block of
// batch_desc_bytes(count) bytes.
void batch_carve(uint8_t* block, uint32_t count, BuildItem** items, uint32_t** tile_prefix, uint32_t** level_prefix,
                 BatchCtl** ctl);
BuildItem make_build_item(const GeomLayout& L, const float* vertices, uint64_t stride_floats, const void* indices,
                          int index16, uint8_t* scratch, uint8_t* result, uint32_t prim_kind = kPrimTriangles);
// Enqueue the whole fused build (the descriptors must already be on the device).
cudaError_t launch_build_batch(const BatchArgs& b, DeviceWords* words, int sm_count, cudaStream_t s);

struct SceneLayout
{
    uint32_t n;
    size_t   nodes_bytes;
    size_t   xforms_off;
    size_t   trailer_off;
    size_t   inst_off;
    size_t   total;
    size_t   s_bounds, s_boxes, s_codes, s_codes_alt, s_idx, s_idx_alt, s_sort, s_sort_bytes, s_total;
    uint32_t sort_tiles, sort_passes;
};
SceneLayout scene_layout(uint32_t n);

// Context-wide device words.
struct DeviceWords
{
    uint32_t error_bits;
    uint32_t probe;           // written by the stream memory-operation probe
    uint32_t lookback_polls;  // onesweep look-back polls before giving up (0: kLookbackPolls)
    uint32_t hold_tile;       // test only: 1 + the sort tile that never publishes its counts (0: none)
    unsigned long long rays;
    unsigned long long node_fetches;
    unsigned long long tri_fetches;
};

// ---- kernel launchers (all enqueue on `s`, return the launch error) ------
struct MeshArgs
{
    const float* vertices;       // triangles: vertex array; AABBs: the box array
    uint64_t     stride_floats;  // vertex stride or box stride, in floats
    const void*  indices;        // triangles only
    int          index16;
    uint32_t     n;              // triangles or boxes
    uint32_t     prim_kind = kPrimTriangles;
};

cudaError_t launch_build_mesh(const MeshArgs& m, const GeomLayout& L, uint8_t* scratch, uint8_t* result,
                              DeviceWords* words, int sm_count, cudaStream_t s);
// RR_BUILD_OPERATION_UPDATE: new vertex positions, same topology.  Leaves take
// their triangle's new vertices, boxes are refitted bottom-up and the 8-wide
// nodes (if any) are collapsed again.  `scratch` holds L.u_total bytes.
cudaError_t launch_update_mesh(const MeshArgs& m, const GeomLayout& L, uint8_t* scratch, uint8_t* result,
                               DeviceWords* words, int sm_count, cudaStream_t s);

// Sort (codes, identity values) stably; bits = 30 (uint32 keys) or 63 (uint64).
// Returns in *sorted_in_alt whether the result is in the alt buffers.
cudaError_t launch_radix_sort(void* codes, void* codes_alt, uint32_t* idx, uint32_t* idx_alt, uint32_t n,
                              int key_bits, uint8_t* sort_scratch, uint32_t tiles, DeviceWords* words,
                              cudaStream_t s, bool* sorted_in_alt);
size_t   radix_sort_scratch_bytes(uint32_t n, int key_bits, uint32_t* tiles, uint32_t* passes);
// Keys per sort tile (and per tile of the fused build's tile-mapped kernels).
uint32_t radix_sort_tile_keys(int key_bits);
// Per-geometry sort of a fused build: every geometry's Morton codes (at
// s_codes) are sorted into s_codes / s_idx in place (an even pass count), its
// digit histograms (s_sort, built by the Morton kernel) already summed and its
// look-back words already zeroed.  One launch per digit pass for all geometries.
cudaError_t launch_radix_sort_batch(const BatchArgs& b, DeviceWords* words, cudaStream_t s);

struct TraceArgs
{
    const uint8_t*  bvh;          // result buffer base (binary nodes at offset 0)
    const WideNode* wide_nodes;   // wide path
    const WideTri*  wide_tris;
    const Bvh4Node* bvh4_nodes;   // 4-wide path (Bvh4QNode when bvh4_q8)
    int             bvh4_q8;      // the 4-wide nodes have 8-bit bounds
    const uint8_t*  rays;         // RRRay[]
    uint32_t        ray_count;
    const uint32_t* indirect;     // optional device count
    void*           hits;
    uint8_t*        scratch;
    size_t          scratch_bytes;
    int             query;        // RRIntersectQuery
    int             output;       // RRIntersectQueryOutput
    int             empty;        // geometry with no triangles
    uint32_t        node_limit;   // binary nodes in the buffer (kInvalid: unknown)
    uint32_t        wide_limit;   // wide-node (8-wide or 4-wide) capacity
    uint32_t        tri_limit;    // wide-triangle capacity
    const uint32_t* bounds;       // mesh box (order-preserving uint encoding) for ray ordering; may be null
    int             ray_order;    // RRCudaTraversalOptions::ray_order
    DeviceWords*    words;
    int             collect_stats;
    int             block_size;
    int             blocks_per_sm;
    int             short_stack;  // 4-wide kernel's shared stack entries per ray (0: kPShort)
    int             sm_count;
    int             box_leaves;   // AABB-list geometry: leaves are boxes
    int             triangle_test;  // RRCudaTriangleTest
    // Streamed rays (host-buffer tracing; the persistent binary and 4-wide
    // kernels): the rays arrive in chunks of 2^stream_shift while the kernel
    // runs, and the hits leave in parts of 2^stream_part_shift rays (a part
    // is a whole number of chunks).
    // stream_words[c] turns non-zero when chunk c is in device memory;
    // stream_words[stream_chunks + p] counts part p's finished rays;
    // stream_words[stream_chunks + stream_parts] is set when a lane gave up
    // waiting for a chunk; stream_words[stream_chunks + stream_parts + 1]
    // counts the entries of stream_late.
    // stream_late: room for ray_count ray indices.  A ray counted in its
    // part's done counter before its hit was written (its part was published
    // while the ray was still in flight) is listed here, and its hit is
    // copied to the host again after the kernel.
    uint32_t*       stream_words;
    uint32_t*       stream_late;
    uint32_t        stream_shift;
    uint32_t        stream_chunks;
    uint32_t        stream_part_shift;
    uint32_t        stream_parts;
    uint32_t        stream_polls;  // arrival-flag polls (about 1 us each) before giving up (0: default)
};
// Words of a streamed trace (arrival flags, done counters, give-up flag,
// late-list count), rounded up to 256 bytes.
inline size_t stream_words_bytes(uint32_t chunks, uint32_t parts)
{
    return ((size_t)(chunks + parts + 2) * 4 + 255) / 256 * 256;
}
// One request of a multi-request traversal launch (rrCudaCmdIntersectBatch).
constexpr uint32_t kReqAny   = 1;  // any-hit query (else closest)
constexpr uint32_t kReqFull  = 2;  // full RRHit output (else instance id)
constexpr uint32_t kReqEmpty = 4;  // geometry without triangles: every ray misses
constexpr uint32_t kReqBoxes = 8;  // AABB-list geometry: leaves are boxes
constexpr uint32_t kReqBvh4  = 16; // traced over the geometry's 4-wide nodes
struct __align__(16) BatchTraceReq
{
    const uint8_t* bvh;   // geometry result buffer (binary nodes at offset 0)
    const uint8_t* rays;  // RRRay[ray_count]
    void*          hits;
    uint32_t       ray_count;
    uint32_t       node_limit;  // binary nodes in the buffer (kInvalid: unknown)
    uint32_t       flags;
    uint32_t       wide_off256; // kReqBvh4: byte offset of the 4-wide nodes / 256
    uint32_t       wide_limit;  // kReqBvh4: 4-wide node capacity
    uint32_t       pad;
};
static_assert(sizeof(BatchTraceReq) == 48, "request layout");

// Scratch of a multi-request launch: control words | request table | ray
// prefix (count + 1) | per-thread stack spill.
struct BatchTraceLayout
{
    size_t req_off, prefix_off, spill_off, total;
};
BatchTraceLayout batch_trace_layout(uint32_t count, uint64_t total_rays);

struct BatchTraceArgs
{
    const BatchTraceReq* req;
    const uint32_t*      prefix;
    uint32_t             count;
    uint32_t             total;  // prefix[count]
    uint8_t*             scratch;
    size_t               scratch_bytes;
    size_t               spill_off;
    DeviceWords*         words;
    int                  sm_count;
    int                  blocks_per_sm;
    int                  collect_stats;
    int                  use_bvh4;  // every request kReqBvh4 or empty: the 4-wide kernel
    int                  bvh4_q8;   // ... and their 4-wide nodes have 8-bit bounds (Bvh4QNode)
};
// Every request's rays in one persistent launch (per ray the visit order of
// the single-request kernel it stands for -- the reference's binary order, or
// the 4-wide kernel's with use_bvh4 -- so each hit equals the single-request
// result).  The request table and prefix must already be in the scratch.
cudaError_t launch_trace_batch(const BatchTraceArgs& a, cudaStream_t s);

cudaError_t launch_trace_binary(const TraceArgs& a, cudaStream_t s);
cudaError_t launch_trace_wide(const TraceArgs& a, cudaStream_t s);
cudaError_t launch_trace_persistent(const TraceArgs& a, cudaStream_t s);
cudaError_t launch_trace_bvh4(const TraceArgs& a, cudaStream_t s);

struct SceneTraceArgs
{
    TraceArgs           base;       // bvh = TLAS buffer
    const float*        xforms;     // [inverse, forward] 12 floats each
    const InstanceDesc* inst;
    uint32_t            inst_count;
    int                 use_wide;        // 8-wide BLAS kernel
    int                 use_persistent;  // persistent binary two-level kernel
    int                 use_bvh4;        // persistent kernel over 4-wide BLASes (all instances of one 4-wide form)
    int                 bvh4_q8;         // ... BVH4Q8 (8-bit bounds)
};
cudaError_t launch_trace_scene(const SceneTraceArgs& a, cudaStream_t s);
cudaError_t launch_trace_scene_persistent(const SceneTraceArgs& a, cudaStream_t s);
cudaError_t launch_trace_scene_bvh4(const SceneTraceArgs& a, cudaStream_t s);

struct SceneBuildArgs
{
    const InstanceDesc* inst;      // device: per instance BLAS pointers
    const float*        forward;   // device: 12 floats per instance
    uint32_t            n;
};
cudaError_t launch_build_scene(const SceneBuildArgs& a, const SceneLayout& L, uint8_t* scratch, uint8_t* result,
                               DeviceWords* words, cudaStream_t s);

size_t trace_scratch_bytes(uint32_t ray_count);
// After a streamed trace: copies the hit records of the late-listed rays
// (count at *late_count, at most cap) from dev_hits to host_hits (a
// device-accessible pointer to the host buffer), rec_bytes (4 or 16) each.
// RR_BUILD_OPERATION_UPDATE of a buffer with 4-wide nodes, after the binary
// refit: each 4-wide node takes its children's new boxes (same topology).
cudaError_t launch_refit_bvh4(uint8_t* result, const GeomLayout& L, DeviceWords* words, int sm_count, cudaStream_t s);
cudaError_t launch_late_scatter(const uint32_t* late_count, const uint32_t* late, uint32_t cap,
                                const uint8_t* dev_hits, uint8_t* host_hits, uint32_t rec_bytes, int sm_count,
                                cudaStream_t s);

}  // namespace rr
