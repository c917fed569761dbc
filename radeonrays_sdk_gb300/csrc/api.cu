// api.cu -- the C-ABI of the GB300 RadeonRays build (librr.so).
//
// Mirrors the reference's API shim (src/core/src/radeonrays.cpp) and its
// Vulkan intersector facade (src/core/src/vlk/intersector.cpp): the same entry
// points, argument checks and error codes, with one backend (CUDA) and no
// virtual dispatch.  Execution model:
//   * a command stream from rrAllocateCommandStream records operations; the
//     first rrSumbitCommandStream captures them into a CUDA graph that later
//     submissions replay (falls back to direct launches if capture fails);
//   * a command stream from rrGetCommandStreamFromCudaStream enqueues each
//     operation immediately on the caller's CUDA stream;
//   * RREvent wraps a cudaEvent_t; rrWaitEvent polls it with a timeout.
// No exception crosses the C boundary; CUDA allocation failures map to
// RR_ERROR_OUT_OF_DEVICE_MEMORY, other failures to RR_ERROR_INTERNAL.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include <cuda.h>  // driver types of the stream memory operations (entry points fetched at run time)

#include "rr_internal.h"

using namespace rr;

// ---------------------------------------------------------------------------
// Logging (the reference wraps spdlog, utils/logger.h:33-110; this is a
// level-filtered stderr/file logger with the same two controls).
namespace
{
std::mutex g_log_mu;
int        g_log_level = RR_LOG_LEVEL_WARN;
FILE*      g_log_file  = nullptr;

void logf(int level, const char* fmt, ...)
{
    if (level < g_log_level || g_log_level >= RR_LOG_LEVEL_OFF) return;
    static const char* names[] = {"", "debug", "info", "warn", "error"};
    std::lock_guard<std::mutex> lk(g_log_mu);
    FILE*                       f = g_log_file ? g_log_file : stderr;
    std::fprintf(f, "[rr %s] ", names[std::min(level, 4)]);
    va_list ap;
    va_start(ap, fmt);
    std::vfprintf(f, fmt, ap);
    va_end(ap);
    std::fputc('\n', f);
    std::fflush(f);
}
#define RR_LOG_INFO(...) logf(RR_LOG_LEVEL_INFO, __VA_ARGS__)
#define RR_LOG_ERROR(...) logf(RR_LOG_LEVEL_ERROR, __VA_ARGS__)

struct CudaFail : std::runtime_error
{
    cudaError_t code;
    CudaFail(cudaError_t c, const char* what) : std::runtime_error(what), code(c) {}
};
inline void check(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) throw CudaFail(e, what);
}

RRError map_error(const CudaFail& f)
{
    RR_LOG_ERROR("%s: %s", f.what(), cudaGetErrorString(f.code));
    return f.code == cudaErrorMemoryAllocation ? RR_ERROR_OUT_OF_DEVICE_MEMORY : RR_ERROR_INTERNAL;
}

// ---------------------------------------------------------------------------
struct BufInfo
{
    uint32_t kind   = 0;
    uint32_t n      = 0;
    uint32_t format = RR_CUDA_NODE_FORMAT_BINARY;
    size_t   trailer_off = 0, wide_off = 0, tris_off = 0, xforms_off = 0, inst_off = 0;
    size_t   wide_capacity = 0;  // geometry: 8-wide or 4-wide node capacity
    bool     scene_wide = false;  // scene: every instance has 8-wide nodes
    bool     scene_bvh4 = false;  // scene: every instance has 4-wide nodes of one form
    bool     scene_bvh4_q8 = false;  // ... with 8-bit bounds
    uint32_t prim_kind  = kPrimTriangles;  // geometry: triangles or AABB list
};

struct Context;

using Op = std::function<cudaError_t(cudaStream_t)>;

// Device memory owned by a recorded op (the descriptors of a fused build).
struct DeviceBlock
{
    void* p = nullptr;
    explicit DeviceBlock(size_t bytes)
    {
        if (bytes) check(cudaMalloc(&p, bytes), "cudaMalloc build descriptors");
    }
    ~DeviceBlock()
    {
        if (p) cudaFree(p);
    }
};

// A geometry build recorded into a command stream and not yet turned into an
// op: consecutive ones are fused into one build (build_batch_op).
struct PendingGeom
{
    MeshArgs   ma;
    GeomLayout L;
    uint8_t*   scratch;
    uint8_t*   result;
};

// Disjoint byte ranges [start, end) of device memory.
struct RangeSet
{
    std::map<uintptr_t, uintptr_t> r;
    bool overlaps(const uint8_t* p, size_t n) const
    {
        if (!p || !n) return false;
        const uintptr_t s = (uintptr_t)p, e = s + n;
        auto            it = r.lower_bound(e);  // first range starting at or after e
        if (it == r.begin()) return false;
        --it;
        return it->second > s;
    }
    void add(const uint8_t* p, size_t n)
    {
        if (p && n) r[(uintptr_t)p] = (uintptr_t)p + n;
    }
};

struct CommandStream
{
    Context*                 ctx      = nullptr;
    bool                     external = false;
    cudaStream_t             stream   = nullptr;
    std::vector<Op>          ops;
    std::vector<PendingGeom> pending;
    RangeSet                 pending_ranges;
    bool                     want_graph   = false;  // an op enqueues many launches
    cudaGraphExec_t          graph        = nullptr;
    size_t                   graph_ops    = 0;
    bool                     graph_failed = false;
    ~CommandStream()
    {
        if (graph) cudaGraphExecDestroy(graph);
    }
};

struct Event
{
    cudaEvent_t ev = nullptr;
};

struct DevicePtr
{
    uint8_t* base    = nullptr;
    size_t   offset  = 0;
    bool     managed = false;  // allocated by rrAllocateDeviceBuffer (owned)
    size_t   size    = 0;
    uint8_t* addr() const { return base + offset; }
};

// Page-locked host blocks for the staging of ops, reused.  cudaMallocHost
// pins pages (milliseconds for large blocks) and cudaFreeHost can wait for
// the device, which serialised multi-request launches that should overlap
// on different streams.  Blocks come in power-of-two sizes from 4 KiB; up to
// kKeep bytes of returned blocks are kept, the rest freed.  Ops hold the
// pool by shared pointer, so it outlives the context if an op does.
struct PinnedPool
{
    static constexpr size_t         kKeep = size_t(256) << 20;
    std::mutex                      mu;
    std::multimap<size_t, void*>    free_blocks;  // capacity -> block
    size_t                          held = 0;
    void* take(size_t bytes, size_t& cap)
    {
        cap = 4096;
        while (cap < bytes) cap <<= 1;
        {
            std::lock_guard<std::mutex> lock(mu);
            auto it = free_blocks.find(cap);
            if (it != free_blocks.end())
            {
                void* p = it->second;
                free_blocks.erase(it);
                held -= cap;
                return p;
            }
        }
        void* p = nullptr;
        check(cudaMallocHost(&p, cap), "cudaMallocHost");
        return p;
    }
    void give(void* p, size_t cap)
    {
        {
            std::lock_guard<std::mutex> lock(mu);
            if (held + cap <= kKeep)
            {
                free_blocks.emplace(cap, p);
                held += cap;
                return;
            }
        }
        cudaFreeHost(p);
    }
    ~PinnedPool()
    {
        for (auto& b : free_blocks) cudaFreeHost(b.second);
    }
};

struct Context
{
    int                    device   = 0;
    int                    sm_count = 1;
    cudaStream_t           stream   = nullptr;
    DeviceWords*           words    = nullptr;
    RRCudaTraversalOptions topts{};
    uint32_t               wait_ms  = 600000;
    bool                   graphs   = true;
    bool                   fuse_builds = true;  // fuse consecutive geometry builds of a command stream
    std::string            gpu_name;
    std::map<std::string, uint32_t> fmt_choice;  // node-format tuner results by mesh-size key
    std::map<std::string, RRCudaTraversalOptions> tuned;  // autotuner results by workload key
    std::map<uintptr_t, BufInfo> registry;
    std::shared_ptr<PinnedPool>  pinned = std::make_shared<PinnedPool>();
    // Ops run at once on external streams, kept (with the memory they own)
    // until an event after them has completed; ops enqueued into a stream
    // capture are kept until the context goes.
    std::deque<std::pair<cudaEvent_t, Op>> retired;
    std::vector<Op>                        kept;
    // Side streams and fork/join events of host-buffer tracing (copy/compute
    // pipelining), created on first use.
    static constexpr int kPipe = 3;
    cudaStream_t         pipe[kPipe]      = {};
    cudaEvent_t          pipe_fork        = nullptr;
    cudaEvent_t          pipe_join[kPipe] = {};
    cudaEvent_t          pipe_kdone       = nullptr;  // streamed plan: after the kernel
    // Stream memory operations (driver entry points looked up once): the
    // streamed host-buffer trace sets arrival flags and waits on done
    // counters with them.  memops: 0 not probed, 1 usable, -1 not available.
    // RR_CUDA_STREAM_RAYS=0 turns the streamed plan off.
    int   memops      = 0;
    void* write_value = nullptr;
    void* wait_value  = nullptr;
    bool  stream_rays = true;
    // Bounded device waits (rrCudaSetWaitLimits): arrival polls of a streamed
    // trace (0: default) and the test hook that never raises one chunk's
    // arrival flag (kInvalid: none).  The look-back limit lives in `words`.
    uint32_t arrival_polls = 0;
    uint32_t drop_arrival  = kInvalid;
    void ensure_pipe()
    {
        if (pipe_fork) return;
        for (int p = 0; p < kPipe; ++p)
        {
            check(cudaStreamCreateWithFlags(&pipe[p], cudaStreamNonBlocking), "pipeline stream");
            check(cudaEventCreateWithFlags(&pipe_join[p], cudaEventDisableTiming), "pipeline event");
        }
        check(cudaEventCreateWithFlags(&pipe_fork, cudaEventDisableTiming), "pipeline event");
        check(cudaEventCreateWithFlags(&pipe_kdone, cudaEventDisableTiming), "pipeline event");
    }
    void retire(Op&& op, cudaStream_t s)
    {
        cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
        cudaStreamIsCapturing(s, &cap);
        if (cap != cudaStreamCaptureStatusNone)
        {
            kept.push_back(std::move(op));
            return;
        }
        cudaEvent_t ev = nullptr;
        if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventRecord(ev, s) != cudaSuccess)
        {
            cudaGetLastError();
            if (ev) cudaEventDestroy(ev);
            cudaStreamSynchronize(s);
            return;
        }
        retired.emplace_back(ev, std::move(op));
        while (!retired.empty() && cudaEventQuery(retired.front().first) != cudaErrorNotReady)
        {
            cudaEventDestroy(retired.front().first);
            retired.pop_front();
        }
        cudaGetLastError();
    }
    ~Context()
    {
        if (stream) cudaStreamSynchronize(stream);
        for (auto& r : retired)
        {
            cudaEventSynchronize(r.first);
            cudaEventDestroy(r.first);
        }
        retired.clear();
        kept.clear();
        for (int p = 0; p < kPipe; ++p)
        {
            if (pipe[p]) cudaStreamSynchronize(pipe[p]);
            if (pipe[p]) cudaStreamDestroy(pipe[p]);
            if (pipe_join[p]) cudaEventDestroy(pipe_join[p]);
        }
        if (pipe_fork) cudaEventDestroy(pipe_fork);
        if (pipe_kdone) cudaEventDestroy(pipe_kdone);
        if (words) cudaFree(words);
        if (stream) cudaStreamDestroy(stream);
    }
};

struct DeviceGuard
{
    int prev = -1;
    explicit DeviceGuard(int dev)
    {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard()
    {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

inline Context*       C(RRContext c) { return reinterpret_cast<Context*>(c); }
inline CommandStream* S(RRCommandStream s) { return reinterpret_cast<CommandStream*>(s); }
inline DevicePtr*     P(RRDevicePtr p) { return reinterpret_cast<DevicePtr*>(p); }
inline Event*         E(RREvent e) { return reinterpret_cast<Event*>(e); }

// Whether a geometry build touches a byte of scratch or result that builds
// already in `used` touch (then they cannot run fused: they would overwrite
// each other's state).  Otherwise its ranges are added.
bool claim_build_ranges(RangeSet& used, const PendingGeom& g)
{
    if (used.overlaps(g.scratch, g.L.s_total) || used.overlaps(g.result, g.L.total)) return false;
    if (g.scratch && g.result && g.L.s_total && g.scratch < g.result + g.L.total && g.result < g.scratch + g.L.s_total)
        return false;
    used.add(g.scratch, g.L.s_total);
    used.add(g.result, g.L.total);
    return true;
}

// The op of a fused build: descriptors of every geometry copied to a device
// block the op owns, then one launch_build_batch.  A single geometry keeps
// its descriptor in its own scratch (no allocation).
Op build_batch_op(Context* ctx, const std::vector<PendingGeom>& geoms, bool* many_launches)
{
    DeviceWords* words = ctx->words;
    const int    sms   = ctx->sm_count;
    *many_launches     = false;
    if (geoms.size() == 1)
    {
        const PendingGeom pg = geoms[0];
        return [=](cudaStream_t s) { return launch_build_mesh(pg.ma, pg.L, pg.scratch, pg.result, words, sms, s); };
    }
    const uint32_t       count = (uint32_t)geoms.size();
    const size_t         bytes = batch_desc_bytes(count);
    std::vector<uint8_t> host(bytes, 0);
    BuildItem*           hi = nullptr;
    uint32_t *           htp = nullptr, *hlp = nullptr;
    BatchCtl*            hctl = nullptr;
    batch_carve(host.data(), count, &hi, &htp, &hlp, &hctl);
    uint64_t tiles = 0, prims = 0;
    uint32_t max_n = 0;
    for (uint32_t i = 0; i < count; ++i)
    {
        const PendingGeom& g = geoms[i];
        hi[i]  = make_build_item(g.L, g.ma.vertices, g.ma.stride_floats, g.ma.indices, g.ma.index16, g.scratch,
                                 g.result, g.ma.prim_kind);
        htp[i] = (uint32_t)tiles;
        tiles += g.L.sort_tiles;
        prims += g.L.n;
        max_n  = std::max(max_n, g.L.n);
    }
    if (tiles >= (1ull << 26)) throw std::runtime_error("fused build too large (more than 2^26 sort tiles)");
    htp[count] = (uint32_t)tiles;
    auto dev   = std::make_shared<DeviceBlock>(bytes);
    check(cudaMemcpy(dev->p, host.data(), bytes, cudaMemcpyHostToDevice), "copy build descriptors");
    BuildItem* di  = nullptr;
    uint32_t * dtp = nullptr, *dlp = nullptr;
    BatchCtl*  dctl = nullptr;
    batch_carve(reinterpret_cast<uint8_t*>(dev->p), count, &di, &dtp, &dlp, &dctl);
    BatchArgs b{};
    b.items        = di;
    b.tile_prefix  = dtp;
    b.level_prefix = dlp;
    b.ctl          = dctl;
    b.count        = count;
    b.total_tiles  = (uint32_t)tiles;
    b.total_prims  = prims;
    b.max_n        = max_n;
    b.format       = geoms[0].L.format;
    b.morton_bits  = geoms[0].L.morton_bits;
    b.restructure_min    = geoms[0].L.restructure_min;
    b.restructure_passes = geoms[0].L.restructure_passes;
    *many_launches = true;
    return [=](cudaStream_t s) {
        (void)dev;  // keeps the descriptors alive as long as the op
        return launch_build_batch(b, words, sms, s);
    };
}

void flush_builds(CommandStream* cs)
{
    if (cs->pending.empty()) return;
    bool many = false;
    Op   op   = build_batch_op(cs->ctx, cs->pending, &many);
    cs->pending.clear();
    cs->pending_ranges.r.clear();
    cs->want_graph = cs->want_graph || many;
    cs->ops.push_back(std::move(op));
}

// Append an op to a command stream, or run it at once on an external one.
// An op that owns memory (owns = true) is kept until the GPU is past it.
void record(CommandStream* cs, Op op, bool owns = false)
{
    if (cs->external)
    {
        check(op(cs->stream), "enqueue");
        if (owns) cs->ctx->retire(std::move(op), cs->stream);
        return;
    }
    flush_builds(cs);
    cs->ops.push_back(std::move(op));
}

struct BuildParams
{
    uint32_t format      = RR_CUDA_NODE_FORMAT_BVH4Q8;  // the default: 4-wide nodes with 8-bit bounds
    uint32_t bits        = 30;
    bool     restructure = false;
};

// RRBuildOptions -> node format, key width and quality.  As in the reference
// (vlk/intersector.cpp:115-119, 170-181), options whose build_flags lack
// RR_BUILD_FLAG_BITS_PREFER_FAST_BUILD ask for the treelet restructure; no
// options at all is a fast build.
bool parse_build_options(const RRBuildOptions* o, BuildParams& bp)
{
    if (o) bp.restructure = (o->build_flags & RR_BUILD_FLAG_BITS_PREFER_FAST_BUILD) == 0;
    if (!o || !o->backend_specific_info) return true;
    const RRCudaBuildOptions* c = reinterpret_cast<const RRCudaBuildOptions*>(o->backend_specific_info);
    if (c->struct_size < sizeof(RRCudaBuildOptions)) return false;
    if (c->node_format != RR_CUDA_NODE_FORMAT_BINARY && c->node_format != RR_CUDA_NODE_FORMAT_WIDE8 &&
        c->node_format != RR_CUDA_NODE_FORMAT_BVH4 && c->node_format != RR_CUDA_NODE_FORMAT_AUTO &&
        c->node_format != RR_CUDA_NODE_FORMAT_BVH4Q8)
        return false;
    if (c->morton_bits != 0 && c->morton_bits != 30 && c->morton_bits != 63) return false;
    bp.format = c->node_format;
    bp.bits   = c->morton_bits == 63 ? 63 : 30;
    return true;
}

// Validation of a triangle-mesh build input (reference radeonrays.cpp:242-299,
// vlk/intersector.cpp:137-175).
//
// AABB lists (RR_PRIMITIVE_TYPE_AABB_LIST, radeonrays.h:194-206) are accepted
// too, where the reference returns RR_ERROR_NOT_IMPLEMENTED
// (radeonrays.cpp:286-289): one RRAABBListPrimitive of `aabb_count` boxes, each
// a (min.xyz, _) (max.xyz, _) float4 pair `aabb_stride` bytes apart (at least
// 32, a multiple of 4).  They are built into binary nodes only.
RRError geometry_source(const RRGeometryBuildInput* in, bool need_buffers, MeshArgs* ma)
{
    if (in->primitive_type == RR_PRIMITIVE_TYPE_AABB_LIST)
    {
        if (in->primitive_count != 1 || !in->aabb_primitives) return RR_ERROR_INVALID_PARAMETER;
        const RRAABBListPrimitive* b = in->aabb_primitives;
        if (need_buffers && b->aabb_count > 0 && !b->aabbs) return RR_ERROR_INVALID_PARAMETER;
        if (b->aabb_stride < 32 || (b->aabb_stride & 3u)) return RR_ERROR_INVALID_PARAMETER;
        if (b->aabb_count >= (1u << 30)) return RR_ERROR_INVALID_PARAMETER;
        ma->vertices      = b->aabbs ? reinterpret_cast<const float*>(P(b->aabbs)->addr()) : nullptr;
        ma->stride_floats = b->aabb_stride >> 2;
        ma->indices       = nullptr;
        ma->index16       = 0;
        ma->n             = b->aabb_count;
        ma->prim_kind     = kPrimAabbs;
        return RR_SUCCESS;
    }
    if (in->primitive_type != RR_PRIMITIVE_TYPE_TRIANGLE_MESH) return RR_ERROR_NOT_IMPLEMENTED;
    if (in->primitive_count != 1 || !in->triangle_mesh_primitives) return RR_ERROR_INVALID_PARAMETER;
    const RRTriangleMeshPrimitive* m = in->triangle_mesh_primitives;
    if (need_buffers && m->triangle_count > 0 && (!m->vertices || !m->triangle_indices))
        return RR_ERROR_INVALID_PARAMETER;
    if (m->vertex_stride < 12 || (m->vertex_stride & 3u)) return RR_ERROR_INVALID_PARAMETER;
    if (m->index_type != RR_INDEX_TYPE_UINT32 && m->index_type != RR_INDEX_TYPE_UINT16)
        return RR_ERROR_INVALID_PARAMETER;
    if (m->triangle_count >= (1u << 30)) return RR_ERROR_INVALID_PARAMETER;
    ma->vertices      = m->vertices ? reinterpret_cast<const float*>(P(m->vertices)->addr()) : nullptr;
    ma->stride_floats = m->vertex_stride >> 2;
    ma->indices       = m->triangle_indices ? P(m->triangle_indices)->addr() : nullptr;
    ma->index16       = m->index_type == RR_INDEX_TYPE_UINT16;
    ma->n             = m->triangle_count;
    ma->prim_kind     = kPrimTriangles;
    return RR_SUCCESS;
}

// Node format of a build: AABB lists have binary nodes only.
inline uint32_t build_format(const MeshArgs& ma, uint32_t requested)
{
    return ma.prim_kind == kPrimAabbs ? (uint32_t)RR_CUDA_NODE_FORMAT_BINARY : requested;
}

// Validate one geometry build (reference radeonrays.cpp:242-299) and resolve
// its buffers.
// RR_CUDA_NODE_FORMAT_AUTO: the node width rrCudaAutotuneNodeFormat chose
// for meshes of this size (triangle-count octave) on this GPU -- from the
// context, else from the RR_CUDA_TUNE_CACHE file -- or BVH4 when none was.
std::string fmt_key(const Context* ctx, uint32_t n)
{
    uint32_t octave = 0;
    while ((1ull << (octave + 1)) <= n) ++octave;
    return "fmt|" + ctx->gpu_name + "|" + std::to_string(octave);
}
uint32_t resolve_format(Context* ctx, uint32_t requested, uint32_t n)
{
    if (requested != RR_CUDA_NODE_FORMAT_AUTO) return requested;
    const std::string key = fmt_key(ctx, n);
    auto              hit = ctx->fmt_choice.find(key);
    if (hit == ctx->fmt_choice.end())
    {
        uint32_t fmt = RR_CUDA_NODE_FORMAT_BVH4Q8;  // the default format when nothing was tuned
        if (const char* path = std::getenv("RR_CUDA_TUNE_CACHE"))
            if (FILE* f = std::fopen(path, "r"))
            {
                char line[512];
                while (std::fgets(line, sizeof(line), f))
                {
                    char*    tab = std::strchr(line, '\t');
                    unsigned v   = 0;
                    if (!tab) continue;
                    *tab = 0;
                    if (key == line && std::sscanf(tab + 1, "%u", &v) == 1 &&
                        (is_bvh4_format(v) || v == RR_CUDA_NODE_FORMAT_WIDE8))
                        fmt = v;
                }
                std::fclose(f);
            }
        hit = ctx->fmt_choice.emplace(key, fmt).first;
    }
    return hit->second;
}

RRError prepare_geometry(Context* ctx, const RRGeometryBuildInput* in, const BuildParams& bp,
                         RRDevicePtr temporary_buffer, RRDevicePtr geometry_buffer, PendingGeom* pg)
{
    RRError e = geometry_source(in, true, &pg->ma);
    if (e != RR_SUCCESS) return e;
    if (!geometry_buffer || (!temporary_buffer && pg->ma.n > 0)) return RR_ERROR_INVALID_PARAMETER;
    const uint32_t fmt       = resolve_format(ctx, bp.format, pg->ma.n);
    pg->L                    = geom_layout(pg->ma.n, build_format(pg->ma, fmt), bp.bits);
    pg->L.restructure_min    = bp.restructure ? kRestructureMinPrims : 0u;
    pg->L.restructure_passes = bp.restructure ? kRestructurePasses : 0u;
    pg->scratch          = temporary_buffer ? P(temporary_buffer)->addr() : nullptr;
    pg->result           = P(geometry_buffer)->addr();
    return RR_SUCCESS;
}

// Remember what a result buffer holds (scene builds and traversal read it).
void register_geometry(Context* ctx, const PendingGeom& pg)
{
    BufInfo bi;
    bi.kind                             = kKindGeom;
    bi.n                                = pg.L.n;
    bi.format                           = pg.L.format;
    bi.trailer_off                      = pg.L.trailer_off;
    bi.wide_off                         = pg.L.wide_off;
    bi.tris_off                         = pg.L.tris_off;
    bi.wide_capacity                    = pg.L.wide_capacity;
    bi.prim_kind                        = pg.ma.prim_kind;
    ctx->registry[(uintptr_t)pg.result] = bi;
}

// Record a geometry build: fused with the builds recorded just before it when
// they share format and key width and touch disjoint memory.
void record_build(CommandStream* cs, const PendingGeom& pg)
{
    if (cs->external || !cs->ctx->fuse_builds)
    {
        std::vector<PendingGeom> one{pg};
        bool                     many = false;
        record(cs, build_batch_op(cs->ctx, one, &many));
        return;
    }
    bool fits = true;
    if (!cs->pending.empty())
    {
        const PendingGeom& f = cs->pending.front();
        fits = f.L.format == pg.L.format && f.L.morton_bits == pg.L.morton_bits &&
               f.L.restructure_min == pg.L.restructure_min && claim_build_ranges(cs->pending_ranges, pg);
    }
    if (!fits)
    {
        flush_builds(cs);
        claim_build_ranges(cs->pending_ranges, pg);
    }
    else if (cs->pending.empty())
        claim_build_ranges(cs->pending_ranges, pg);
    cs->pending.push_back(pg);
}

// 3x4 affine inverse in double, rounded once to float.
void inverse34(const float* m, float* out)
{
    double a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[6], g = m[8], h = m[9], i = m[10];
    double A = e * i - f * h, B = -(d * i - f * g), Cc = d * h - e * g;
    double det = a * A + b * B + c * Cc;
    if (det == 0.0)
    {
        for (int k = 0; k < 12; ++k) out[k] = 0.f;
        return;
    }
    double r = 1.0 / det;
    double inv[9];
    inv[0] = A * r;
    inv[1] = -(b * i - c * h) * r;
    inv[2] = (b * f - c * e) * r;
    inv[3] = B * r;
    inv[4] = (a * i - c * g) * r;
    inv[5] = -(a * f - c * d) * r;
    inv[6] = Cc * r;
    inv[7] = -(a * h - b * g) * r;
    inv[8] = (a * e - b * d) * r;
    double tx = m[3], ty = m[7], tz = m[11];
    for (int row = 0; row < 3; ++row)
    {
        out[row * 4 + 0] = (float)inv[row * 3 + 0];
        out[row * 4 + 1] = (float)inv[row * 3 + 1];
        out[row * 4 + 2] = (float)inv[row * 3 + 2];
        out[row * 4 + 3] = (float)(-(inv[row * 3 + 0] * tx + inv[row * 3 + 1] * ty + inv[row * 3 + 2] * tz));
    }
}

// A staging block of the context's pinned pool, returned to it when the op
// that owns it is destroyed (after the op's copies have completed).
struct PinnedBlock
{
    std::shared_ptr<PinnedPool> pool;
    void*                       p   = nullptr;
    size_t                      cap = 0;
    PinnedBlock(const std::shared_ptr<PinnedPool>& from, size_t bytes) : pool(from)
    {
        if (bytes) p = pool->take(bytes, cap);
    }
    ~PinnedBlock()
    {
        if (p) pool->give(p, cap);
    }
};

}  // namespace

#define RR_TRY(...)                                                  \
    try                                                              \
    {                                                                \
        __VA_ARGS__                                                  \
    }                                                                \
    catch (const CudaFail& f)                                        \
    {                                                                \
        return map_error(f);                                         \
    }                                                                \
    catch (const std::bad_alloc&)                                    \
    {                                                                \
        RR_LOG_ERROR("out of host memory");                          \
        return RR_ERROR_OUT_OF_HOST_MEMORY;                          \
    }                                                                \
    catch (const std::exception& ex)                                 \
    {                                                                \
        RR_LOG_ERROR("%s", ex.what());                               \
        return RR_ERROR_INTERNAL;                                    \
    }                                                                \
    catch (...)                                                      \
    {                                                                \
        return RR_ERROR_INTERNAL;                                    \
    }

namespace
{
typedef CUresult (*PfnStreamValue32)(CUstream, CUdeviceptr, cuuint32_t, unsigned int);

// Look up cuStreamWriteValue32 / cuStreamWaitValue32 and check them once on
// the context's stream: write 1 to a device word, read it back, then wait for
// it (already 1, so the wait cannot block).
bool memops_ok(Context* ctx)
{
    if (ctx->memops) return ctx->memops > 0;
    ctx->memops = -1;
    if (!ctx->stream_rays) return false;
    cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
    void *w = nullptr, *v = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuStreamWriteValue32", &w, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuStreamWaitValue32", &v, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
        q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !w || !v)
    {
        cudaGetLastError();
        return false;
    }
    const CUdeviceptr word = (CUdeviceptr)(uintptr_t)&ctx->words->probe;
    uint32_t          back = 0;
    if (cudaMemsetAsync(&ctx->words->probe, 0, 4, ctx->stream) != cudaSuccess ||
        reinterpret_cast<PfnStreamValue32>(w)((CUstream)ctx->stream, word, 1u, CU_STREAM_WRITE_VALUE_DEFAULT) !=
            CUDA_SUCCESS ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess ||
        cudaMemcpy(&back, &ctx->words->probe, 4, cudaMemcpyDeviceToHost) != cudaSuccess || back != 1u)
    {
        cudaStreamSynchronize(ctx->stream);
        cudaGetLastError();
        return false;
    }
    if (reinterpret_cast<PfnStreamValue32>(v)((CUstream)ctx->stream, word, 1u, CU_STREAM_WAIT_VALUE_GEQ) !=
            CUDA_SUCCESS ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess)
    {
        cudaGetLastError();
        return false;
    }
    ctx->write_value = w;
    ctx->wait_value  = v;
    ctx->memops      = 1;
    return true;
}

// Streamed rays of a host-buffer trace: copy-in chunks of 2^shift rays,
// copy-out parts of 2^part_shift rays; `words` the arrival / done / give-up
// words (stream_words_bytes(chunks, parts) bytes at the end of the scratch,
// which the kernel's spill region leaves out).
struct StreamPlan
{
    uint32_t* words      = nullptr;
    uint32_t* late       = nullptr;  // late list (ray_count entries)
    uint32_t  shift      = 0;
    uint32_t  chunks     = 0;
    uint32_t  part_shift = 0;
    uint32_t  parts      = 0;
    size_t    scratch_bytes = 0;  // scratch left to the kernel
};

// The precise triangle test runs on triangle geometries only (the two-level,
// AABB-list and multi-request kernels keep the reference's test).
bool precise_unsupported(Context* ctx, const uint8_t* bvh)
{
    if (ctx->topts.triangle_test != RR_CUDA_TRIANGLE_TEST_WATERTIGHT) return false;
    auto it = ctx->registry.find((uintptr_t)bvh);
    if (it == ctx->registry.end()) return false;  // traversed as binary triangle nodes
    return it->second.kind != kKindGeom || it->second.prim_kind != kPrimTriangles;
}

// The launch of one rrCmdIntersect: arguments from the buffers and the
// traversal options, kernel chosen by the buffer kind and options.  With a
// stream plan, returns an empty Op unless the persistent binary or the
// 4-wide kernel would run (the kernels with a streamed variant).
Op trace_op(Context* ctx, uint8_t* bvh, const uint8_t* rays, uint32_t ray_count, const uint32_t* indirect, void* hits,
            uint8_t* scratch, int query, int output, const RRCudaTraversalOptions& o,
            const StreamPlan* sp = nullptr)
{
    TraceArgs a{};
    a.bvh           = bvh;
    a.rays          = rays;
    a.ray_count     = ray_count;
    a.indirect      = indirect;
    a.hits          = hits;
    a.scratch       = scratch;
    a.scratch_bytes = trace_scratch_bytes(ray_count);
    a.query         = query;
    a.output        = output;
    a.words         = ctx->words;
    a.collect_stats = o.collect_stats ? 1 : 0;
    a.block_size    = (int)o.block_size;
    a.blocks_per_sm = (int)o.blocks_per_sm;
    a.short_stack   = (int)o.short_stack;
    a.ray_order     = (int)o.ray_order;
    a.sm_count      = ctx->sm_count;
    a.stream_polls  = ctx->arrival_polls;
    a.triangle_test = (int)o.triangle_test;
    auto    it      = ctx->registry.find((uintptr_t)bvh);
    BufInfo bi;
    if (it != ctx->registry.end()) bi = it->second;
    const uint32_t trav  = o.traversal;
    const uint32_t nodes = bi.n == 0 ? 0u : 2u * bi.n - 1u;
    a.node_limit         = bi.kind == 0 ? kInvalid : nodes;
    a.box_leaves         = bi.kind == kKindGeom && bi.prim_kind == kPrimAabbs;
    a.wide_limit         = bi.n > 1 ? bi.n - 1 : 1u;
    a.tri_limit          = bi.n;
    if (bi.kind == kKindScene)
    {
        SceneTraceArgs sa;
        sa.base       = a;
        sa.base.empty = bi.n == 0;
        sa.xforms     = reinterpret_cast<const float*>(bvh + bi.xforms_off);
        sa.inst       = reinterpret_cast<const InstanceDesc*>(bvh + bi.inst_off);
        sa.inst_count = bi.n;
        // AUTO: the persistent binary two-level kernel (fastest on incoherent
        // rays; the 8-wide BLAS kernel stays selectable as WIDE).
        sa.use_wide       = bi.scene_wide && trav == RR_CUDA_TRAVERSAL_WIDE;
        sa.use_persistent = trav == RR_CUDA_TRAVERSAL_AUTO || trav == RR_CUDA_TRAVERSAL_BINARY_PERSISTENT;
        sa.use_bvh4       = bi.scene_bvh4 && trav == RR_CUDA_TRAVERSAL_BVH4;
        sa.bvh4_q8        = bi.scene_bvh4_q8 ? 1 : 0;
        if (sp) return Op();
        return [=](cudaStream_t s) { return launch_trace_scene(sa, s); };
    }
    // Geometry (registered) or an unknown buffer, traversed as binary nodes
    // from the root like the reference (vlk/intersector.cpp:290).
    a.empty             = (bi.kind == kKindGeom && bi.n == 0);
    const bool has_wide = bi.kind == kKindGeom && bi.format == RR_CUDA_NODE_FORMAT_WIDE8 && bi.n > 0;
    // AUTO: the 4-wide kernel on a triangle geometry with 4-wide nodes (the
    // default format; the fastest kernel on incoherent rays), else the
    // persistent binary kernel (bit-identical to BINARY);
    // rrCudaAutotuneTraversal refines the choice per workload.
    // With the precise test, fp32 and quantised 4-wide nodes take the robust
    // box test (trace_bvh4.cuh).
    const bool has_bvh4 = bi.kind == kKindGeom && is_bvh4_format(bi.format) && bi.n > 0 &&
                          bi.prim_kind == kPrimTriangles;
    if (trav == RR_CUDA_TRAVERSAL_BINARY_PERSISTENT || (trav == RR_CUDA_TRAVERSAL_AUTO && !has_bvh4))
    {
        if (sp)
        {
            if (a.collect_stats || a.indirect) return Op();
            a.stream_words      = sp->words;
            a.stream_late       = sp->late;
            a.stream_shift      = sp->shift;
            a.stream_chunks     = sp->chunks;
            a.stream_part_shift = sp->part_shift;
            a.stream_parts      = sp->parts;
            a.scratch_bytes     = sp->scratch_bytes;
        }
        return [=](cudaStream_t s) { return launch_trace_persistent(a, s); };
    }
    if ((trav == RR_CUDA_TRAVERSAL_BVH4 || trav == RR_CUDA_TRAVERSAL_AUTO) && has_bvh4)
    {
        a.bvh4_nodes = reinterpret_cast<const Bvh4Node*>(bvh + bi.wide_off);
        a.bvh4_q8    = bi.format == RR_CUDA_NODE_FORMAT_BVH4Q8 ? 1 : 0;
        a.wide_limit = (uint32_t)bi.wide_capacity;
        if (sp)
        {
            if (a.collect_stats || a.indirect) return Op();
            a.stream_words      = sp->words;
            a.stream_late       = sp->late;
            a.stream_shift      = sp->shift;
            a.stream_chunks     = sp->chunks;
            a.stream_part_shift = sp->part_shift;
            a.stream_parts      = sp->parts;
            a.scratch_bytes     = sp->scratch_bytes;
        }
        return [=](cudaStream_t s) { return launch_trace_bvh4(a, s); };
    }
    if (sp) return Op();
    if (has_wide && trav == RR_CUDA_TRAVERSAL_WIDE)
    {
        a.wide_nodes = reinterpret_cast<const WideNode*>(bvh + bi.wide_off);
        a.wide_tris  = reinterpret_cast<const WideTri*>(bvh + bi.tris_off);
        a.bounds     = reinterpret_cast<const uint32_t*>(bvh + bi.trailer_off + offsetof(Trailer, bounds));
        return [=](cudaStream_t s) { return launch_trace_wide(a, s); };
    }
    return [=](cudaStream_t s) { return launch_trace_binary(a, s); };
}

// Host-buffer trace as one persistent launch over all rays (empty Op when the
// plan does not apply: fewer than 2^16 rays, no stream memory operations, a
// host hit buffer the device cannot write, or a traversal other than the
// persistent binary or 4-wide kernel).  On stream s:
//   s:        clear the words, fork;
//   pipe[0]:  per chunk, copy its rays in, then set its arrival flag;
//   s:        the streamed kernel (waits, bounded, for each chunk's flag);
//   pipe[1]:  per part (eight chunks), wait until its done counter reaches
//             the part's size, then copy its hits out; then wait for the
//             kernel and scatter the late-listed hits (launch_late_scatter)
//             over the parts' copies;
//   s:        join both side streams.
// Everything is enqueued after what it depends on, so even side streams that
// share one hardware queue with s only serialise.  The copy-out waits are
// enqueued only after the kernel launched, and the kernel counts every ray
// of every part (traced, a miss after a failed wait, or late-listed), so
// each wait ends.
// Measured on the 16.8 M-ray heightfield: when parts were counted by
// finished rays instead, they completed 1.5-2 ms after their rays were
// claimed (their slowest rays), and a quarter of the hits were still to copy
// when the kernel ended.
Op streamed_host_trace(Context* ctx, uint8_t* bvh, int query, const uint8_t* host_rays, uint32_t ray_count, int output,
                       uint8_t* host_hits, uint8_t* dr, uint8_t* dh, uint8_t* sc, size_t scratch_total,
                       uint32_t chunk_rays)
{
    if (ray_count < (1u << 16) || !memops_ok(ctx)) return Op();
    // The late scatter writes the host hit buffer from a kernel, so the plan
    // needs it device-accessible (page-locked or registered memory).
    cudaPointerAttributes pa{};
    uint8_t*              hh_dev = nullptr;
    if (cudaPointerGetAttributes(&pa, host_hits) == cudaSuccess && pa.type == cudaMemoryTypeHost && pa.devicePointer)
        hh_dev = static_cast<uint8_t*>(pa.devicePointer);
    cudaGetLastError();
    if (!hh_dev) return Op();
    // Copy-in chunks: 2^17 rays by default (4 MiB; the first one is the wait
    // before the kernel starts).  Copy-out parts: eight chunks (16 MiB of full
    // hits), so that each warp publishes few counts and late-lists few rays.
    // (Measured on the 16.8 M-ray heightfield: 2^16 / 2^17 / 2^18-ray chunks
    // with 2^20-ray parts gave 3,241 / 3,517 / 3,508 Mrays/s end to end;
    // parts of two / four / eight chunks 3,145 / 3,465 / 3,500.)
    uint32_t shift = 17;
    if (chunk_rays)
        for (shift = 12; shift < 24 && (2u << shift) <= chunk_rays;) ++shift;
    StreamPlan sp;
    sp.shift            = shift;
    sp.chunks           = (uint32_t)(((uint64_t)ray_count + (1ull << shift) - 1) >> shift);
    sp.part_shift       = shift + 3;
    sp.parts            = (uint32_t)(((uint64_t)ray_count + (1ull << sp.part_shift) - 1) >> sp.part_shift);
    const size_t wbytes = stream_words_bytes(sp.chunks, sp.parts);
    const size_t woff   = (scratch_total - wbytes) / kAlign * kAlign;
    sp.words            = reinterpret_cast<uint32_t*>(sc + woff);
    // The late list: 4 bytes per ray below the words; the spill stacks keep
    // the rest (trace_scratch_bytes gives 256 bytes per ray).
    const size_t lbytes = (size_t)ray_count * sizeof(uint32_t);
    if (woff < lbytes + 2 * kAlign) return Op();  // room for the list and the kernel's 256-byte header
    const size_t loff = (woff - lbytes) / kAlign * kAlign;
    sp.late           = reinterpret_cast<uint32_t*>(sc + loff);
    sp.scratch_bytes  = loff;
    Op tr = trace_op(ctx, bvh, dr, ray_count, nullptr, dh, sc, query, output, ctx->topts, &sp);
    if (!tr) return Op();
    const auto     wr = reinterpret_cast<PfnStreamValue32>(ctx->write_value);
    const auto     wt = reinterpret_cast<PfnStreamValue32>(ctx->wait_value);
    cudaStream_t   in = ctx->pipe[0], out = ctx->pipe[1];
    cudaEvent_t    fork = ctx->pipe_fork, j_in = ctx->pipe_join[0], j_out = ctx->pipe_join[1];
    cudaEvent_t    kdone = ctx->pipe_kdone;
    uint32_t*      words = sp.words;
    uint32_t*      late  = sp.late;
    const int      sms   = ctx->sm_count;
    const uint32_t nch = sp.chunks, nparts = sp.parts, pshift = sp.part_shift;
    const uint32_t drop = ctx->drop_arrival;  // test hook: this chunk's flag is never raised
    const size_t   hs  = output == RR_INTERSECT_QUERY_OUTPUT_FULL_HIT ? 16 : 4;
    return [=](cudaStream_t s) -> cudaError_t {
        cudaError_t e = cudaMemsetAsync(words, 0, wbytes, s);
        if (e == cudaSuccess) e = cudaEventRecord(fork, s);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(in, fork, 0);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(out, fork, 0);
        if (e != cudaSuccess) return e;
        for (uint32_t c = 0; c < nch && e == cudaSuccess; ++c)
        {
            const uint64_t off = (uint64_t)c << shift;
            const uint64_t n   = std::min<uint64_t>(1ull << shift, ray_count - off);
            e = cudaMemcpyAsync(dr + 32 * off, host_rays + 32 * off, 32 * n, cudaMemcpyHostToDevice, in);
            if (e == cudaSuccess && c != drop &&
                wr((CUstream)in, (CUdeviceptr)(uintptr_t)(words + c), 1u, CU_STREAM_WRITE_VALUE_DEFAULT) != CUDA_SUCCESS)
                e = cudaErrorUnknown;
        }
        if (e == cudaSuccess) e = tr(s);
        const bool launched = e == cudaSuccess;
        if (launched) e = cudaEventRecord(kdone, s);
        for (uint32_t p = 0; launched && p < nparts && e == cudaSuccess; ++p)
        {
            const uint64_t off = (uint64_t)p << pshift;
            const uint64_t n   = std::min<uint64_t>(1ull << pshift, ray_count - off);
            if (wt((CUstream)out, (CUdeviceptr)(uintptr_t)(words + nch + p), (cuuint32_t)n, CU_STREAM_WAIT_VALUE_GEQ) !=
                CUDA_SUCCESS)
                e = cudaErrorUnknown;
            else
                e = cudaMemcpyAsync(host_hits + hs * off, dh + hs * off, hs * n, cudaMemcpyDeviceToHost, out);
        }
        // The late-listed hits, after every part's copy and after the kernel.
        if (launched && e == cudaSuccess) e = cudaStreamWaitEvent(out, kdone, 0);
        if (launched && e == cudaSuccess)
            e = launch_late_scatter(words + nch + nparts + 1, late, ray_count, dh, hh_dev, (uint32_t)hs, sms, out);
        cudaError_t j = cudaEventRecord(j_in, in);
        if (j == cudaSuccess) j = cudaStreamWaitEvent(s, j_in, 0);
        if (j == cudaSuccess) j = cudaEventRecord(j_out, out);
        if (j == cudaSuccess) j = cudaStreamWaitEvent(s, j_out, 0);
        return e != cudaSuccess ? e : j;
    };
}
}  // namespace

namespace
{
// The traversal autotuner (rrCudaAutotuneTraversal) on a device buffer.
// With use_cache false the cached decision is ignored and every candidate is
// timed again; *best_ms (optional) receives the winner's time per launch
// (negative when the decision came from the cache).  Throws CudaFail.
RRError autotune_traversal(Context* ctx, uint8_t* bvh, RRIntersectQuery query, uint8_t* rays_p, uint32_t ray_count,
                           RRIntersectQueryOutput query_output, uint8_t* hits_p, uint8_t* scratch_p, bool use_cache,
                           RRCudaTraversalOptions* chosen, float* best_ms_out)
{
    if (best_ms_out) *best_ms_out = -1.f;
    {
        auto        it  = ctx->registry.find((uintptr_t)bvh);
        BufInfo     bi;
        if (it != ctx->registry.end()) bi = it->second;
        const bool has_wide = (bi.kind == kKindGeom && bi.format == RR_CUDA_NODE_FORMAT_WIDE8 && bi.n > 0) ||
                              (bi.kind == kKindScene && bi.scene_wide);
        // Workload key: device, buffer kind, node format and size, query,
        // output, ray-count octave (the format decides the candidates).
        uint32_t octave = 0;
        while ((1ull << (octave + 1)) <= ray_count) ++octave;
        const uint32_t tt = ctx->topts.triangle_test;
        if (precise_unsupported(ctx, bvh)) return RR_ERROR_NOT_IMPLEMENTED;
        const std::string key = ctx->gpu_name + "|" + std::to_string(bi.kind) + "|" + std::to_string(bi.format) +
                                "|" + std::to_string(bi.n) + "|" + std::to_string((int)query) + "|" +
                                std::to_string((int)query_output) + "|" + std::to_string(octave) +
                                (tt ? "|t" + std::to_string(tt) : std::string());
        auto hit = use_cache ? ctx->tuned.find(key) : ctx->tuned.end();
        const char* cache_path = std::getenv("RR_CUDA_TUNE_CACHE");
        if (use_cache && hit == ctx->tuned.end() && cache_path)
        {
            if (FILE* f = std::fopen(cache_path, "r"))
            {
                char     line[512];
                while (std::fgets(line, sizeof(line), f))
                {
                    char*    tab = std::strchr(line, '\t');
                    unsigned t = 0, ro = 0, bps = 0, depth = 0;
                    if (!tab) continue;
                    *tab = 0;
                    if (key == line && std::sscanf(tab + 1, "%u %u %u %u", &t, &ro, &bps, &depth) >= 3)
                    {
                        RRCudaTraversalOptions o{};
                        o.struct_size   = sizeof(o);
                        o.traversal     = t;
                        o.ray_order     = ro;
                        o.blocks_per_sm = bps;
                        o.short_stack   = depth;
                        o.triangle_test = tt;
                        ctx->tuned[key] = o;
                    }
                }
                std::fclose(f);
            }
            hit = ctx->tuned.find(key);
        }
        if (hit == ctx->tuned.end())
        {
            std::vector<RRCudaTraversalOptions> cand;
            // The precise test runs in the persistent kernels only.
            auto add = [&](uint32_t trav, uint32_t order) {
                if (tt && trav != RR_CUDA_TRAVERSAL_BINARY_PERSISTENT && trav != RR_CUDA_TRAVERSAL_BVH4) return;
                RRCudaTraversalOptions o{};
                o.struct_size   = sizeof(o);
                o.traversal     = trav;
                o.ray_order     = order;
                o.triangle_test = tt;
                cand.push_back(o);
            };
            add(RR_CUDA_TRAVERSAL_BINARY, 0);
            add(RR_CUDA_TRAVERSAL_BINARY_PERSISTENT, 0);
            if ((bi.kind == kKindGeom && is_bvh4_format(bi.format) && bi.n > 0 &&
                 bi.prim_kind == kPrimTriangles) ||
                (bi.kind == kKindScene && bi.scene_bvh4))
                add(RR_CUDA_TRAVERSAL_BVH4, 0);
            if (has_wide)
            {
                add(RR_CUDA_TRAVERSAL_WIDE, 1);
                if (bi.kind == kKindGeom && ray_count >= (1u << 20)) add(RR_CUDA_TRAVERSAL_WIDE, 2);
            }
            cudaEvent_t e0, e1;
            check(cudaEventCreate(&e0), "event");
            check(cudaEventCreate(&e1), "event");
            float best_ms = 1e30f;
            RRCudaTraversalOptions best = cand[0];
            auto try_cand = [&](const RRCudaTraversalOptions& o, float margin) {
                Op op = trace_op(ctx, bvh, rays_p, ray_count, nullptr, hits_p, scratch_p, query, query_output, o);
                check(op(ctx->stream), "tune warm-up");
                check(cudaEventRecord(e0, ctx->stream), "event");
                for (int r = 0; r < 3; ++r) check(op(ctx->stream), "tune run");
                check(cudaEventRecord(e1, ctx->stream), "event");
                check(cudaEventSynchronize(e1), "event");
                float ms = 0.f;
                check(cudaEventElapsedTime(&ms, e0, e1), "event");
                RR_LOG_INFO("autotune %s: traversal %u order %u blocks/SM %u stack %u -> %.3f ms", key.c_str(),
                            o.traversal, o.ray_order, o.blocks_per_sm, o.short_stack, ms / 3.f);
                if (ms < best_ms * margin)
                {
                    best_ms = ms;
                    best    = o;
                }
            };
            // Stage 1: kernel and node width.  Stage 2: the winner's launch
            // shape (resident blocks per SM, against the occupancy maximum)
            // and, for the 4-wide kernel, its shared-stack depth; a stage-2
            // variant must be 1 % faster to replace the default shape, so
            // run-to-run noise does not move it.
            for (const auto& o : cand) try_cand(o, 1.0f);
            const RRCudaTraversalOptions w = best;
            if (w.traversal != RR_CUDA_TRAVERSAL_BINARY)
                for (uint32_t bps : {4u, 6u})
                {
                    RRCudaTraversalOptions o = w;
                    o.blocks_per_sm          = bps;
                    try_cand(o, 0.99f);
                }
            if (w.traversal == RR_CUDA_TRAVERSAL_BVH4 && bi.kind == kKindGeom)
                for (uint32_t depth : {12u, 24u})
                {
                    RRCudaTraversalOptions o = w;
                    o.short_stack            = depth;
                    try_cand(o, 0.99f);
                }
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            if (best_ms_out) *best_ms_out = best_ms / 3.f;
            ctx->tuned[key] = best;
            if (cache_path)
                if (FILE* f = std::fopen(cache_path, "a"))
                {
                    std::fprintf(f, "%s\t%u %u %u %u\n", key.c_str(), best.traversal, best.ray_order,
                                 best.blocks_per_sm, best.short_stack);
                    std::fclose(f);
                }
            hit = ctx->tuned.find(key);
        }
        RRCudaTraversalOptions o = hit->second;
        o.collect_stats          = 0;
        ctx->topts               = o;
        if (chosen) *chosen = o;
        return RR_SUCCESS;
    }
}

}  // namespace

extern "C" {

RR_API RRError rrSetLogLevel(RRLogLevel log_level)
{
    if (log_level < RR_LOG_LEVEL_DEBUG || log_level > RR_LOG_LEVEL_OFF) return RR_ERROR_INVALID_PARAMETER;
    g_log_level = log_level;
    RR_LOG_INFO("rrSetLogLevel(%d)", (int)log_level);
    return RR_SUCCESS;
}

RR_API RRError rrSetLogFile(char const* filename)
{
    if (!filename) return RR_ERROR_INVALID_PARAMETER;
    FILE* f = std::fopen(filename, "a");
    if (!f) return RR_ERROR_INTERNAL;
    std::lock_guard<std::mutex> lk(g_log_mu);
    if (g_log_file) std::fclose(g_log_file);
    g_log_file = f;
    return RR_SUCCESS;
}

RR_API RRError rrCreateContext(uint32_t api_version, RRApi api, RRContext* context)
{
    RR_LOG_INFO("rrCreateContext(%u)", api_version);
    if (!context) return RR_ERROR_INVALID_PARAMETER;
    if (api != RR_API_CUDA) return RR_ERROR_UNSUPPORTED_API;
    RR_TRY({
        int count = 0;
        if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
        {
            cudaGetLastError();
            RR_LOG_ERROR("no CUDA device");
            return RR_ERROR_INTERNAL;
        }
        std::unique_ptr<Context> c(new Context);
        check(cudaGetDevice(&c->device), "cudaGetDevice");
        check(cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, c->device), "sm count");
        {
            cudaDeviceProp prop{};
            check(cudaGetDeviceProperties(&prop, c->device), "device properties");
            c->gpu_name = prop.name;
        }
        check(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "stream");
        check(cudaMalloc(&c->words, sizeof(DeviceWords)), "cudaMalloc words");
        check(cudaMemset(c->words, 0, sizeof(DeviceWords)), "memset words");
        c->topts.struct_size = sizeof(RRCudaTraversalOptions);
        c->topts.traversal   = RR_CUDA_TRAVERSAL_AUTO;
        const char* g        = std::getenv("RR_CUDA_GRAPHS");
        c->graphs            = !(g && g[0] == '0');
        const char* fb       = std::getenv("RR_CUDA_FUSE_BUILDS");
        c->fuse_builds       = !(fb && fb[0] == '0');
        const char* sr       = std::getenv("RR_CUDA_STREAM_RAYS");
        c->stream_rays       = !(sr && sr[0] == '0');
        *context             = reinterpret_cast<RRContext>(c.release());
        return RR_SUCCESS;
    })
}

RR_API RRError rrDestroyContext(RRContext context)
{
    if (!context) return RR_ERROR_INVALID_PARAMETER;
    RR_TRY({
        DeviceGuard g(C(context)->device);
        delete C(context);
        return RR_SUCCESS;
    })
}

RR_API RRError rrGetGeometryBuildMemoryRequirements(RRContext                   context,
                                                    const RRGeometryBuildInput* build_input,
                                                    const RRBuildOptions*       build_options,
                                                    RRMemoryRequirements*       memory_requirements)
{
    if (!context || !build_input || !memory_requirements) return RR_ERROR_INVALID_PARAMETER;
    RR_TRY({
        MeshArgs ma;
        RRError  e = geometry_source(build_input, false, &ma);
        if (e != RR_SUCCESS) return e;
        BuildParams bp;
        if (!parse_build_options(build_options, bp)) return RR_ERROR_INVALID_PARAMETER;
        if (bp.format == RR_CUDA_NODE_FORMAT_AUTO)
        {
            // Sized for either node width the tuner may pick.
            const GeomLayout a = geom_layout(ma.n, build_format(ma, RR_CUDA_NODE_FORMAT_BVH4), bp.bits);
            const GeomLayout b = geom_layout(ma.n, build_format(ma, RR_CUDA_NODE_FORMAT_WIDE8), bp.bits);
            const GeomLayout c = geom_layout(ma.n, build_format(ma, RR_CUDA_NODE_FORMAT_BVH4Q8), bp.bits);
            memory_requirements->result_buffer_size           = std::max({a.total, b.total, c.total});
            memory_requirements->temporary_build_buffer_size  = std::max({a.s_total, b.s_total, c.s_total});
            memory_requirements->temporary_update_buffer_size = std::max({a.u_total, b.u_total, c.u_total});
            return RR_SUCCESS;
        }
        GeomLayout L                                      = geom_layout(ma.n, build_format(ma, bp.format), bp.bits);
        memory_requirements->result_buffer_size           = L.total;
        memory_requirements->temporary_build_buffer_size  = L.s_total;
        memory_requirements->temporary_update_buffer_size = L.u_total;
        return RR_SUCCESS;
    })
}

namespace
{
// RR_BUILD_OPERATION_UPDATE (reference vlk/intersector.cpp:178-201,
// vlk/update_hlbvh.cpp:140-180): the buffer must hold a build of a mesh with
// the same triangle count on this context; its node format and key width are
// kept.  The binary format needs no scratch; WIDE8 needs u_total bytes.
RRError record_update(Context* ctx, const RRGeometryBuildInput* in, RRDevicePtr temporary_buffer,
                      RRDevicePtr geometry_buffer, CommandStream* cs)
{
    MeshArgs ma;
    RRError  e = geometry_source(in, true, &ma);
    if (e != RR_SUCCESS) return e;
    if (!geometry_buffer) return RR_ERROR_INVALID_PARAMETER;
    uint8_t* result = P(geometry_buffer)->addr();
    auto     it     = ctx->registry.find((uintptr_t)result);
    if (it == ctx->registry.end() || it->second.kind != kKindGeom || it->second.n != ma.n ||
        it->second.prim_kind != ma.prim_kind)
        return RR_ERROR_INVALID_PARAMETER;
    uint32_t bits = 30;
    // The key width is not needed by an update (no Morton codes); the layout
    // only depends on it for scratch offsets that an update does not use.
    const GeomLayout L = geom_layout(ma.n, it->second.format, bits);
    if (L.u_total > 0 && !temporary_buffer) return RR_ERROR_INVALID_PARAMETER;
    uint8_t*     scratch = temporary_buffer ? P(temporary_buffer)->addr() : nullptr;
    DeviceWords* words   = ctx->words;
    const int    sms     = ctx->sm_count;
    record(cs, [=](cudaStream_t s) { return launch_update_mesh(ma, L, scratch, result, words, sms, s); });
    return RR_SUCCESS;
}
}  // namespace

RR_API RRError rrCmdBuildGeometry(RRContext                   context,
                                  RRBuildOperation            build_operation,
                                  const RRGeometryBuildInput* build_input,
                                  const RRBuildOptions*       build_options,
                                  RRDevicePtr                 temporary_buffer,
                                  RRDevicePtr                 geometry_buffer,
                                  RRCommandStream             command_stream)
{
    RR_LOG_INFO("rrCmdBuildGeometry");
    if (!context || !command_stream || !build_input) return RR_ERROR_INVALID_PARAMETER;
    RR_TRY({
        if (build_operation == RR_BUILD_OPERATION_UPDATE)
        {
            Context*    ctx = C(context);
            DeviceGuard g(ctx->device);
            return record_update(ctx, build_input, temporary_buffer, geometry_buffer, S(command_stream));
        }
        if (build_operation != RR_BUILD_OPERATION_BUILD) return RR_ERROR_INVALID_PARAMETER;
        BuildParams bp;
        if (!parse_build_options(build_options, bp)) return RR_ERROR_INVALID_PARAMETER;
        Context*    ctx = C(context);
        DeviceGuard g(ctx->device);
        PendingGeom pg;
        RRError     e = prepare_geometry(ctx, build_input, bp, temporary_buffer, geometry_buffer, &pg);
        if (e != RR_SUCCESS) return e;
        record_build(S(command_stream), pg);
        register_geometry(ctx, pg);
        return RR_SUCCESS;
    })
}

RR_API RRError rrCudaRegisterGeometry(RRContext context, RRDevicePtr geometry_buffer, uint32_t triangle_count)
{
    RR_LOG_INFO("rrCudaRegisterGeometry(%u)", triangle_count);
    if (!context || !geometry_buffer || triangle_count >= (1u << 30)) return RR_ERROR_INVALID_PARAMETER;
    RR_TRY({
        Context*       ctx    = C(context);
        DeviceGuard    g(ctx->device);
        uint8_t*       result = P(geometry_buffer)->addr();
        const uint32_t n      = triangle_count;
        const size_t   toff   = align_up(n == 0 ? 0 : (2ull * n - 1) * sizeof(BvhNode), kAlign);
        Trailer        t{};
        check(cudaMemcpy(&t, result + toff, sizeof(Trailer), cudaMemcpyDeviceToHost), "read trailer");
        if (t.magic != kMagic || t.version != kVersion || t.kind != kKindGeom || t.leaf_count != n ||
            t.node_count != (n == 0 ? 0u : 2u * n - 1u))
            return RR_ERROR_INVALID_PARAMETER;
        if (t.node_format != RR_CUDA_NODE_FORMAT_BINARY && t.node_format != RR_CUDA_NODE_FORMAT_WIDE8 &&
            !is_bvh4_format(t.node_format))
            return RR_ERROR_INVALID_PARAMETER;
        const GeomLayout L = geom_layout(n, t.node_format, t.morton_bits);
        if (t.wide_nodes_off != L.wide_off || t.wide_tris_off != L.tris_off) return RR_ERROR_INVALID_PARAMETER;
        if (t.prim_kind != kPrimTriangles && t.prim_kind != kPrimAabbs) return RR_ERROR_INVALID_PARAMETER;
        PendingGeom pg{};
        pg.L            = L;
        pg.result       = result;
        pg.ma.prim_kind = t.prim_kind;
        register_geometry(ctx, pg);
        return RR_SUCCESS;
    })
}

RR_API RRError rrCudaCmdBuildGeometries(RRContext                   context,
                                        uint32_t                    count,
                                        const RRGeometryBuildInput* build_inputs,
                                        const RRBuildOptions*       build_options,
                                        const RRDevicePtr*          temporary_buffers,
                                        const RRDevicePtr*          geometry_buffers,
                                        RRCommandStream             command_stream)
{
    RR_LOG_INFO("rrCudaCmdBuildGeometries(%u)", count);
    if (!context || !command_stream || (count > 0 && (!build_inputs || !temporary_buffers || !geometry_buffers)))
        return RR_ERROR_INVALID_PARAMETER;
    if (count == 0) return RR_SUCCESS;
    RR_TRY({
        BuildParams bp;
        if (!parse_build_options(build_options, bp)) return RR_ERROR_INVALID_PARAMETER;
        Context*                 ctx = C(context);
        DeviceGuard              g(ctx->device);
        std::vector<PendingGeom> geoms(count);
        RangeSet                 used;
        if (bp.format == RR_CUDA_NODE_FORMAT_AUTO)
        {
            // One node width for the whole fused build: the largest mesh's.
            uint32_t nmax = 0;
            for (uint32_t i = 0; i < count; ++i)
            {
                MeshArgs ma;
                RRError  e = geometry_source(build_inputs + i, false, &ma);
                if (e != RR_SUCCESS) return e;
                nmax = std::max(nmax, ma.n);
            }
            bp.format = resolve_format(ctx, RR_CUDA_NODE_FORMAT_AUTO, nmax);
        }
        for (uint32_t i = 0; i < count; ++i)
        {
            RRError e =
                prepare_geometry(ctx, build_inputs + i, bp, temporary_buffers[i], geometry_buffers[i], &geoms[i]);
            if (e != RR_SUCCESS) return e;
            if (!claim_build_ranges(used, geoms[i])) return RR_ERROR_INVALID_PARAMETER;
        }
        CommandStream* cs   = S(command_stream);
        bool           many = false;
        Op             op   = build_batch_op(ctx, geoms, &many);
        record(cs, std::move(op), many);
        cs->want_graph = cs->want_graph || many;
        for (const PendingGeom& pg : geoms) register_geometry(ctx, pg);
        return RR_SUCCESS;
    })
}

RR_API RRError rrGetSceneBuildMemoryRequirements(RRContext                context,
                                                 const RRSceneBuildInput* build_input,
                                                 const RRBuildOptions*    build_options,
                                                 RRMemoryRequirements*    memory_requirements)
{
    (void)build_options;
    if (!context || !build_input || !memory_requirements) return RR_ERROR_INVALID_PARAMETER;
    RR_TRY({
        SceneLayout L                                     = scene_layout(build_input->instance_count);
        memory_requirements->result_buffer_size           = L.total;
        memory_requirements->temporary_build_buffer_size  = L.s_total;
        memory_requirements->temporary_update_buffer_size = 0;
        return RR_SUCCESS;
    })
}

RR_API RRError rrCmdBuildScene(RRContext                context,
                               const RRSceneBuildInput* build_input,
                               const RRBuildOptions*    build_options,
                               RRDevicePtr              temporary_buffer,
                               RRDevicePtr              scene_buffer,
                               RRCommandStream          command_stream)
{
    (void)build_options;
    RR_LOG_INFO("rrCmdBuildScene");
    if (!context || !command_stream || !build_input) return RR_ERROR_INVALID_PARAMETER;
    RR_TRY({
        const uint32_t n = build_input->instance_count;
        if (n > 0 && !build_input->instances) return RR_ERROR_INVALID_PARAMETER;
        if (n >= (1u << 24)) return RR_ERROR_INVALID_PARAMETER;
        if (!scene_buffer || (!temporary_buffer && n > 0)) return RR_ERROR_INVALID_PARAMETER;
        Context*    ctx = C(context);
        DeviceGuard g(ctx->device);
        SceneLayout L = scene_layout(n);
        for (uint32_t i = 0; i < n; ++i)
            if (!build_input->instances[i].geometry) return RR_ERROR_INVALID_PARAMETER;
        // Host staging: [xforms 2n x 12 floats: inverse, forward][InstanceDesc n].
        const size_t xbytes = (size_t)n * 2 * 48, ibytes = (size_t)n * sizeof(InstanceDesc);
        auto         stage  = std::make_shared<PinnedBlock>(ctx->pinned, xbytes + ibytes);
        float*       xf     = reinterpret_cast<float*>(stage->p);
        InstanceDesc* id    = reinterpret_cast<InstanceDesc*>(reinterpret_cast<uint8_t*>(stage->p) + xbytes);
        bool          all_wide = n > 0;
        bool          all_bvh4 = n > 0;  // every instance 4-wide of one form (or empty)
        uint32_t      fmt4     = 0;
        for (uint32_t i = 0; i < n; ++i)
        {
            const RRInstance& in = build_input->instances[i];
            inverse34(&in.transform[0][0], xf + 24ull * i);
            std::memcpy(xf + 24ull * i + 12, &in.transform[0][0], 48);
            uint8_t* blas = P(in.geometry)->addr();
            auto     it   = ctx->registry.find((uintptr_t)blas);
            InstanceDesc d{};
            d.blas = (uint64_t)(uintptr_t)blas;
            if (it != ctx->registry.end() && it->second.kind == kKindGeom)
            {
                // Instances of AABB-list geometry are not supported by the
                // two-level kernels (their leaves are triangles).
                if (it->second.prim_kind == kPrimAabbs) return RR_ERROR_NOT_IMPLEMENTED;
                d.leaf_count = it->second.n;
                if (it->second.format == RR_CUDA_NODE_FORMAT_WIDE8 && it->second.n > 0)
                {
                    d.wide_nodes = (uint64_t)(uintptr_t)(blas + it->second.wide_off);
                    d.wide_tris  = (uint64_t)(uintptr_t)(blas + it->second.tris_off);
                }
                else
                    all_wide = false;
                if (is_bvh4_format(it->second.format) && it->second.n > 0 &&
                    (fmt4 == 0 || fmt4 == it->second.format))
                {
                    d.wide_nodes = (uint64_t)(uintptr_t)(blas + it->second.wide_off);  // its 4-wide nodes
                    fmt4         = it->second.format;
                }
                else if (it->second.n > 0)
                    all_bvh4 = false;
                d.flags = 1;  // known geometry
            }
            else
            {
                d.leaf_count = 0xffffffffu;  // unknown: traverse binary nodes from the root
                all_wide     = false;
                all_bvh4     = false;
            }
            id[i] = d;
        }
        uint8_t*     scratch = temporary_buffer ? P(temporary_buffer)->addr() : nullptr;
        uint8_t*     result  = P(scene_buffer)->addr();
        DeviceWords* words   = ctx->words;
        record(
            S(command_stream),
            [=](cudaStream_t s) -> cudaError_t {
            cudaError_t e = cudaSuccess;
            if (n > 0)
            {
                e = cudaMemcpyAsync(result + L.xforms_off, stage->p, xbytes, cudaMemcpyHostToDevice, s);
                if (e == cudaSuccess)
                    e = cudaMemcpyAsync(result + L.inst_off, reinterpret_cast<uint8_t*>(stage->p) + xbytes, ibytes,
                                        cudaMemcpyHostToDevice, s);
                if (e != cudaSuccess) return e;
            }
            SceneBuildArgs sa;
            sa.inst    = reinterpret_cast<const InstanceDesc*>(result + L.inst_off);
            sa.forward = reinterpret_cast<const float*>(result + L.xforms_off);
            sa.n       = n;
            return launch_build_scene(sa, L, scratch, result, words, s);
            },
            true);
        BufInfo bi;
        bi.kind        = kKindScene;
        bi.n           = n;
        bi.trailer_off = L.trailer_off;
        bi.xforms_off  = L.xforms_off;
        bi.inst_off    = L.inst_off;
        bi.scene_wide  = all_wide;
        bi.scene_bvh4  = all_bvh4;
        bi.scene_bvh4_q8 = all_bvh4 && fmt4 == RR_CUDA_NODE_FORMAT_BVH4Q8;
        ctx->registry[(uintptr_t)result] = bi;
        return RR_SUCCESS;
    })
}

RR_API RRError rrCmdIntersect(RRContext              context,
                              RRDevicePtr            scene_buffer,
                              RRIntersectQuery       query,
                              RRDevicePtr            rays,
                              uint32_t               ray_count,
                              RRDevicePtr            indirect_ray_count,
                              RRIntersectQueryOutput query_output,
                              RRDevicePtr            hits,
                              RRDevicePtr            scratch,
                              RRCommandStream        command_stream)
{
    RR_LOG_INFO("rrCmdIntersect");
    if (!context || !scene_buffer || !rays || !hits || !scratch || !command_stream) return RR_ERROR_INVALID_PARAMETER;
    if (query != RR_INTERSECT_QUERY_CLOSEST && query != RR_INTERSECT_QUERY_ANY) return RR_ERROR_INVALID_PARAMETER;
    if (query_output != RR_INTERSECT_QUERY_OUTPUT_FULL_HIT && query_output != RR_INTERSECT_QUERY_OUTPUT_INSTANCE_ID)
        return RR_ERROR_INVALID_PARAMETER;
    RR_TRY({
        Context*    ctx = C(context);
        DeviceGuard g(ctx->device);
        if (precise_unsupported(ctx, P(scene_buffer)->addr())) return RR_ERROR_NOT_IMPLEMENTED;
        const uint32_t* ind =
            indirect_ray_count ? reinterpret_cast<const uint32_t*>(P(indirect_ray_count)->addr()) : nullptr;
        record(S(command_stream), trace_op(ctx, P(scene_buffer)->addr(), P(rays)->addr(), ray_count, ind,
                                           P(hits)->addr(), P(scratch)->addr(), query, query_output, ctx->topts));
        return RR_SUCCESS;
    })
}

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
                                             RRCommandStream        command_stream)
{
    RR_LOG_INFO("rrCudaCmdIntersectHostBuffers");
    if (!context || !scene_buffer || !host_rays || !host_hits || !rays || !hits || !scratch || !command_stream ||
        !ray_count)
        return RR_ERROR_INVALID_PARAMETER;
    if (query != RR_INTERSECT_QUERY_CLOSEST && query != RR_INTERSECT_QUERY_ANY) return RR_ERROR_INVALID_PARAMETER;
    if (query_output != RR_INTERSECT_QUERY_OUTPUT_FULL_HIT && query_output != RR_INTERSECT_QUERY_OUTPUT_INSTANCE_ID)
        return RR_ERROR_INVALID_PARAMETER;
    RR_TRY({
        Context*    ctx = C(context);
        DeviceGuard g(ctx->device);
        if (precise_unsupported(ctx, P(scene_buffer)->addr())) return RR_ERROR_NOT_IMPLEMENTED;
        ctx->ensure_pipe();
        // Chunks go round-robin to the side streams; each stream owns an equal
        // share of the scratch (rrGetTraceMemoryRequirements(ray_count) bytes).
        const size_t   total = trace_scratch_bytes(ray_count);
        const int      np    = ray_count >= 3u * 8192u ? Context::kPipe : 1;
        const size_t   region = np == 1 ? total : total / np / kAlign * kAlign;
        const uint64_t fit    = np == 1 ? ray_count : (region - 256) / 256;
        uint64_t       chunk  = chunk_rays ? chunk_rays : (1u << 21);
        if (chunk > fit) chunk = fit;
        if (chunk > ray_count) chunk = ray_count;
        const size_t hs = query_output == RR_INTERSECT_QUERY_OUTPUT_FULL_HIT ? 16 : 4;
        std::vector<Op> chunks;
        std::vector<int> lane;
        uint8_t*        bvh = P(scene_buffer)->addr();
        uint8_t*        dr  = P(rays)->addr();
        uint8_t*        dh  = P(hits)->addr();
        uint8_t*        sc  = P(scratch)->addr();
        int             k   = 0;
        for (uint64_t off = 0; off < ray_count; off += chunk, ++k)
        {
            const uint32_t n = (uint32_t)std::min<uint64_t>(chunk, ray_count - off);
            const int      p = k % np;
            Op             tr = trace_op(ctx, bvh, dr + 32 * off, n, nullptr, dh + hs * off, sc + (size_t)p * region, query,
                                         query_output, ctx->topts);
            const uint8_t* hr = reinterpret_cast<const uint8_t*>(host_rays) + 32 * off;
            uint8_t*       hh = reinterpret_cast<uint8_t*>(host_hits) + hs * off;
            uint8_t*       r  = dr + 32 * off;
            uint8_t*       h  = dh + hs * off;
            chunks.push_back([=](cudaStream_t st) -> cudaError_t {
                cudaError_t e = cudaMemcpyAsync(r, hr, 32ull * n, cudaMemcpyHostToDevice, st);
                if (e == cudaSuccess) e = tr(st);
                if (e == cudaSuccess) e = cudaMemcpyAsync(hh, h, hs * n, cudaMemcpyDeviceToHost, st);
                return e;
            });
            lane.push_back(p);
        }
        cudaStream_t side[Context::kPipe];
        cudaEvent_t  join[Context::kPipe];
        for (int p = 0; p < Context::kPipe; ++p)
        {
            side[p] = ctx->pipe[p];
            join[p] = ctx->pipe_join[p];
        }
        cudaEvent_t fork = ctx->pipe_fork;
        Op          chunked = [=](cudaStream_t s) -> cudaError_t {
            cudaError_t e = cudaSuccess;
            if (np == 1)
            {
                for (size_t i = 0; i < chunks.size() && e == cudaSuccess; ++i) e = chunks[i](s);
                return e;
            }
            e = cudaEventRecord(fork, s);
            for (int p = 0; p < np && e == cudaSuccess; ++p) e = cudaStreamWaitEvent(side[p], fork, 0);
            for (size_t i = 0; i < chunks.size() && e == cudaSuccess; ++i) e = chunks[i](side[lane[i]]);
            for (int p = 0; p < np && e == cudaSuccess; ++p)
            {
                e = cudaEventRecord(join[p], side[p]);
                if (e == cudaSuccess) e = cudaStreamWaitEvent(s, join[p], 0);
            }
            return e;
        };
        Op streamed = streamed_host_trace(ctx, bvh, query, reinterpret_cast<const uint8_t*>(host_rays), ray_count,
                                          query_output, reinterpret_cast<uint8_t*>(host_hits), dr, dh, sc, total,
                                          chunk_rays);
        // The streamed plan runs unless the stream is being captured into a
        // graph (its stream memory operations order work in a way a graph
        // does not see); the chunked plan is the fallback.
        record(S(command_stream), [=](cudaStream_t s) -> cudaError_t {
            if (streamed)
            {
                cudaStreamCaptureStatus cap = cudaStreamCaptureStatusActive;
                if (cudaStreamIsCapturing(s, &cap) == cudaSuccess && cap == cudaStreamCaptureStatusNone)
                    return streamed(s);
                cudaGetLastError();
            }
            return chunked(s);
        });
        return RR_SUCCESS;
    })
}

RR_API RRError rrGetTraceMemoryRequirements(RRContext context, uint32_t ray_count, size_t* scratch_size)
{
    if (!context || !scratch_size || !ray_count) return RR_ERROR_INVALID_PARAMETER;
    *scratch_size = trace_scratch_bytes(ray_count);
    return RR_SUCCESS;
}

RR_API RRError rrCudaGetIntersectBatchMemoryRequirements(RRContext context, uint32_t request_count,
                                                         uint32_t total_ray_count, size_t* scratch_size)
{
    if (!context || !scratch_size || !request_count) return RR_ERROR_INVALID_PARAMETER;
    *scratch_size = batch_trace_layout(request_count, total_ray_count).total;
    return RR_SUCCESS;
}

namespace
{
// One request of a multi-request launch, resolved to device addresses.
struct DevRequest
{
    uint8_t*               bvh;
    RRIntersectQuery       query;
    RRIntersectQueryOutput output;
    uint8_t*               rays;
    uint32_t               ray_count;
    uint8_t*               hits;
};

// The op of one multi-request launch: the request table and ray prefix are
// staged in pinned host memory (owned by the op) and copied into the scratch
// before the persistent launch.
RRError batch_trace_op(Context* ctx, const std::vector<DevRequest>& dq, uint8_t* sc, Op* out)
{
    const uint32_t         count = (uint32_t)dq.size();
    const BatchTraceLayout L0    = batch_trace_layout(count, 0);
    const size_t           pre   = ((size_t)count + 1) * sizeof(uint32_t);
    const size_t           gap   = L0.prefix_off - L0.req_off;
    auto                   stage = std::make_shared<PinnedBlock>(ctx->pinned, gap + pre);
    BatchTraceReq*         rq    = reinterpret_cast<BatchTraceReq*>(stage->p);
    uint32_t*              pf    = reinterpret_cast<uint32_t*>(reinterpret_cast<uint8_t*>(stage->p) + gap);
    std::memset(stage->p, 0, gap + pre);
    uint64_t total = 0;
    // The 4-wide kernel when the traversal option allows it and every request
    // with rays has a triangle geometry with 4-wide nodes (or none at all).
    // The 4-wide nodes must all have the same form (fp32 or 8-bit bounds).
    const uint32_t trav = ctx->topts.traversal;
    bool           use4 = trav == RR_CUDA_TRAVERSAL_AUTO || trav == RR_CUDA_TRAVERSAL_BVH4;
    uint32_t       fmt4 = 0;
    for (uint32_t k = 0; k < count && use4; ++k)
    {
        auto it = ctx->registry.find((uintptr_t)dq[k].bvh);
        if (it == ctx->registry.end())
        {
            use4 = dq[k].ray_count == 0;
            continue;
        }
        const BufInfo& b = it->second;
        if (b.kind != kKindGeom)
        {
            use4 = false;
            continue;
        }
        if (b.n == 0 || dq[k].ray_count == 0) continue;
        use4 = is_bvh4_format(b.format) && (fmt4 == 0 || fmt4 == b.format) && b.prim_kind == kPrimTriangles &&
               b.wide_off % 256 == 0 && b.wide_off / 256 <= 0xffffffffull;
        fmt4 = b.format;
    }
    for (uint32_t k = 0; k < count; ++k)
    {
        const DevRequest& q = dq[k];
        if (q.query != RR_INTERSECT_QUERY_CLOSEST && q.query != RR_INTERSECT_QUERY_ANY)
            return RR_ERROR_INVALID_PARAMETER;
        if (q.output != RR_INTERSECT_QUERY_OUTPUT_FULL_HIT && q.output != RR_INTERSECT_QUERY_OUTPUT_INSTANCE_ID)
            return RR_ERROR_INVALID_PARAMETER;
        auto    it = ctx->registry.find((uintptr_t)q.bvh);
        BufInfo bi;
        if (it != ctx->registry.end()) bi = it->second;
        if (bi.kind == kKindScene) return RR_ERROR_NOT_IMPLEMENTED;
        BatchTraceReq r{};
        r.bvh        = q.bvh;
        r.rays       = q.ray_count ? q.rays : nullptr;
        r.hits       = q.ray_count ? q.hits : nullptr;
        r.ray_count  = q.ray_count;
        r.node_limit = bi.kind == 0 ? kInvalid : (bi.n == 0 ? 0u : 2u * bi.n - 1u);
        r.flags      = (q.query == RR_INTERSECT_QUERY_ANY ? kReqAny : 0u) |
                  (q.output == RR_INTERSECT_QUERY_OUTPUT_FULL_HIT ? kReqFull : 0u) |
                  (bi.kind == kKindGeom && bi.n == 0 ? kReqEmpty : 0u) |
                  (bi.kind == kKindGeom && bi.prim_kind == kPrimAabbs ? kReqBoxes : 0u);
        if (use4 && bi.kind == kKindGeom && bi.n > 0 && is_bvh4_format(bi.format))
        {
            r.flags |= kReqBvh4;
            r.wide_off256 = (uint32_t)(bi.wide_off / 256);
            r.wide_limit  = (uint32_t)bi.wide_capacity;
        }
        rq[k] = r;
        pf[k] = (uint32_t)total;
        total += q.ray_count;
        if (total >= 0xffffffffull) return RR_ERROR_INVALID_PARAMETER;
    }
    pf[count]                = (uint32_t)total;
    const BatchTraceLayout L = batch_trace_layout(count, total);
    BatchTraceArgs         a{};
    a.req              = reinterpret_cast<const BatchTraceReq*>(sc + L.req_off);
    a.prefix           = reinterpret_cast<const uint32_t*>(sc + L.prefix_off);
    a.count            = count;
    a.total            = (uint32_t)total;
    a.scratch          = sc;
    a.scratch_bytes    = L.total;
    a.spill_off        = L.spill_off;
    a.words            = ctx->words;
    a.sm_count         = ctx->sm_count;
    a.blocks_per_sm    = (int)ctx->topts.blocks_per_sm;
    a.collect_stats    = ctx->topts.collect_stats ? 1 : 0;
    a.use_bvh4         = use4 ? 1 : 0;
    a.bvh4_q8          = use4 && fmt4 == RR_CUDA_NODE_FORMAT_BVH4Q8 ? 1 : 0;
    const size_t bytes = gap + pre;
    *out               = [=](cudaStream_t s) -> cudaError_t {
        cudaError_t e = cudaMemcpyAsync(sc + L.req_off, stage->p, bytes, cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return e;
        return launch_trace_batch(a, s);
    };
    return RR_SUCCESS;
}
}  // namespace

RR_API RRError rrCudaCmdIntersectBatch(RRContext                     context,
                                       uint32_t                      request_count,
                                       const RRCudaIntersectRequest* requests,
                                       RRDevicePtr                   scratch,
                                       RRCommandStream               command_stream)
{
    RR_LOG_INFO("rrCudaCmdIntersectBatch(%u)", request_count);
    if (!context || !requests || !request_count || !scratch || !command_stream) return RR_ERROR_INVALID_PARAMETER;
    RR_TRY({
        Context*    ctx = C(context);
        DeviceGuard g(ctx->device);
        std::vector<DevRequest> dq(request_count);
        for (uint32_t k = 0; k < request_count; ++k)
        {
            const RRCudaIntersectRequest& q = requests[k];
            if (!q.geometry || (q.ray_count && (!q.rays || !q.hits))) return RR_ERROR_INVALID_PARAMETER;
            dq[k] = DevRequest{P(q.geometry)->addr(), q.query, q.output, q.ray_count ? P(q.rays)->addr() : nullptr,
                               q.ray_count, q.ray_count ? P(q.hits)->addr() : nullptr};
        }
        Op      op;
        RRError e = batch_trace_op(ctx, dq, P(scratch)->addr(), &op);
        if (e != RR_SUCCESS) return e;
        record(S(command_stream), std::move(op), true);
        return RR_SUCCESS;
    })
}

RR_API RRError rrCudaCmdIntersectBatchHost(RRContext                         context,
                                           uint32_t                          request_count,
                                           const RRCudaHostIntersectRequest* requests,
                                           RRDevicePtr                       rays,
                                           RRDevicePtr                       hits,
                                           RRDevicePtr                       scratch,
                                           RRCommandStream                   command_stream)
{
    RR_LOG_INFO("rrCudaCmdIntersectBatchHost(%u)", request_count);
    if (!context || !requests || !request_count || !rays || !hits || !scratch || !command_stream)
        return RR_ERROR_INVALID_PARAMETER;
    RR_TRY({
        Context*    ctx = C(context);
        DeviceGuard g(ctx->device);
        uint8_t*    dr  = P(rays)->addr();
        uint8_t*    dh  = P(hits)->addr();
        std::vector<DevRequest> dq(request_count);
        struct Copy
        {
            const void* host_rays;
            void*       host_hits;
            uint8_t*    dev_rays;
            uint8_t*    dev_hits;
            size_t      ray_bytes, hit_bytes;
        };
        std::vector<Copy> copies;
        uint64_t          off = 0;
        for (uint32_t k = 0; k < request_count; ++k)
        {
            const RRCudaHostIntersectRequest& q = requests[k];
            if (!q.geometry || (q.ray_count && (!q.host_rays || !q.host_hits))) return RR_ERROR_INVALID_PARAMETER;
            const size_t hs = q.output == RR_INTERSECT_QUERY_OUTPUT_FULL_HIT ? 16 : 4;
            dq[k] = DevRequest{P(q.geometry)->addr(), q.query, q.output, dr + 32 * off, q.ray_count, dh + 16 * off};
            if (q.ray_count)
                copies.push_back(Copy{q.host_rays, q.host_hits, dr + 32 * off, dh + 16 * off, 32ull * q.ray_count,
                                      hs * q.ray_count});
            off += q.ray_count;
        }
        Op      trace;
        RRError e = batch_trace_op(ctx, dq, P(scratch)->addr(), &trace);
        if (e != RR_SUCCESS) return e;
        const size_t hit_total = 16 * off;
        record(
            S(command_stream),
            [=](cudaStream_t s) -> cudaError_t {
                cudaError_t e = cudaSuccess;
                for (size_t i = 0; i < copies.size() && e == cudaSuccess; ++i)
                    e = cudaMemcpyAsync(copies[i].dev_rays, copies[i].host_rays, copies[i].ray_bytes,
                                        cudaMemcpyHostToDevice, s);
                // Fields a miss leaves untouched read back as 0xFFFFFFFF.
                if (e == cudaSuccess) e = cudaMemsetAsync(dh, 0xff, hit_total, s);
                if (e == cudaSuccess) e = trace(s);
                for (size_t i = 0; i < copies.size() && e == cudaSuccess; ++i)
                    e = cudaMemcpyAsync(copies[i].host_hits, copies[i].dev_hits, copies[i].hit_bytes,
                                        cudaMemcpyDeviceToHost, s);
                return e;
            },
            true);
        return RR_SUCCESS;
    })
}

RR_API RRError rrAllocateCommandStream(RRContext context, RRCommandStream* command_stream)
{
    if (!context || !command_stream) return RR_ERROR_INVALID_PARAMETER;
    RR_TRY({
        CommandStream* cs = new CommandStream;
        cs->ctx           = C(context);
        cs->stream        = C(context)->stream;
        *command_stream   = reinterpret_cast<RRCommandStream>(cs);
        return RR_SUCCESS;
    })
}

RR_API RRError rrReleaseCommandStream(RRContext context, RRCommandStream command_stream)
{
    if (!context || !command_stream) return RR_ERROR_INVALID_PARAMETER;
    if (S(command_stream)->external) return RR_ERROR_INVALID_PARAMETER;
    RR_TRY({
        DeviceGuard g(C(context)->device);
        delete S(command_stream);
        return RR_SUCCESS;
    })
}

RR_API RRError rrSumbitCommandStream(RRContext context, RRCommandStream command_stream, RREvent wait_event,
                                     RREvent* out_event)
{
    RR_LOG_INFO("rrSumbitCommandStream");
    if (!context || !command_stream || !out_event) return RR_ERROR_INVALID_PARAMETER;
    RR_TRY({
        Context*       ctx = C(context);
        CommandStream* cs  = S(command_stream);
        DeviceGuard    g(ctx->device);
        cudaStream_t   st = cs->stream;
        if (wait_event) check(cudaStreamWaitEvent(st, E(wait_event)->ev, 0), "cudaStreamWaitEvent");
        if (!cs->external)
        {
            flush_builds(cs);
            bool done = false;
            if (ctx->graphs && !cs->graph_failed && (cs->ops.size() > 1 || cs->want_graph))
            {
                if (!cs->graph || cs->graph_ops != cs->ops.size())
                {
                    if (cs->graph)
                    {
                        cudaGraphExecDestroy(cs->graph);
                        cs->graph = nullptr;
                    }
                    cudaGraph_t graph = nullptr;
                    bool        ok    = cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed) == cudaSuccess;
                    for (auto& op : cs->ops)
                        if (ok && op(st) != cudaSuccess) ok = false;
                    cudaError_t ec = cudaStreamEndCapture(st, &graph);
                    ok             = ok && ec == cudaSuccess && graph;
                    if (ok && cudaGraphInstantiate(&cs->graph, graph, 0) != cudaSuccess) ok = false;
                    if (graph) cudaGraphDestroy(graph);
                    cudaGetLastError();
                    if (!ok)
                    {
                        cs->graph_failed = true;
                        if (cs->graph) cudaGraphExecDestroy(cs->graph);
                        cs->graph = nullptr;
                    }
                    else
                        cs->graph_ops = cs->ops.size();
                }
                if (cs->graph)
                {
                    check(cudaGraphLaunch(cs->graph, st), "cudaGraphLaunch");
                    done = true;
                }
            }
            if (!done)
                for (auto& op : cs->ops) check(op(st), "command");
        }
        std::unique_ptr<Event> ev(new Event);
        check(cudaEventCreateWithFlags(&ev->ev, cudaEventDisableTiming), "cudaEventCreate");
        check(cudaEventRecord(ev->ev, st), "cudaEventRecord");
        *out_event = reinterpret_cast<RREvent>(ev.release());
        return RR_SUCCESS;
    })
}

RR_API RRError rrReleaseEvent(RRContext context, RREvent event)
{
    if (!context || !event) return RR_ERROR_INVALID_PARAMETER;
    RR_TRY({
        DeviceGuard g(C(context)->device);
        cudaEventDestroy(E(event)->ev);
        delete E(event);
        return RR_SUCCESS;
    })
}

RR_API RRError rrWaitEvent(RRContext context, RREvent event)
{
    if (!context || !event) return RR_ERROR_INVALID_PARAMETER;
    RR_TRY({
        Context*    ctx = C(context);
        DeviceGuard g(ctx->device);
        const auto  t0 = std::chrono::steady_clock::now();
        for (uint64_t spin = 0;; ++spin)
        {
            cudaError_t e = cudaEventQuery(E(event)->ev);
            if (e == cudaSuccess) return RR_SUCCESS;
            if (e != cudaErrorNotReady) throw CudaFail(e, "cudaEventQuery");
            const auto ms =
                std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0).count();
            if ((uint64_t)ms > ctx->wait_ms)
            {
                RR_LOG_ERROR("rrWaitEvent: timed out after %u ms", ctx->wait_ms);
                return RR_ERROR_INTERNAL;
            }
            if (spin < 2000)
                std::this_thread::yield();
            else
                std::this_thread::sleep_for(std::chrono::microseconds(50));
        }
    })
}

RR_API RRError rrReleaseDevicePtr(RRContext context, RRDevicePtr ptr)
{
    if (!context || !ptr) return RR_ERROR_INVALID_PARAMETER;
    RR_TRY({
        DeviceGuard g(C(context)->device);
        DevicePtr* p = P(ptr);
        if (p->managed && p->base) cudaFree(p->base);
        delete p;
        return RR_SUCCESS;
    })
}

RR_API RRError rrReleaseExternalCommandStream(RRContext context, RRCommandStream command_stream)
{
    if (!context || !command_stream) return RR_ERROR_INVALID_PARAMETER;
    delete S(command_stream);
    return RR_SUCCESS;
}

RR_API RRError rrGetDevicePtrFromCudaPtr(RRContext context, void* cuda_ptr, size_t offset, RRDevicePtr* device_ptr)
{
    if (!context || !cuda_ptr || !device_ptr) return RR_ERROR_INVALID_PARAMETER;
    RR_TRY({
        DevicePtr* p = new DevicePtr;
        p->base      = reinterpret_cast<uint8_t*>(cuda_ptr);
        p->offset    = offset;
        *device_ptr  = reinterpret_cast<RRDevicePtr>(p);
        return RR_SUCCESS;
    })
}

RR_API RRError rrGetCudaPtrFromDevicePtr(RRContext context, RRDevicePtr device_ptr, void** cuda_ptr)
{
    if (!context || !device_ptr || !cuda_ptr) return RR_ERROR_INVALID_PARAMETER;
    *cuda_ptr = P(device_ptr)->addr();
    return RR_SUCCESS;
}

RR_API RRError rrGetCommandStreamFromCudaStream(RRContext context, void* cuda_stream, RRCommandStream* command_stream)
{
    if (!context || !command_stream) return RR_ERROR_INVALID_PARAMETER;
    RR_TRY({
        CommandStream* cs = new CommandStream;
        cs->ctx           = C(context);
        cs->external      = true;
        cs->stream        = reinterpret_cast<cudaStream_t>(cuda_stream);
        *command_stream   = reinterpret_cast<RRCommandStream>(cs);
        return RR_SUCCESS;
    })
}

RR_API RRError rrAllocateDeviceBuffer(RRContext context, size_t size, RRDevicePtr* device_ptr)
{
    if (!context || !size || !device_ptr) return RR_ERROR_INVALID_PARAMETER;
    RR_TRY({
        DeviceGuard g(C(context)->device);
        void*       mem = nullptr;
        check(cudaMallocManaged(&mem, size), "cudaMallocManaged");
        DevicePtr* p = new DevicePtr;
        p->base      = reinterpret_cast<uint8_t*>(mem);
        p->managed   = true;
        p->size      = size;
        *device_ptr  = reinterpret_cast<RRDevicePtr>(p);
        return RR_SUCCESS;
    })
}

RR_API RRError rrMapDevicePtr(RRContext context, RRDevicePtr device_ptr, void** mapping_ptr)
{
    if (!context || !device_ptr || !mapping_ptr) return RR_ERROR_INVALID_PARAMETER;
    DevicePtr* p = P(device_ptr);
    if (!p->managed) return RR_ERROR_INVALID_PARAMETER;
    RR_TRY({
        DeviceGuard g(C(context)->device);
        // Managed memory: make prior device work visible before the host reads.
        check(cudaStreamSynchronize(C(context)->stream), "sync");
        check(cudaDeviceSynchronize(), "sync");
        *mapping_ptr = p->addr();
        return RR_SUCCESS;
    })
}

RR_API RRError rrUnmapDevicePtr(RRContext context, RRDevicePtr device_ptr, void** mapping_ptr)
{
    if (!context || !device_ptr) return RR_ERROR_INVALID_PARAMETER;
    if (!P(device_ptr)->managed) return RR_ERROR_INVALID_PARAMETER;
    if (mapping_ptr) *mapping_ptr = nullptr;
    return RR_SUCCESS;
}

RR_API RRError rrCudaSetTraversalOptions(RRContext context, const RRCudaTraversalOptions* options)
{
    if (!context || !options || options->struct_size < sizeof(RRCudaTraversalOptions)) return RR_ERROR_INVALID_PARAMETER;
    if (options->traversal > RR_CUDA_TRAVERSAL_BVH4 || options->ray_order > 2)
        return RR_ERROR_INVALID_PARAMETER;
    if (options->block_size && (options->block_size % 32 || options->block_size > 1024)) return RR_ERROR_INVALID_PARAMETER;
    if (options->short_stack && (options->short_stack < 12 || options->short_stack > 32)) return RR_ERROR_INVALID_PARAMETER;
    if (options->triangle_test > RR_CUDA_TRIANGLE_TEST_WATERTIGHT) return RR_ERROR_INVALID_PARAMETER;
    // The precise test runs in the persistent kernels (binary and 4-wide).
    if (options->triangle_test == RR_CUDA_TRIANGLE_TEST_WATERTIGHT && options->traversal != RR_CUDA_TRAVERSAL_AUTO &&
        options->traversal != RR_CUDA_TRAVERSAL_BINARY_PERSISTENT && options->traversal != RR_CUDA_TRAVERSAL_BVH4)
        return RR_ERROR_INVALID_PARAMETER;
    C(context)->topts = *options;
    return RR_SUCCESS;
}

RR_API RRError rrCudaGetTraversalOptions(RRContext context, RRCudaTraversalOptions* options)
{
    if (!context || !options) return RR_ERROR_INVALID_PARAMETER;
    *options = C(context)->topts;
    return RR_SUCCESS;
}

RR_API RRError rrCudaGetDeviceErrors(RRContext context, uint32_t* error_bits)
{
    if (!context || !error_bits) return RR_ERROR_INVALID_PARAMETER;
    RR_TRY({
        Context*    ctx = C(context);
        DeviceGuard g(ctx->device);
        check(cudaDeviceSynchronize(), "sync");
        uint32_t v = 0;
        check(cudaMemcpy(&v, &ctx->words->error_bits, 4, cudaMemcpyDeviceToHost), "read error word");
        check(cudaMemset(&ctx->words->error_bits, 0, 4), "clear error word");
        *error_bits = v;
        return RR_SUCCESS;
    })
}

RR_API RRError rrCudaGetTraversalStats(RRContext context, RRCudaTraversalStats* stats)
{
    if (!context || !stats) return RR_ERROR_INVALID_PARAMETER;
    RR_TRY({
        Context*    ctx = C(context);
        DeviceGuard g(ctx->device);
        check(cudaDeviceSynchronize(), "sync");
        DeviceWords w;
        check(cudaMemcpy(&w, ctx->words, sizeof(w), cudaMemcpyDeviceToHost), "read stats");
        check(cudaMemset(&ctx->words->rays, 0, 3 * sizeof(unsigned long long)), "clear stats");
        stats->rays             = w.rays;
        stats->node_fetches     = w.node_fetches;
        stats->triangle_fetches = w.tri_fetches;
        stats->node_bytes       = 0;
        stats->triangle_bytes   = sizeof(WideTri);
        return RR_SUCCESS;
    })
}

RR_API RRError rrCudaSetWaitTimeout(RRContext context, uint32_t milliseconds)
{
    if (!context) return RR_ERROR_INVALID_PARAMETER;
    C(context)->wait_ms = milliseconds;
    return RR_SUCCESS;
}

RR_API RRError rrCudaSetWaitLimits(RRContext context, const RRCudaWaitLimits* limits)
{
    if (!context || !limits || limits->struct_size < sizeof(RRCudaWaitLimits)) return RR_ERROR_INVALID_PARAMETER;
    RR_TRY({
        Context*    ctx = C(context);
        DeviceGuard g(ctx->device);
        // The device words are read by kernels: change them in stream order.
        const uint32_t w[2] = {limits->lookback_polls,
                               limits->test_hold_sort_tile == kInvalid ? 0u : limits->test_hold_sort_tile + 1u};
        check(cudaMemcpyAsync(&ctx->words->lookback_polls, w, sizeof(w), cudaMemcpyHostToDevice, ctx->stream),
              "wait limits");
        check(cudaStreamSynchronize(ctx->stream), "wait limits");
        ctx->arrival_polls = limits->arrival_polls;
        ctx->drop_arrival  = limits->test_drop_arrival_chunk;
        return RR_SUCCESS;
    })
}

RR_API RRError rrCudaAutotuneTraversal(RRContext              context,
                                       RRDevicePtr            scene_buffer,
                                       RRIntersectQuery       query,
                                       RRDevicePtr            rays,
                                       uint32_t               ray_count,
                                       RRIntersectQueryOutput query_output,
                                       RRDevicePtr            hits,
                                       RRDevicePtr            scratch,
                                       RRCudaTraversalOptions* chosen)
{
    if (!context || !scene_buffer || !rays || !hits || !scratch || !ray_count) return RR_ERROR_INVALID_PARAMETER;
    if (query != RR_INTERSECT_QUERY_CLOSEST && query != RR_INTERSECT_QUERY_ANY) return RR_ERROR_INVALID_PARAMETER;
    if (query_output != RR_INTERSECT_QUERY_OUTPUT_FULL_HIT && query_output != RR_INTERSECT_QUERY_OUTPUT_INSTANCE_ID)
        return RR_ERROR_INVALID_PARAMETER;
    RR_TRY({
        Context*    ctx = C(context);
        DeviceGuard g(ctx->device);
        return autotune_traversal(ctx, P(scene_buffer)->addr(), query, P(rays)->addr(), ray_count, query_output,
                                  P(hits)->addr(), P(scratch)->addr(), true, chosen, nullptr);
    })
}

RR_API RRError rrCudaAutotuneNodeFormat(RRContext                   context,
                                        const RRGeometryBuildInput* build_input,
                                        const RRBuildOptions*       build_options,
                                        RRIntersectQuery            query,
                                        RRDevicePtr                 rays,
                                        uint32_t                    ray_count,
                                        RRIntersectQueryOutput      query_output,
                                        RRDevicePtr                 hits,
                                        RRDevicePtr                 scratch,
                                        uint32_t*                   node_format)
{
    if (!context || !build_input || !rays || !hits || !scratch || !ray_count) return RR_ERROR_INVALID_PARAMETER;
    if (query != RR_INTERSECT_QUERY_CLOSEST && query != RR_INTERSECT_QUERY_ANY) return RR_ERROR_INVALID_PARAMETER;
    if (query_output != RR_INTERSECT_QUERY_OUTPUT_FULL_HIT && query_output != RR_INTERSECT_QUERY_OUTPUT_INSTANCE_ID)
        return RR_ERROR_INVALID_PARAMETER;
    RR_TRY({
        BuildParams bp;
        if (!parse_build_options(build_options, bp)) return RR_ERROR_INVALID_PARAMETER;
        Context*    ctx = C(context);
        DeviceGuard g(ctx->device);
        MeshArgs    ma;
        RRError     e = geometry_source(build_input, true, &ma);
        if (e != RR_SUCCESS) return e;
        if (ma.n == 0 || ma.prim_kind != kPrimTriangles) return RR_ERROR_INVALID_PARAMETER;
        if (ctx->topts.triangle_test == RR_CUDA_TRIANGLE_TEST_WATERTIGHT) return RR_ERROR_NOT_IMPLEMENTED;
        uint32_t               best_fmt = RR_CUDA_NODE_FORMAT_BVH4;
        float                  best_ms  = 1e30f;
        RRCudaTraversalOptions best_opt{};
        // Each width: a temporary build on the context's stream (the tuner
        // allocates; a build call never does), then the traversal tuner on
        // the caller's rays, timed afresh.
        for (uint32_t fmt : {(uint32_t)RR_CUDA_NODE_FORMAT_BVH4, (uint32_t)RR_CUDA_NODE_FORMAT_BVH4Q8,
                             (uint32_t)RR_CUDA_NODE_FORMAT_WIDE8})
        {
            PendingGeom pg;
            pg.ma                    = ma;
            pg.L                     = geom_layout(ma.n, fmt, bp.bits);
            pg.L.restructure_min     = bp.restructure ? kRestructureMinPrims : 0u;
            pg.L.restructure_passes  = bp.restructure ? kRestructurePasses : 0u;
            uint8_t *sc = nullptr, *res = nullptr;
            check(cudaMalloc(&sc, pg.L.s_total), "cudaMalloc tuner scratch");
            if (cudaMalloc(&res, pg.L.total) != cudaSuccess)
            {
                cudaFree(sc);
                throw CudaFail(cudaErrorMemoryAllocation, "cudaMalloc tuner result");
            }
            pg.scratch = sc;
            pg.result  = res;
            float                  ms = -1.f;
            RRCudaTraversalOptions o{};
            RRError                r  = RR_SUCCESS;
            try
            {
                bool many = false;
                Op   op   = build_batch_op(ctx, {pg}, &many);
                check(op(ctx->stream), "tuner build");
                check(cudaStreamSynchronize(ctx->stream), "tuner build");
                register_geometry(ctx, pg);
                r = autotune_traversal(ctx, res, query, P(rays)->addr(), ray_count, query_output, P(hits)->addr(),
                                       P(scratch)->addr(), false, &o, &ms);
            }
            catch (...)
            {
                ctx->registry.erase((uintptr_t)res);
                cudaStreamSynchronize(ctx->stream);
                cudaFree(sc);
                cudaFree(res);
                throw;
            }
            ctx->registry.erase((uintptr_t)res);
            cudaStreamSynchronize(ctx->stream);
            cudaFree(sc);
            cudaFree(res);
            if (r != RR_SUCCESS) return r;
            RR_LOG_INFO("node-format tune: format %u -> traversal %u, %.3f ms", fmt, o.traversal, ms);
            if (ms >= 0.f && ms < best_ms)
            {
                best_ms  = ms;
                best_fmt = fmt;
                best_opt = o;
            }
        }
        const std::string key = fmt_key(ctx, ma.n);
        ctx->fmt_choice[key]  = best_fmt;
        if (const char* path = std::getenv("RR_CUDA_TUNE_CACHE"))
            if (FILE* f = std::fopen(path, "a"))
            {
                std::fprintf(f, "%s\t%u\n", key.c_str(), best_fmt);
                std::fclose(f);
            }
        ctx->topts = best_opt;
        if (node_format) *node_format = best_fmt;
        return RR_SUCCESS;
    })
}

}  // extern "C"
