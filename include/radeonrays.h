/*
 * radeonrays.h -- public C interface of the GB300-native RadeonRays intersector.
 *
 * Drop-in replacement for the reference interface
 * (src/core/include/radeonrays.h of RadeonRays SDK): every type keeps its size,
 * member order and enum values, and every entry point keeps its name (including
 * the historical spellings `rrSumbitCommandStream` and `RR_INAVLID_VALUE`),
 * argument order and error conventions.  The only addition is the API value
 * RR_API_CUDA; the CUDA interop entry points live in radeonrays_cuda.h.
 *
 * Execution model: rrCmd* calls record work into a command stream; nothing runs
 * until rrSumbitCommandStream.  A command stream obtained from a CUDA stream
 * (radeonrays_cuda.h) enqueues immediately instead.
 *
 * Threading: calls on different contexts from different threads are safe;
 * calls on one context must be serialised by the caller.
 */
#ifndef RADEONRAYS_H
#define RADEONRAYS_H

#define RR_API_MAJOR_VERSION 0x000000
#define RR_API_MINOR_VERSION 0x000001
#define RR_API_PATCH_VERSION 0x000001
#define RR_API_VERSION (RR_API_MAJOR_VERSION * 1000000 + RR_API_MINOR_VERSION * 1000 + RR_API_PATCH_VERSION)

#if defined(_WIN32)
#define RR_API
#else
#define RR_API __attribute__((visibility("default")))
#endif

#include <stddef.h>
#include <stdint.h>

struct _RRDevicePtr;
struct _RREvent;
struct _RRContext;
struct _RRCommandStream;

typedef uint32_t                 RRBuildFlags;
typedef uint32_t                 RRRayMask;
typedef struct _RRDevicePtr*     RRDevicePtr;
typedef struct _RRContext*       RRContext;
typedef struct _RREvent*         RREvent;
typedef struct _RRCommandStream* RRCommandStream;

/* reference: radeonrays.h:52-55 (spelling kept) */
enum
{
    RR_INAVLID_VALUE = ~0u
};

/* reference: radeonrays.h:57-68 */
typedef enum
{
    RR_SUCCESS                    = 0,
    RR_ERROR_NOT_IMPLEMENTED      = 1,
    RR_ERROR_INTERNAL             = 2,
    RR_ERROR_OUT_OF_HOST_MEMORY   = 3,
    RR_ERROR_OUT_OF_DEVICE_MEMORY = 4,
    RR_ERROR_INVALID_API_VERSION  = 5,
    RR_ERROR_INVALID_PARAMETER    = 6,
    RR_ERROR_UNSUPPORTED_API      = 7,
    RR_ERROR_UNSUPPORTED_INTEROP  = 8
} RRError;

/* reference: radeonrays.h:70-74.  RR_API_CUDA is the only backend of this
 * library; DX and VK are rejected with RR_ERROR_UNSUPPORTED_API. */
typedef enum
{
    RR_API_DX   = 1,
    RR_API_VK   = 2,
    RR_API_CUDA = 3
} RRApi;

/* reference: radeonrays.h:76-83 */
typedef enum
{
    RR_LOG_LEVEL_DEBUG = 1,
    RR_LOG_LEVEL_INFO  = 2,
    RR_LOG_LEVEL_WARN  = 3,
    RR_LOG_LEVEL_ERROR = 4,
    RR_LOG_LEVEL_OFF   = 5
} RRLogLevel;

/* reference: radeonrays.h:90-94 */
typedef enum
{
    RR_BUILD_OPERATION_BUILD  = 1,
    RR_BUILD_OPERATION_UPDATE = 2
} RRBuildOperation;

/* reference: radeonrays.h:101-105 */
typedef enum
{
    RR_BUILD_FLAG_BITS_PREFER_FAST_BUILD = 1,
    RR_BUILD_FLAG_BITS_ALLOW_UPDATE      = 2
} RRBuildFlagBits;

/* reference: radeonrays.h:113-117 */
typedef enum
{
    RR_PRIMITIVE_TYPE_TRIANGLE_MESH,
    RR_PRIMITIVE_TYPE_AABB_LIST
} RRPrimitiveType;

/* reference: radeonrays.h:122-126 */
typedef enum
{
    RR_INDEX_TYPE_UINT32,
    RR_INDEX_TYPE_UINT16
} RRIndexType;

/* reference: radeonrays.h:131-135 */
typedef enum
{
    RR_INTERSECT_QUERY_CLOSEST = 0,
    RR_INTERSECT_QUERY_ANY     = 1
} RRIntersectQuery;

/* reference: radeonrays.h:139-143 */
typedef enum
{
    RR_INTERSECT_QUERY_OUTPUT_FULL_HIT,
    RR_INTERSECT_QUERY_OUTPUT_INSTANCE_ID
} RRIntersectQueryOutput;

/* 32 bytes.  reference: radeonrays.h:147-153 */
typedef struct
{
    float origin[3];
    float min_t;
    float direction[3];
    float max_t;
} RRRay;

/* 16 bytes.  On a miss only inst_id is written (RR_INAVLID_VALUE); uv and
 * prim_id keep whatever the buffer held.  reference: radeonrays.h:157-162 */
typedef struct
{
    float    uv[2];
    uint32_t inst_id;
    uint32_t prim_id;
} RRHit;

/* reference: radeonrays.h:166-173.  backend_specific_info may point to an
 * RRCudaBuildOptions (radeonrays_cuda.h). */
typedef struct
{
    RRBuildFlags build_flags;
    void*        backend_specific_info;
} RRBuildOptions;

/* reference: radeonrays.h:182-192.  vertex_stride is in bytes (multiple of 4). */
typedef struct
{
    RRDevicePtr vertices;
    uint32_t    vertex_count;
    uint32_t    vertex_stride;

    RRDevicePtr triangle_indices;
    uint32_t    triangle_count;

    RRIndexType index_type;
} RRTriangleMeshPrimitive;

/* reference: radeonrays.h:201-206 */
typedef struct
{
    RRDevicePtr aabbs;
    uint32_t    aabb_count;
    uint32_t    aabb_stride;
} RRAABBListPrimitive;

/* reference: radeonrays.h:213-226 */
typedef struct
{
    RRPrimitiveType primitive_type;
    uint32_t        primitive_count;
    union
    {
        RRTriangleMeshPrimitive* triangle_mesh_primitives;
        RRAABBListPrimitive*     aabb_primitives;
    };
} RRGeometryBuildInput;

/* Row-major 3x4 object-to-world transform.  reference: radeonrays.h:228-232 */
typedef struct
{
    RRDevicePtr geometry;
    float       transform[3][4];
} RRInstance;

/* reference: radeonrays.h:246-252 */
typedef struct
{
    const RRInstance* instances;
    uint32_t          instance_count;
} RRSceneBuildInput;

/* reference: radeonrays.h:254-259 */
typedef struct
{
    size_t temporary_build_buffer_size;
    size_t temporary_update_buffer_size;
    size_t result_buffer_size;
} RRMemoryRequirements;

#ifdef __cplusplus
extern "C" {
#endif

/* reference: radeonrays.h:276.  api must be RR_API_CUDA. */
RR_API RRError rrCreateContext(uint32_t api_version, RRApi api, RRContext* context);
/* reference: radeonrays.h:286 */
RR_API RRError rrDestroyContext(RRContext context);
/* reference: radeonrays.h:295 */
RR_API RRError rrSetLogLevel(RRLogLevel log_level);
/* reference: radeonrays.h:304 */
RR_API RRError rrSetLogFile(char const* filename);

/* reference: radeonrays.h:322-328 */
RR_API RRError rrCmdBuildGeometry(RRContext                   context,
                                  RRBuildOperation            build_operation,
                                  const RRGeometryBuildInput* build_input,
                                  const RRBuildOptions*       build_options,
                                  RRDevicePtr                 temporary_buffer,
                                  RRDevicePtr                 geometry_buffer,
                                  RRCommandStream             command_stream);

/* reference: radeonrays.h:338-341 */
RR_API RRError rrGetGeometryBuildMemoryRequirements(RRContext                   context,
                                                    const RRGeometryBuildInput* build_input,
                                                    const RRBuildOptions*       build_options,
                                                    RRMemoryRequirements*       memory_requirements);

/* reference: radeonrays.h:357-362 */
RR_API RRError rrCmdBuildScene(RRContext                context,
                               const RRSceneBuildInput* build_input,
                               const RRBuildOptions*    build_options,
                               RRDevicePtr              temporary_buffer,
                               RRDevicePtr              scene_buffer,
                               RRCommandStream          command_stream);

/* reference: radeonrays.h:372-375 */
RR_API RRError rrGetSceneBuildMemoryRequirements(RRContext                context,
                                                 const RRSceneBuildInput* build_input,
                                                 const RRBuildOptions*    build_options,
                                                 RRMemoryRequirements*    memory_requirements);

/* reference: radeonrays.h:391-400 */
RR_API RRError rrCmdIntersect(RRContext              context,
                              RRDevicePtr            scene_buffer,
                              RRIntersectQuery       query,
                              RRDevicePtr            rays,
                              uint32_t               ray_count,
                              RRDevicePtr            indirect_ray_count,
                              RRIntersectQueryOutput query_output,
                              RRDevicePtr            hits,
                              RRDevicePtr            scratch,
                              RRCommandStream        command_stream);

/* reference: radeonrays.h:409 */
RR_API RRError rrGetTraceMemoryRequirements(RRContext context, uint32_t ray_count, size_t* scratch_size);
/* reference: radeonrays.h:418 */
RR_API RRError rrAllocateCommandStream(RRContext context, RRCommandStream* command_stream);
/* reference: radeonrays.h:427 */
RR_API RRError rrReleaseCommandStream(RRContext context, RRCommandStream command_stream);
/* reference: radeonrays.h:438-441 (spelling kept) */
RR_API RRError rrSumbitCommandStream(RRContext       context,
                                     RRCommandStream command_stream,
                                     RREvent         wait_event,
                                     RREvent*        out_event);
/* reference: radeonrays.h:449 */
RR_API RRError rrReleaseEvent(RRContext context, RREvent event);
/* reference: radeonrays.h:457 */
RR_API RRError rrWaitEvent(RRContext context, RREvent event);
/* reference: radeonrays.h:465 */
RR_API RRError rrReleaseDevicePtr(RRContext context, RRDevicePtr ptr);
/* reference: radeonrays.h:473 */
RR_API RRError rrReleaseExternalCommandStream(RRContext context, RRCommandStream command_stream);

#ifdef __cplusplus
}
#endif

#endif /* RADEONRAYS_H */
