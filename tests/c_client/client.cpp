// client.cpp -- a C++ client of librr.so written against the public headers
// only, in the flow of the reference's BasicTest (test/test_vk/basic_test.h):
// context, device pointers from CUDA allocations, geometry build and
// closest-hit intersection recorded into a command stream, submit, wait.
// Then the same trace through an external CUDA stream with the autotuner's
// choice.  The mesh is a flat 64 x 64 grid of quads at z = 0 (two triangles
// per quad); one ray per quad falls straight down onto a point inside a known
// triangle, so every hit (primitive and barycentrics) is known analytically.
// Exit status 0 and a final "ok" line when every check passes.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "radeonrays.h"
#include "radeonrays_cuda.h"

namespace
{
int failures = 0;

void expect(bool ok, const char* what)
{
    if (!ok)
    {
        std::printf("FAIL: %s\n", what);
        ++failures;
    }
}

#define RR_CHECK(call) expect((call) == RR_SUCCESS, #call)
#define CUDA_CHECK(call) expect((call) == cudaSuccess, #call)

constexpr int kGrid = 64;  // quads per side

struct Ray
{
    float o[3], tmin, d[3], tmax;
};
struct Hit
{
    float    uv[2];
    uint32_t inst_id, prim_id;
};

// Triangle t0 of quad (i, j) is (v00, v10, v11), t1 is (v00, v11, v01); the
// ray of quad (i, j) goes to local point (0.75, 0.25) for even quads (t0) and
// (0.25, 0.75) for odd ones (t1).
void make_scene(std::vector<float>& v, std::vector<uint32_t>& idx, std::vector<Ray>& rays,
                std::vector<uint32_t>& want_prim, std::vector<float>& want_uv)
{
    const float h = 1.0f / kGrid;
    for (int j = 0; j <= kGrid; ++j)
        for (int i = 0; i <= kGrid; ++i)
        {
            v.push_back(i * h);
            v.push_back(j * h);
            v.push_back(0.0f);
        }
    for (int j = 0; j < kGrid; ++j)
        for (int i = 0; i < kGrid; ++i)
        {
            const uint32_t v00 = j * (kGrid + 1) + i, v10 = v00 + 1, v01 = v00 + kGrid + 1, v11 = v01 + 1;
            const uint32_t t0[3] = {v00, v10, v11}, t1[3] = {v00, v11, v01};
            idx.insert(idx.end(), t0, t0 + 3);
            idx.insert(idx.end(), t1, t1 + 3);
            const bool  odd = ((i + j) & 1) != 0;
            const float lu = odd ? 0.25f : 0.75f, lv = odd ? 0.75f : 0.25f;
            Ray         r{};
            r.o[0] = (i + lu) * h;
            r.o[1] = (j + lv) * h;
            r.o[2] = 1.0f;
            r.d[2] = -1.0f;
            r.tmax = 1e30f;
            rays.push_back(r);
            const uint32_t q = 2u * (uint32_t)(j * kGrid + i);
            want_prim.push_back(odd ? q + 1 : q);
            // Barycentrics (u, w) of p = v0 + u (v1 - v0) + w (v2 - v0):
            // t0 gives (lu - lv, lv), t1 gives (lu, lv - lu).
            want_uv.push_back(odd ? lu : lu - lv);
            want_uv.push_back(odd ? lv - lu : lv);
        }
}

int check_hits(const std::vector<Hit>& hits, const std::vector<uint32_t>& want_prim,
               const std::vector<float>& want_uv, const char* what)
{
    int bad = 0;
    for (size_t k = 0; k < hits.size(); ++k)
    {
        const bool ok = hits[k].inst_id == 0 && hits[k].prim_id == want_prim[k] &&
                        std::fabs(hits[k].uv[0] - want_uv[2 * k]) < 1e-4f &&
                        std::fabs(hits[k].uv[1] - want_uv[2 * k + 1]) < 1e-4f;
        bad += ok ? 0 : 1;
    }
    if (bad) std::printf("FAIL: %s: %d of %zu hits differ\n", what, bad, hits.size());
    failures += bad ? 1 : 0;
    return bad;
}
}  // namespace

int main()
{
    std::vector<float>    v, want_uv;
    std::vector<uint32_t> idx, want_prim;
    std::vector<Ray>      rays;
    make_scene(v, idx, rays, want_prim, want_uv);
    const uint32_t nv = (uint32_t)(v.size() / 3), nt = (uint32_t)(idx.size() / 3), nr = (uint32_t)rays.size();

    RRContext ctx = nullptr;
    RR_CHECK(rrCreateContext(RR_API_VERSION, RR_API_CUDA, &ctx));
    if (!ctx) return 1;

    float*    d_v = nullptr;
    uint32_t* d_i = nullptr;
    Ray*      d_rays = nullptr;
    Hit*      d_hits = nullptr;
    CUDA_CHECK(cudaMalloc(&d_v, v.size() * sizeof(float)));
    CUDA_CHECK(cudaMalloc(&d_i, idx.size() * sizeof(uint32_t)));
    CUDA_CHECK(cudaMalloc(&d_rays, nr * sizeof(Ray)));
    CUDA_CHECK(cudaMalloc(&d_hits, nr * sizeof(Hit)));
    CUDA_CHECK(cudaMemcpy(d_v, v.data(), v.size() * sizeof(float), cudaMemcpyHostToDevice));
    CUDA_CHECK(cudaMemcpy(d_i, idx.data(), idx.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    CUDA_CHECK(cudaMemcpy(d_rays, rays.data(), nr * sizeof(Ray), cudaMemcpyHostToDevice));

    RRDevicePtr vptr = nullptr, iptr = nullptr, rptr = nullptr, hptr = nullptr;
    RR_CHECK(rrGetDevicePtrFromCudaPtr(ctx, d_v, 0, &vptr));
    RR_CHECK(rrGetDevicePtrFromCudaPtr(ctx, d_i, 0, &iptr));
    RR_CHECK(rrGetDevicePtrFromCudaPtr(ctx, d_rays, 0, &rptr));
    RR_CHECK(rrGetDevicePtrFromCudaPtr(ctx, d_hits, 0, &hptr));

    RRTriangleMeshPrimitive mesh{};
    mesh.vertices         = vptr;
    mesh.vertex_count     = nv;
    mesh.vertex_stride    = 3 * sizeof(float);
    mesh.triangle_indices = iptr;
    mesh.triangle_count   = nt;
    mesh.index_type       = RR_INDEX_TYPE_UINT32;
    RRGeometryBuildInput in{};
    in.primitive_type           = RR_PRIMITIVE_TYPE_TRIANGLE_MESH;
    in.primitive_count          = 1;
    in.triangle_mesh_primitives = &mesh;
    RRBuildOptions opts{};
    opts.build_flags           = RR_BUILD_FLAG_BITS_PREFER_FAST_BUILD;
    opts.backend_specific_info = nullptr;  // the default node format

    RRMemoryRequirements req{};
    RR_CHECK(rrGetGeometryBuildMemoryRequirements(ctx, &in, &opts, &req));
    size_t trace_bytes = 0;
    RR_CHECK(rrGetTraceMemoryRequirements(ctx, nr, &trace_bytes));
    void *d_scratch = nullptr, *d_geom = nullptr, *d_tscratch = nullptr;
    CUDA_CHECK(cudaMalloc(&d_scratch, req.temporary_build_buffer_size));
    CUDA_CHECK(cudaMalloc(&d_geom, req.result_buffer_size));
    CUDA_CHECK(cudaMalloc(&d_tscratch, trace_bytes));
    RRDevicePtr sptr = nullptr, gptr = nullptr, tptr = nullptr;
    RR_CHECK(rrGetDevicePtrFromCudaPtr(ctx, d_scratch, 0, &sptr));
    RR_CHECK(rrGetDevicePtrFromCudaPtr(ctx, d_geom, 0, &gptr));
    RR_CHECK(rrGetDevicePtrFromCudaPtr(ctx, d_tscratch, 0, &tptr));

    // Build and trace recorded into one command stream, submitted once.
    RRCommandStream cs = nullptr;
    RR_CHECK(rrAllocateCommandStream(ctx, &cs));
    RR_CHECK(rrCmdBuildGeometry(ctx, RR_BUILD_OPERATION_BUILD, &in, &opts, sptr, gptr, cs));
    RR_CHECK(rrCmdIntersect(ctx, gptr, RR_INTERSECT_QUERY_CLOSEST, rptr, nr, nullptr,
                            RR_INTERSECT_QUERY_OUTPUT_FULL_HIT, hptr, tptr, cs));
    RREvent ev = nullptr;
    RR_CHECK(rrSumbitCommandStream(ctx, cs, nullptr, &ev));
    RR_CHECK(rrWaitEvent(ctx, ev));
    RR_CHECK(rrReleaseEvent(ctx, ev));
    RR_CHECK(rrReleaseCommandStream(ctx, cs));
    std::vector<Hit> hits(nr);
    CUDA_CHECK(cudaMemcpy(hits.data(), d_hits, nr * sizeof(Hit), cudaMemcpyDeviceToHost));
    check_hits(hits, want_prim, want_uv, "recorded build + trace");

    // The autotuner's pick, traced through an external CUDA stream.
    RRCudaTraversalOptions chosen{};
    chosen.struct_size = sizeof(chosen);
    RR_CHECK(rrCudaAutotuneTraversal(ctx, gptr, RR_INTERSECT_QUERY_CLOSEST, rptr, nr,
                                     RR_INTERSECT_QUERY_OUTPUT_FULL_HIT, hptr, tptr, &chosen));
    cudaStream_t st = nullptr;
    CUDA_CHECK(cudaStreamCreate(&st));
    RRCommandStream ext = nullptr;
    RR_CHECK(rrGetCommandStreamFromCudaStream(ctx, (void*)st, &ext));
    CUDA_CHECK(cudaMemset(d_hits, 0xff, nr * sizeof(Hit)));
    RR_CHECK(rrCmdIntersect(ctx, gptr, RR_INTERSECT_QUERY_CLOSEST, rptr, nr, nullptr,
                            RR_INTERSECT_QUERY_OUTPUT_FULL_HIT, hptr, tptr, ext));
    CUDA_CHECK(cudaStreamSynchronize(st));
    CUDA_CHECK(cudaMemcpy(hits.data(), d_hits, nr * sizeof(Hit), cudaMemcpyDeviceToHost));
    check_hits(hits, want_prim, want_uv, "autotuned trace on an external stream");
    RR_CHECK(rrReleaseExternalCommandStream(ctx, ext));

    uint32_t device_errors = 0;
    RR_CHECK(rrCudaGetDeviceErrors(ctx, &device_errors));
    expect(device_errors == 0, "device error word is clear");

    for (RRDevicePtr p : {vptr, iptr, rptr, hptr, sptr, gptr, tptr}) RR_CHECK(rrReleaseDevicePtr(ctx, p));
    RR_CHECK(rrDestroyContext(ctx));
    cudaStreamDestroy(st);
    for (void* p : {(void*)d_v, (void*)d_i, (void*)d_rays, (void*)d_hits, d_scratch, d_geom, d_tscratch}) cudaFree(p);
    if (failures) return 1;
    std::printf("ok: %u triangles, %u rays, traversal %u\n", nt, nr, chosen.traversal);
    return 0;
}
