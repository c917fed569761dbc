// ref_harness.cpp -- C entry points around the reference's own CPU traversal.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/Makefile against the unmodified
// headers of the reference's bvh_analyzer tool (bvh_analyzer/bvh.h,
// transform.h) where they lie in the reference checkout; the output goes to
// oracle/_ref/ and is never shipped or linked by the product.
//
// What it exposes:
//   rrref_trace    -- bvh::BvhIntersect (bvh_analyzer/bvh.h:225-328) over a
//                     BVH in the reference's 64-byte Vulkan node layout,
//                     converted with bvh::Transform2<VkBvhNode>
//                     (bvh_analyzer/transform.h:56-125).
//   rrref_validate -- bvh::Bvh::IsValid (bvh.h:129-184) and CalculateSAH
//                     (bvh.h:186-223).
//
// The two private members are reached by compiling the header with `private`
// spelled `public`; all standard headers it uses are included first so that
// only the reference's own class is affected.
//
// bvh_analyzer/float3.h `rcp` calls unqualified abs() on floats.  Under
// libstdc++ only `int abs(int)` is visible at global scope, so every direction
// component with |d| < 1 becomes +-1e5 and the tool misses nearly every ray.
// The tool was written against MSVC, whose global abs has float overloads;
// `using std::abs;` below restores that overload set without touching the
// reference sources.
#include <cstdlib>
using std::abs;
#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <iostream>
#include <limits>
#include <map>
#include <numeric>
#include <ostream>
#include <queue>
#include <set>
#include <stack>
#include <stdexcept>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#define private public
#include "bvh.h"
#include "transform.h"
#undef private

#define STB_IMAGE_WRITE_IMPLEMENTATION
#include "stb_image_write.h"

namespace
{
struct Loaded
{
    bvh::Bvh<2u> tree;
    Loaded(const void* nodes, uint32_t internal, uint32_t tris) : tree(internal, tris)
    {
        tree.TransformBvh(bvh::Transform2<bvh::VkBvhNode>, nodes, nullptr);
    }
};
}  // namespace

extern "C" {

// Closest (any = 0) or any (any = 1) hit of every ray; hits are 16-byte
// {uv[2], inst_id, prim_id} records as bvh::Hit.  Returns wall seconds of the
// ray loop alone.
double rrref_trace(const void* vk_nodes, uint32_t internal, uint32_t tris, const void* rays, uint32_t nrays, int any,
                   void* hits_out, int threads)
{
    Loaded                L(vk_nodes, internal, tris);
    const bvh::Ray*       r    = reinterpret_cast<const bvh::Ray*>(rays);
    bvh::Hit*             h    = reinterpret_cast<bvh::Hit*>(hits_out);
    const bvh::QueryType  type = any ? bvh::QueryType::kAnyHit : bvh::QueryType::kClosestHit;
    std::atomic<uint32_t> next{0};
    auto                  t0 = std::chrono::steady_clock::now();
    auto                  work = [&]() {
        bvh::BvhIntersect<2u> isect(L.tree, type);
        for (;;)
        {
            uint32_t b = next.fetch_add(256);
            if (b >= nrays) break;
            uint32_t e = std::min<uint32_t>(nrays, b + 256);
            for (uint32_t i = b; i < e; ++i) h[i] = isect(r[i]);
        }
    };
    if (threads <= 1)
        work();
    else
    {
        std::vector<std::thread> pool;
        for (int t = 0; t < threads; ++t) pool.emplace_back(work);
        for (auto& th : pool) th.join();
    }
    auto t1 = std::chrono::steady_clock::now();
    return std::chrono::duration<double>(t1 - t0).count();
}

// Structural validity (parent links, child-box containment, every node and
// primitive reached once) and SAH of a BVH in the Vulkan node layout.
int rrref_validate(const void* vk_nodes, uint32_t internal, uint32_t tris, float* sah)
{
    Loaded L(vk_nodes, internal, tris);
    bool   ok = L.tree.IsValid();
    if (sah) *sah = ok ? L.tree.CalculateSAH() : 0.f;
    return ok ? 1 : 0;
}
}
