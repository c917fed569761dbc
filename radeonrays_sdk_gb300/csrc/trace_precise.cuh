// trace_precise.cuh -- the opt-in precise triangle test
// (RRCudaTraversalOptions::triangle_test = RR_CUDA_TRIANGLE_TEST_WATERTIGHT)
// and the conservative box test that goes with it.  FP32 arithmetic only.
//
// No reference counterpart: the reference's test (vlk/kernels/common.h:103-137,
// Moller-Trumbore, restated in trace_common.cuh) is kept as the default
// because its hits are the reference's bit for bit.  This mode trades that
// identity for three properties:
//
//  * watertight hit decision (Woop, Benthin, Wald, "Watertight Ray/Triangle
//    Intersection", JCGT 2013): the vertices are translated to the ray origin
//    and sheared so that the ray runs along +z; the hit is decided by the
//    signs of the three 2-D edge functions U, V, W.  Each edge function
//    depends only on its edge's two sheared vertices, and its sign is
//    computed exactly (below), so a ray that crosses an edge shared by two
//    triangles hits at least one of them: no ray leaks through a mesh.
//  * accurate distance: t = dot(n, v0 - o) / dot(n, d) with n = e1 x e2,
//    every difference of inputs exact (two-term "double-float" values built
//    with error-free transformations), the dot products compensated, and the
//    quotient corrected by its exact remainder.  The fp32 t is within about
//    one ulp of the exact intersection of the fp32 ray with the fp32
//    triangle.
//  * accurate barycentrics: the hit point relative to v0, q = t d - (v0 - o),
//    in double-float from the double-float t, then u, v by Cramer's rule in
//    the projection that drops the normal's largest axis (whose 2x2
//    determinant is that component of n).
//
// Exact sign of a*b - c*d: p1 = fl(a*b) and p2 = fl(c*d) are rounded
// monotonically, so fl(p1 - p2) != 0 has the sign of a*b - c*d; when it is
// 0 (p1 == p2) the exact value is (a*b - p1) - (c*d - p2), two exact fma
// residues whose rounded difference keeps the sign.  Swapping the edge's
// vertices swaps the two products, which negates the result exactly, so two
// triangles see one shared edge with opposite signs.
//
// The box test (Ize, "Robust BVH Ray Traversal", JCGT 2013): slab distances
// (p - o) * inv with inv = 1 / d rounded once (no clamping of small
// components; 1 / 0 = inf, and a NaN plane -- a ray lying in it -- is ignored
// by min / max), and the far distance scaled by 1 + 2 gamma_3, which bounds
// the three roundings of each distance.  A box that the exact ray segment
// [min_t, closest t] touches is never culled, so the closest hit does not
// depend on the tree or the visit order, except between triangles hit at
// exactly the same t.
//
// The CPU oracle restates the same operations in the same order
// (oracle/rr_oracle.cpp, precise_*), so hits are bit-identical to it.
#pragma once
#include "trace_common.cuh"

namespace rr
{
// 1 + 2 gamma_3 with gamma_3 = 3u / (1 - 3u), u = 2^-24, rounded up.
constexpr float kRobustFar = 1.00000036f;

struct DF
{
    float h, l;
};

__device__ __forceinline__ DF two_sum(float a, float b)
{
    const float s  = a + b;
    const float bb = s - a;
    return DF{s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ DF two_diff(float a, float b)
{
    const float s  = a - b;
    const float bb = s - a;
    return DF{s, (a - (s - bb)) - (b + bb)};
}
// |a| >= |b| (or a == 0).
__device__ __forceinline__ DF fast_two_sum(float a, float b)
{
    const float s = a + b;
    return DF{s, b - (s - a)};
}
__device__ __forceinline__ DF two_prod(float a, float b)
{
    const float p = a * b;
    return DF{p, fmaf(a, b, -p)};
}

// a*b - c*d with the exact sign (see the file comment).
__device__ __forceinline__ float exact_sign_dop(float a, float b, float c, float d)
{
    const float p1 = a * b, p2 = c * d;
    const float r  = p1 - p2;
    if (r != 0.0f) return r;
    return fmaf(a, b, -p1) - fmaf(c, d, -p2);
}

// a*b - c*d for double-float a, b, c, d, as a double-float.
__device__ __forceinline__ DF df_dop(DF a, DF b, DF c, DF d)
{
    const DF    p  = two_prod(a.h, b.h);
    const DF    q  = two_prod(c.h, d.h);
    const DF    s  = two_diff(p.h, q.h);
    const float lo = s.l + (p.l - q.l) + ((a.h * b.l + a.l * b.h) - (c.h * d.l + c.l * d.h));
    return fast_two_sum(s.h, lo);
}

// Sum of three double-float products a_i * b_i (b_i possibly exact: l = 0).
__device__ __forceinline__ DF df_dot3(DF ax, DF ay, DF az, DF bx, DF by, DF bz)
{
    const DF    px = two_prod(ax.h, bx.h), py = two_prod(ay.h, by.h), pz = two_prod(az.h, bz.h);
    const DF    s1 = two_sum(px.h, py.h);
    const DF    s2 = two_sum(s1.h, pz.h);
    const float lx = px.l + (ax.h * bx.l + ax.l * bx.h);
    const float ly = py.l + (ay.h * by.l + ay.l * by.h);
    const float lz = pz.l + (az.h * bz.l + az.l * bz.h);
    const float lo = ((s1.l + s2.l) + lx) + (ly + lz);
    return fast_two_sum(s2.h, lo);
}

// n / d for double-float n, d (d.h != 0): fp32 quotient plus the correction
// from its exact remainder, as a double-float.
__device__ __forceinline__ DF df_div(DF n, DF d)
{
    const float q = n.h / d.h;
    const float r = fmaf(-q, d.h, n.h) + (n.l - q * d.l);
    return fast_two_sum(q, r / d.h);
}

// The triangle's exact edges and origin offset, and its normal n = e1 x e2.
struct PreciseTri
{
    DF wx, wy, wz;     // v0 - o
    DF e1x, e1y, e1z;  // v1 - v0
    DF e2x, e2y, e2z;  // v2 - v0
    DF nx, ny, nz;
};
__device__ __forceinline__ PreciseTri precise_setup(const Ray& r, F3 v0, F3 v1, F3 v2)
{
    PreciseTri p;
    p.wx  = two_diff(v0.x, r.o.x);
    p.wy  = two_diff(v0.y, r.o.y);
    p.wz  = two_diff(v0.z, r.o.z);
    p.e1x = two_diff(v1.x, v0.x);
    p.e1y = two_diff(v1.y, v0.y);
    p.e1z = two_diff(v1.z, v0.z);
    p.e2x = two_diff(v2.x, v0.x);
    p.e2y = two_diff(v2.y, v0.y);
    p.e2z = two_diff(v2.z, v0.z);
    p.nx  = df_dop(p.e1y, p.e2z, p.e1z, p.e2y);
    p.ny  = df_dop(p.e1z, p.e2x, p.e1x, p.e2z);
    p.nz  = df_dop(p.e1x, p.e2y, p.e1y, p.e2x);
    return p;
}

// t = dot(n, v0 - o) / dot(n, d) as a double-float; ok = false when the ray
// is parallel to the plane (dot(n, d) == 0).
__device__ __forceinline__ DF precise_t(const PreciseTri& p, const Ray& r, bool& ok)
{
    const DF z  = DF{0.f, 0.f};
    const DF N  = df_dot3(p.nx, p.ny, p.nz, p.wx, p.wy, p.wz);
    const DF D  = df_dot3(p.nx, p.ny, p.nz, DF{r.d.x, 0.f}, DF{r.d.y, 0.f}, DF{r.d.z, 0.f});
    ok          = D.h != 0.0f;
    return ok ? df_div(N, D) : z;
}

// Watertight decision, then the accurate distance.  Same contract as
// isect_tri: the distance of a hit in [min_t, t_max], else t_max.
__device__ __forceinline__ float isect_tri_precise(const Ray& r, F3 v0, F3 v1, F3 v2, float t_max)
{
    // Ray-dependent shear (per test: the kernels keep no extra ray state).
    const float adx = fabsf(r.d.x), ady = fabsf(r.d.y), adz = fabsf(r.d.z);
    const int   kz  = (adx >= ady && adx >= adz) ? 0 : (ady >= adz ? 1 : 2);
    int         kx  = kz == 2 ? 0 : kz + 1;
    int         ky  = kx == 2 ? 0 : kx + 1;
    const float d3[3] = {r.d.x, r.d.y, r.d.z};
    if (d3[kz] < 0.0f)
    {
        const int k = kx;
        kx          = ky;
        ky          = k;
    }
    const float sx = d3[kx] / d3[kz], sy = d3[ky] / d3[kz];
    const float o3[3] = {r.o.x, r.o.y, r.o.z};
    const float a3[3] = {v0.x - o3[0], v0.y - o3[1], v0.z - o3[2]};
    const float b3[3] = {v1.x - o3[0], v1.y - o3[1], v1.z - o3[2]};
    const float c3[3] = {v2.x - o3[0], v2.y - o3[1], v2.z - o3[2]};
    const float ax = a3[kx] - sx * a3[kz], ay = a3[ky] - sy * a3[kz];
    const float bx = b3[kx] - sx * b3[kz], by = b3[ky] - sy * b3[kz];
    const float cx = c3[kx] - sx * c3[kz], cy = c3[ky] - sy * c3[kz];
    const float U = exact_sign_dop(cx, by, cy, bx);
    const float V = exact_sign_dop(ax, cy, ay, cx);
    const float W = exact_sign_dop(bx, ay, by, ax);
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return t_max;
    if (U + V + W == 0.0f) return t_max;
    bool             ok;
    const PreciseTri p = precise_setup(r, v0, v1, v2);
    const DF         t = precise_t(p, r, ok);
    if (!ok || !(t.h >= r.tmin) || t.h > t_max) return t_max;
    return t.h;
}

// Barycentrics (u: weight of v1, v: weight of v2) of the ray's hit point on
// the triangle's plane: q = t d - (v0 - o) in double-float, then Cramer's
// rule in the projection that drops the normal's largest axis.
__device__ __forceinline__ float2 barycentrics_precise(const Ray& r, F3 v0, F3 v1, F3 v2)
{
    bool             ok;
    const PreciseTri p = precise_setup(r, v0, v1, v2);
    const DF         t = precise_t(p, r, ok);
    if (!ok) return make_float2(0.f, 0.f);
    auto q_of = [&](float d, DF w) {
        DF          pr = two_prod(t.h, d);
        const DF    s  = two_diff(pr.h, w.h);
        const float lo = s.l + ((pr.l + t.l * d) - w.l);
        return fast_two_sum(s.h, lo);
    };
    const DF    qx = q_of(r.d.x, p.wx), qy = q_of(r.d.y, p.wy), qz = q_of(r.d.z, p.wz);
    const float anx = fabsf(p.nx.h), any = fabsf(p.ny.h), anz = fabsf(p.nz.h);
    DF          qa, qb, e1a, e1b, e2a, e2b, det;
    if (anz >= anx && anz >= any)
    {
        qa = qx, qb = qy, e1a = p.e1x, e1b = p.e1y, e2a = p.e2x, e2b = p.e2y, det = p.nz;
    }
    else if (anx >= any)
    {
        qa = qy, qb = qz, e1a = p.e1y, e1b = p.e1z, e2a = p.e2y, e2b = p.e2z, det = p.nx;
    }
    else
    {
        qa = qz, qb = qx, e1a = p.e1z, e1b = p.e1x, e2a = p.e2z, e2b = p.e2x, det = p.ny;
    }
    if (det.h == 0.0f) return make_float2(0.f, 0.f);
    const DF u = df_div(df_dop(qa, e2b, qb, e2a), det);
    const DF v = df_div(df_dop(e1a, qb, e1b, qa), det);
    return make_float2(u.h, v.h);
}

// The far distance moved outward by 2 gamma_3 of its magnitude.
__device__ __forceinline__ float robust_far(float t1) { return t1 * (t1 >= 0.0f ? kRobustFar : 2.0f - kRobustFar); }

// Conservative slab test of a box: hit iff t0 <= t1.
__device__ __forceinline__ void isect_box_robust(F3 lo, F3 hi, F3 inv, F3 o, float tmax_, float tmin_, float& t0,
                                                 float& t1)
{
    const float fx = (hi.x - o.x) * inv.x, fy = (hi.y - o.y) * inv.y, fz = (hi.z - o.z) * inv.z;
    const float nx = (lo.x - o.x) * inv.x, ny = (lo.y - o.y) * inv.y, nz = (lo.z - o.z) * inv.z;
    t1 = robust_far(fminf(fminf(fmaxf(fz, nz), fminf(fmaxf(fx, nx), fmaxf(fy, ny))), tmax_));
    t0 = fmaxf(fmaxf(fminf(fz, nz), fmaxf(fminf(fx, nx), fminf(fy, ny))), tmin_);
}

__device__ __forceinline__ F3 exact_invdir(F3 d) { return f3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z); }

// Full hit of the precise test.
template <bool kFull>
__device__ __forceinline__ void write_hit_precise(void* hits, uint32_t gid, const Ray& r, F3 v0, F3 v1, F3 v2,
                                                  uint32_t inst, uint32_t prim, uint32_t id_out)
{
    if (kFull)
    {
        const float2 uv = barycentrics_precise(r, v0, v1, v2);
        reinterpret_cast<uint4*>(hits)[gid] = make_uint4(__float_as_uint(uv.x), __float_as_uint(uv.y), inst, prim);
    }
    else
        reinterpret_cast<uint32_t*>(hits)[gid] = id_out;
}

}  // namespace rr
