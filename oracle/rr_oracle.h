/* rr_oracle.h -- CPU oracle of the RadeonRays BVH build + traversal path.
 * Test infrastructure only (see rr_oracle.cpp). */
#ifndef RR_ORACLE_H
#define RR_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 64-byte binary node, vlk/kernels/bvh2.h:25-35. */
typedef struct
{
    float    aabb0_min_or_v0[3];
    uint32_t child0;
    float    aabb0_max_or_v1[3];
    uint32_t child1;
    float    aabb1_min_or_v2[3];
    uint32_t parent;
    float    aabb1_max_or_v3[3];
    uint32_t update;
} rro_node;

typedef struct
{
    float origin[3];
    float min_t;
    float direction[3];
    float max_t;
} rro_ray;

typedef struct
{
    float    uv[2];
    uint32_t inst_id;
    uint32_t prim_id;
} rro_hit;

int  rro_version(void);
void rro_mesh_aabb(const float* vertices, uint32_t vertex_stride, const void* indices, int index16, uint32_t ntri,
                   uint32_t out[8]);
void rro_morton(const float* vertices, uint32_t vertex_stride, const void* indices, int index16, uint32_t ntri,
                const uint32_t aabb[8], int bits, void* codes);
void rro_sort32(const uint32_t* codes, uint32_t n, uint32_t* sorted_codes, uint32_t* sorted_idx);
void rro_sort64(const uint64_t* codes, uint32_t n, uint64_t* sorted_codes, uint32_t* sorted_idx);
void rro_emit(const void* sorted_codes, int bits, const uint32_t* sorted_idx, uint32_t n, rro_node* nodes,
              int threads);
uint32_t rro_restructure(rro_node* nodes, uint32_t n, uint32_t min_prims, int passes);
/* rro_trace with box leaves (AABB-list geometry) when box_leaves != 0. */
void rro_trace_leaves(const rro_node* nodes, uint32_t n_nodes, const rro_ray* rays, uint32_t nrays, int query,
                      int output, void* hits, uint64_t* fetches, int threads, int box_leaves);
void rro_fit(const float* vertices, uint32_t vertex_stride, const void* indices, int index16, uint32_t n,
             rro_node* nodes);
void rro_build_mesh(const float* vertices, uint32_t vertex_stride, const void* indices, int index16, uint32_t n,
                    int bits, rro_node* nodes, uint32_t* out_sorted_idx, void* out_sorted_codes, int threads);
void rro_trace(const rro_node* nodes, uint32_t n_nodes, const rro_ray* rays, uint32_t nrays, int query, int output,
               void* hits, uint64_t* fetches, int threads);
void rro_build_scene(const rro_node* const* blas_roots, const uint32_t* blas_leaf_counts, const float* transforms,
                     uint32_t count, rro_node* out_nodes, float* out_xforms);
void rro_trace_scene(const rro_node* tlas, const float* xforms, const rro_node* const* blas, const rro_ray* rays,
                     uint32_t nrays, int query, int output, void* hits, int threads);
void rro_fp64_hit(const rro_ray* rays, const float* tri9, const uint32_t* valid, uint32_t nrays, double* out_tuv);
void rro_trace_t(const rro_node* nodes, uint32_t n_nodes, const rro_ray* rays, uint32_t nrays, float* out_t,
                 int threads);
void rro_tri_test(const rro_ray* rays, const float* tri9, uint32_t nrays, float* out_tuv);
/* The precise triangle test (watertight decision, accurate t and uv, robust
 * box test): traversal in the reference's visit order, and the test alone. */
void rro_trace_precise(const rro_node* nodes, uint32_t n_nodes, const rro_ray* rays, uint32_t nrays, int query,
                       int output, void* hits, float* out_t, int threads);
void rro_tri_test_precise(const rro_ray* rays, const float* tri9, uint32_t nrays, float* out_tuv);

#ifdef __cplusplus
}
#endif
#endif
