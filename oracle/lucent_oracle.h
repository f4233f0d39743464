/*
 * Lucent oracle: a CPU restatement of the reference's BVH, ray and lighting
 * arithmetic, used ONLY as the checker by tests/, by __graft_entry__.smoke()
 * and by bench.py's CPU-baseline leg. Nothing in the product links or calls it.
 *
 * Numerics follow JavaScript: every `number` is an IEEE binary64, every store
 * into a Float32Array rounds to binary32. The file is compiled with
 * -ffp-contract=off -fno-fast-math so no fused multiply-add changes a result.
 *
 * Every function cites the reference file:line it restates.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes shared with the product ABI's convention: 0 = OK. */
#define ORC_OK 0
#define ORC_ERR_INVALID 1
#define ORC_ERR_STACK 6

/* buildBVH (src/math/bvh.ts:52-252). `n_floats` must be a multiple of 9
 * (bvh.ts:54-57). nodes_out holds max(1, 2N-1)*8 floats, tri_out N u32.
 * bounds_out = [minx,miny,minz,maxx,maxy,maxz]. */
int orc_build_bvh(const float* positions, uint64_t n_floats, int max_leaf, int bins,
                  float* nodes_out, uint32_t* node_count_out, uint32_t* tri_out, double* bounds_out);

/* Maximum depth (root = 0) of a flattened BVH; -1 if malformed. */
int orc_bvh_depth(const float* nodes, uint32_t node_count);

/* intersectBVH (src/math/bvh.ts:265-320) over n rays given as 6 doubles
 * (origin xyz, dir xyz). Misses write id -1 and t = +inf. Uses `threads`
 * std::threads (0 = all cores). Returns ORC_ERR_STACK if a traversal would
 * overflow the reference's 64-entry stack. */
int orc_intersect_bvh(const float* nodes, uint32_t node_count, const uint32_t* tri, uint32_t tri_count,
                      const float* positions, const double* rays, uint64_t n, double t_min, double t_max,
                      int32_t* id_out, double* t_out, double* u_out, double* v_out, int threads);

/* Same, rays given as 6 floats each (converted exactly to double). Also
 * counts node visits and triangle tests per ray in the reference's own
 * left-first order when the count arrays are non-null. */
int orc_intersect_bvh_f32(const float* nodes, uint32_t node_count, const uint32_t* tri, uint32_t tri_count,
                          const float* positions, const float* rays, uint64_t n, double t_min, double t_max,
                          int32_t* id_out, double* t_out, double* u_out, double* v_out, int threads);

/* Nodes popped / triangles tested per ray in intersectBVH's own order. */
int orc_ts_traversal_counts(const float* nodes, const uint32_t* tri, uint32_t tri_count, const float* positions,
                            const float* rays, uint64_t n, double t_min, double t_max, uint32_t* popped_out,
                            uint32_t* tests_out, int threads);

/* intersectAllTriangles (src/math/bvh.ts:323-348), brute force. */
int orc_intersect_all(const float* positions, uint32_t tri_count, const double* rays, uint64_t n,
                      double t_min, double t_max, int32_t* id_out, double* t_out, double* u_out,
                      double* v_out, int threads);

/* intersectTriangle (src/math/ray.ts:22-45). Returns 1 on hit. */
int orc_intersect_triangle(const double* origin, const double* dir, const double* v0, const double* v1,
                           const double* v2, double t_min, double t_max, double* t, double* u, double* v);

/* intersectSphere (src/math/ray.ts:48-67). Returns 1 on hit. */
int orc_intersect_sphere(const double* origin, const double* dir, const double* center, double radius,
                         double t_min, double t_max, double* t);

/* AABB.intersect (src/math/aabb.ts:84-98): entry distance or +inf. */
double orc_aabb_intersect(const double* bmin, const double* bmax, const double* origin,
                          const double* inv_dir, double t_max);

/* Per-ray work counts under the GLSL traversal order (src/shaders/scene.glsl:
 * 218-267, near-first with both child boxes read per inner node, f32):
 * inner nodes visited and triangles tested. Used for algorithmic bytes. */
int orc_glsl_traversal_counts(const float* nodes, uint32_t node_count, const float* positions_leaf_order,
                              uint32_t tri_count, const float* rays, uint64_t n, float t_min,
                              uint32_t* inner_out, uint32_t* tris_out, int32_t* slot_out, int threads);

/* buildAliasTable (src/math/alias.ts:17-65). prob f32, alias u32, pmf f64.
 * Returns ORC_ERR_INVALID for an empty or negative / non-finite weight list. */
int orc_build_alias(const double* weights, uint32_t n, float* prob, uint32_t* alias, double* pmf,
                    double* total);

/* buildEnvSampler (src/scene/environment.ts:52-85): writes gw*gh*4 floats. */
int orc_build_env_sampler(const float* rgb, uint32_t width, uint32_t height, uint32_t max_width,
                          uint32_t* gw, uint32_t* gh, float* table, double* total);

/* bakeSky (src/scene/environment.ts:106-132): width x width/2 x 3 floats. */
void orc_bake_sky(uint32_t width, const double* zenith, const double* horizon, const double* ground,
                  double intensity, int enabled, double sun_elevation_deg, double sun_azimuth_deg,
                  const double* sun_color, double sun_intensity, double sun_angular_radius_deg, float* out);

/* sheenAlbedo / sheenAlbedoLUT (src/scene/sheen.ts:24-60). */
double orc_sheen_albedo(double cos_v, double roughness, int steps);
void orc_sheen_lut(int size, int steps, float* out);

#ifdef __cplusplus
}
#endif
