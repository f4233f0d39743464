/*
 * Lucent GB300 C ABI.
 *
 * A drop-in for the hot path of Lucent (a TypeScript/WebGL2 path tracer): the
 * BVH builder and CPU pick-ray intersector of src/math/bvh.ts, and the
 * renderer passes of src/renderer.ts. Plain pointers and sizes only; every
 * call returns a lucent_status (0 = OK) and, on failure, leaves a message for
 * lucent_last_error() in the calling thread. `stream` is a cudaStream_t (NULL
 * = the legacy default stream). Functions taking host buffers copy in, run,
 * copy out and synchronise; `_device` variants take device pointers and are
 * asynchronous on `stream`.
 */
#ifndef LUCENT_H
#define LUCENT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t lucent_status;
#define LUCENT_OK 0
#define LUCENT_ERR_INVALID 1     /* bad argument (the reference throws Error) */
#define LUCENT_ERR_CUDA 2        /* a CUDA runtime call failed */
#define LUCENT_ERR_OOM 3         /* device allocation failed */
#define LUCENT_ERR_DEVICE 4      /* a kernel raised its error word (stack, queue, iteration cap) */
#define LUCENT_ERR_UNSUPPORTED 5 /* input outside the documented limits */

/* Message of the last failed call on this thread ("" if none). */
const char* lucent_last_error(void);
/* ABI version: major * 10000 + minor * 100 + patch. */
int32_t lucent_version(void);

/* ---------------------------------------------------------------------------
 * BVH build: buildBVH (src/math/bvh.ts:52-252) and buildBVHAsync
 * (src/math/bvh-async.ts:8-31). Binned SAH on the GPU; the node array and the
 * triangle order equal the reference's bit for bit.
 * ------------------------------------------------------------------------- */
typedef struct lucent_bvh_opts {
  uint32_t max_leaf_size; /* BVHOptions.maxLeafSize, default 4 (bvh.ts:33) */
  uint32_t bins;          /* BVHOptions.bins, default 12 (bvh.ts:33); at most 32 */
} lucent_bvh_opts;

typedef struct lucent_bvh lucent_bvh;

/* buildBVH(positions, opts) (bvh.ts:52). `positions` = n_floats host floats,
 * 9 per triangle (n_floats % 9 != 0 fails as in bvh.ts:55-57; non-finite
 * values and more than 2^23 triangles are rejected). `opts` may be NULL for
 * the reference's defaults. Outputs (each may be NULL): nodes_out holds
 * max(1, 2N-1) * 8 floats (the reference's allocation, bvh.ts:79),
 * tri_indices_out N u32, bounds_out 6 doubles [min.xyz, max.xyz]. When
 * handle_out is non-NULL the built BVH also stays on the device as a
 * lucent_bvh ready for lucent_bvh_intersect (no re-upload). Node bounds equal
 * the reference's as numbers (the sign of a zero bound is not reproduced). */
lucent_status lucent_bvh_build(const float* positions, uint64_t n_floats, const lucent_bvh_opts* opts,
                               float* nodes_out, uint32_t* node_count_out, uint32_t* tri_indices_out,
                               double* bounds_out, lucent_bvh** handle_out, void* stream);
/* Same over device-resident positions (9 floats per triangle); creates the
 * device BVH only. The replacement for buildBVHAsync (bvh-async.ts:8): the
 * build never runs on the calling CPU thread's critical path. */
lucent_status lucent_bvh_build_device(const float* positions_d, uint32_t tri_count, const lucent_bvh_opts* opts,
                                      lucent_bvh** handle_out, void* stream);
/* Copies a device BVH back in the reference's layout (buffers sized by the
 * caller: node_count * 8 floats, tri_count u32). */
lucent_status lucent_bvh_download(const lucent_bvh* bvh, float* nodes_out, uint32_t* tri_indices_out);

/* ---------------------------------------------------------------------------
 * Closest hit: intersectBVH (src/math/bvh.ts:265-320). Hit ids equal the
 * reference's on identical rays; t, u, v are the reference's binary64 values
 * rounded to binary32.
 * ------------------------------------------------------------------------- */

/* Uploads a BVH in the reference's layout: `nodes` = node_count * 8 floats
 * [min.xyz, leftFirst, max.xyz, count] (bvh.ts:6-16), `tri_indices` = the
 * reference's triIndices, `positions` = 9 floats per triangle in the original
 * order. Replaces the BVH + positions pair passed to intersectBVH (bvh.ts:265). */
lucent_status lucent_bvh_create(const float* nodes, uint32_t node_count, const uint32_t* tri_indices,
                                uint32_t tri_count, const float* positions, lucent_bvh** out);
void lucent_bvh_destroy(lucent_bvh* bvh);
/* Node and triangle counts of an uploaded BVH. */
lucent_status lucent_bvh_info(const lucent_bvh* bvh, uint32_t* node_count, uint32_t* tri_count);
/* Traversal mode: 0 = f32 bounded-error path with binary64 fallback (default),
 * 1 = every decision in binary64. Both return identical results. */
#define LUCENT_TRAVERSE_FAST 0
#define LUCENT_TRAVERSE_EXACT 1
lucent_status lucent_bvh_set_mode(lucent_bvh* bvh, int32_t mode);

/* n rays, 6 floats each (origin xyz, direction xyz), host buffers. t_min and
 * t_max as in intersectBVH(bvh, positions, ray, tMin = 1e-5, tMax = Infinity).
 * prim_out[i] = source triangle index or -1 on a miss; t_out is +inf on a miss.
 * t_out, u_out, v_out may be NULL. */
lucent_status lucent_bvh_intersect(lucent_bvh* bvh, const float* rays, uint32_t n, double t_min, double t_max,
                                   int32_t* prim_out, float* t_out, float* u_out, float* v_out, void* stream);
/* Same with device pointers; asynchronous. Errors raised by the kernels are
 * reported by lucent_bvh_check(). */
lucent_status lucent_bvh_intersect_device(lucent_bvh* bvh, const float* rays_d, uint32_t n, double t_min,
                                          double t_max, int32_t* prim_d, float* t_d, float* u_d, float* v_d,
                                          void* stream);
/* Synchronises `stream` and reports (then clears) the device error word. */
lucent_status lucent_bvh_check(lucent_bvh* bvh, void* stream);
/* Rays as 6 doubles each (the reference's binary64 Ray, src/math/ray.ts:4-7),
 * host buffers; t, u, v returned in binary64. Used for pick rays. */
lucent_status lucent_bvh_intersect_f64(lucent_bvh* bvh, const double* rays, uint32_t n, double t_min,
                                       double t_max, int32_t* prim_out, double* t_out, double* u_out,
                                       double* v_out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* LUCENT_H */
