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
/* Traversal mode: 0 = f32 bounded-error path with binary64 fallback and the
 * top six BVH levels staged in shared memory, 1 = every decision in binary64,
 * 2 = mode 0 reading every node from global memory, 3 = mode 0's decisions
 * over a four-wide view of the tree (each inner step reads a node's four
 * grandchildren; built on first use, 128 bytes per node; the default). All
 * return identical results. lucent_bvh_intersect_noalloc always uses 0. */
#define LUCENT_TRAVERSE_FAST 0
#define LUCENT_TRAVERSE_EXACT 1
#define LUCENT_TRAVERSE_FAST_GLOBAL 2
#define LUCENT_TRAVERSE_WIDE 3
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

/* Closest hit that allocates no device memory. It has no counterpart in the
 * reference: it exists for callers that may not call cudaMalloc (a host whose
 * own allocator owns the device's memory, a loop that must not take the
 * allocator's implicit synchronisation, a plugin whose host owns every
 * allocation). Inputs and outputs are the caller's device buffers:
 *   nodes_d   node_count nodes of 8 floats: min.xyz, leftFirst, max.xyz, count,
 *             with leftFirst and count stored as int32 bit patterns (the
 *             reference's layout, bvh.ts:6-16, with integer fields);
 *   tris_d    tri_count triangles in BVH leaf (slot) order, 12 floats each:
 *             v0.xyz, source index as int32 bits, v1.xyz, 0, v2.xyz, 0;
 *   rays_d    n rays of 6 floats; prim/t/u/v as in lucent_bvh_intersect.
 * The kernels' scratch is a file-scope device array of 4 MiB + 256 B that
 * every GPU loading the library keeps until exit, so n is limited to
 * 1,048,576 rays per call (larger n fails with LUCENT_ERR_UNSUPPORTED). All
 * calls share that array: calls that overlap on the GPU (other threads, other
 * streams) race on it and must be serialised by the caller. Every call looks
 * up the array's device address with the calling thread's current device.
 * The tree is checked on the device before any traversal reads it (children
 * inside the node array and after their parent, leaf ranges inside the
 * triangle array, finite bounds, source indices below tri_count); a tree that
 * fails returns LUCENT_ERR_INVALID naming the first bad record, and nothing
 * is written to the outputs. With tri_count == 0 every ray misses: prim = -1,
 * t = +inf, u = v = 0. The call returns after the work completes (it
 * synchronises `stream`) and reports kernel errors like lucent_bvh_check. */
lucent_status lucent_bvh_intersect_noalloc(const float* nodes_d, uint32_t node_count, const float* tris_d,
                                           uint32_t tri_count, const float* rays_d, uint32_t n, double t_min,
                                           double t_max, int32_t* prim_d, float* t_d, float* u_d, float* v_d,
                                           void* stream);

/* ---------------------------------------------------------------------------
 * Renderer: the Renderer class of src/renderer.ts:171-871 without its WebGL
 * plumbing. Accumulation targets, scene data and the path state live on the
 * GPU; host buffers are copied in and out by the calls that take them.
 * ------------------------------------------------------------------------- */
typedef struct lucent_renderer lucent_renderer;

/* PackedScene inputs before the BVH-order gather (scene.ts:106-134, 162-305).
 * Per triangle in mergeMeshes order: positions (9 floats), normals (9),
 * optional uvs (6), material index, light index (-1 = none) and alpha-test
 * flag. The BVH is built on the GPU unless a reference-layout BVH over the
 * same triangles is supplied (packScene's `prebuilt`, scene.ts:206-209).
 * Materials are packed by packMaterials (40 floats each, material.ts:121-131);
 * texture maps must be -1 (texture layers are not part of this ABI).
 * Lights are 16 floats each (scene.ts:88-95), at most 8; spheres are
 * (centre, radius), at most 64. ground_material: the packed ground material
 * (the plane itself is switched by lucent_renderer_upload_ground). */
typedef struct lucent_scene_desc {
  uint32_t tri_count;
  const float* positions;
  const float* normals;
  const float* uvs;
  const int32_t* tri_material;
  const int32_t* tri_light;
  const uint8_t* tri_alpha;
  const float* bvh_nodes;
  uint32_t bvh_node_count;
  const uint32_t* bvh_tri_indices;
  const float* materials;
  uint32_t material_count;
  const float* spheres;
  const int32_t* sphere_materials;
  const int32_t* sphere_lights;
  uint32_t sphere_count;
  const float* lights;
  uint32_t light_count;
  int32_t ground_material;
  /* Texture maps (SceneTexture, scene.ts:58-62; buildTextureArrays,
   * renderer.ts:314-333). texture_count decoded images of 8-bit RGBA, rows
   * top to bottom (texture_rgba8[i] holds texture_width[i] *
   * texture_height[i] * 4 bytes). color_layers / data_layers: the scene
   * texture index of each layer of the sRGB (base colour, emissive) and
   * linear (metal-rough, normal) arrays; the material map fields (texel 4)
   * hold layer indices (packScene, scene.ts:271-283). All may be 0 / NULL. */
  uint32_t texture_count;
  const uint8_t* const* texture_rgba8;
  const uint32_t* texture_width;
  const uint32_t* texture_height;
  const int32_t* color_layers;
  uint32_t color_layer_count;
  const int32_t* data_layers;
  uint32_t data_layer_count;
} lucent_scene_desc;

/* uploadLighting (renderer.ts:355-413): the analytic sun and an equirect
 * radiance map (RGB floats, rows top to bottom). The map's importance
 * sampler (buildEnvSampler, environment.ts:52-85, max grid width 1024) is
 * built here. A map whose luminance sums to 0 disables environment sampling. */
typedef struct lucent_lighting {
  int32_t sun_enabled;
  float sun_dir[3];
  float sun_radiance[3];
  float sun_cos_angle;
  float sun_pdf;
  uint32_t env_width, env_height;
  const float* env_rgb;
  float env_rotation_cos, env_rotation_sin;
  float env_intensity;
  int32_t env_background;
  float backdrop[3];
} lucent_lighting;

/* uploadCamera (renderer.ts:424-439): basis already normalised. */
typedef struct lucent_camera {
  float position[3], right[3], up[3], forward[3];
  float tan_half_fov, aperture, focus_distance;
} lucent_camera;

/* applySettings (renderer.ts:454-460): RenderSettings.maxBounces /
 * fireflyClamp / temporal (reproject the history when the camera moves,
 * renderer.ts:441-451; the reference's default is on). */
typedef struct lucent_settings {
  uint32_t max_bounces;
  float firefly_clamp;
  int32_t temporal;
} lucent_settings;

/* stats() (renderer.ts:832-854) plus ray counters. */
typedef struct lucent_render_stats {
  uint32_t samples;        /* samples behind the current average (frame) */
  uint32_t seed;           /* next RNG stream index (uSeed) */
  uint32_t width, height;
  uint32_t triangles, bvh_nodes;
  uint64_t closest_rays;   /* closest-hit rays traced since creation */
  uint64_t shadow_rays;    /* shadow rays traced since creation */
  double last_trace_ms;    /* device time of the last lucent_renderer_trace */
  /* device ms of the last trace per phase (camera, closest hit, shade, shadow
   * rays, resolve + queue upkeep, accumulate); zero unless profiling is on */
  double phase_ms[6];
  /* closest-hit traversal counters accumulated while profiling is 2: rays,
   * slab tests decided in binary64, triangle tests decided in binary64,
   * binary64 recomputations of the running closest distance, binary64 final
   * hit reports */
  uint64_t traversal[5];
  /* kernels launched by lucent_renderer_reset and lucent_renderer_trace since
   * creation (a replayed wave graph counts the kernels it holds) */
  uint64_t kernel_launches;
} lucent_render_stats;

lucent_status lucent_renderer_create(uint32_t width, uint32_t height, lucent_renderer** out);
void lucent_renderer_destroy(lucent_renderer* r);
/* loadScene(scene, bvh?) (renderer.ts:279-312). */
lucent_status lucent_renderer_load_scene(lucent_renderer* r, const lucent_scene_desc* scene);
lucent_status lucent_renderer_upload_lighting(lucent_renderer* r, const lucent_lighting* lighting);
/* buildEnvSampler(img, maxWidth) (src/scene/environment.ts:52-85, with
 * buildAliasTable, src/math/alias.ts:17-65): the table upload_lighting builds
 * from an equirect RGB map (rows top to bottom). Host code, no device work.
 * Writes *gw, *gh, and (each may be NULL) gw * gh * 4 floats to `table`
 * (keep probability, alias cell, pdfUV, alias pdfUV) and the weight sum to
 * *total (0: a black map, light sampling off). */
lucent_status lucent_env_sampler(const float* rgb, uint32_t width, uint32_t height, uint32_t max_width, uint32_t* gw,
                                 uint32_t* gh, float* table, double* total);
/* buildEnvSampler on the GPU from a device RGB map (width * height * 3
 * floats, rows top to bottom): the same grid and table layout as
 * lucent_env_sampler, written to table_d (gw * gh * 4 floats, device). The
 * cell weights equal the reference's bit for bit; the total and the alias
 * pairing (Vose's stack order in closed form over prefix sums of the light
 * deficits and heavy excesses) use exact double-double scans where the
 * reference sums left to right in binary64, so keep probabilities may differ
 * from the host table by the reference's own rounding (about 1e-8); aliases
 * and pdf columns match, the table reproduces the pmf (alias.test's
 * criterion) and never draws a zero-weight cell. At most 1024 * 1024 cells. No reference counterpart (the
 * reference builds the table on the CPU, environment.ts:52-85); for hosts
 * whose map already lives on the device. Synchronises `stream`. */
lucent_status lucent_env_sampler_device(const float* rgb_d, uint32_t width, uint32_t height, uint32_t max_width,
                                        uint32_t* gw, uint32_t* gh, float* table_d, double* total, void* stream);
/* Replaces the renderer's environment map with a device RGB map and builds
 * its sampler on the GPU (lucent_env_sampler_device); the other lighting
 * uniforms stay as lucent_renderer_upload_lighting set them. Resets the
 * accumulation. For loops that change the map every step (inverse
 * rendering): no host round trip, no host alias build. Synchronous. */
lucent_status lucent_renderer_set_env_device(lucent_renderer* r, const float* rgb_d, uint32_t width, uint32_t height,
                                             void* stream);
/* Same from a host map (uploaded, sampler built on the GPU): what an
 * optimiser keeping the map in host memory calls every step. */
lucent_status lucent_renderer_set_env(lucent_renderer* r, const float* rgb, uint32_t width, uint32_t height,
                                      void* stream);
/* uploadGround (renderer.ts:415-421). */
lucent_status lucent_renderer_upload_ground(lucent_renderer* r, int32_t enabled, float height);
/* With temporal on and samples accumulated, the history is kept and the
 * first sample traced after the move reprojects it (trace.frag:275-322,
 * at most HISTORY_CAP = 8 samples of it per pixel); otherwise a reset. */
lucent_status lucent_renderer_upload_camera(lucent_renderer* r, const lucent_camera* camera);
lucent_status lucent_renderer_apply_settings(lucent_renderer* r, const lucent_settings* settings);
/* resize (renderer.ts:476-496): new accumulation targets, history cleared. */
lucent_status lucent_renderer_resize(lucent_renderer* r, uint32_t width, uint32_t height);
/* reset (renderer.ts:463-473). The RNG stream index is not reset (it never is). */
lucent_status lucent_renderer_reset(lucent_renderer* r);
/* Sets the next RNG stream index (uSeed); the reference starts at 0. */
lucent_status lucent_renderer_set_seed(lucent_renderer* r, uint32_t seed);
/* traceSamples(count) (renderer.ts:702-737): `samples` more samples per
 * pixel into the running average. Asynchronous on `stream`: the samples are
 * in the targets for work queued on `stream` after the call. With pipelining
 * (lucent_renderer_set_pipelining, default on) the paths themselves are
 * traced on the renderer's own streams and may start before work queued on
 * `stream` earlier; they read only the renderer's scene, lighting, camera and
 * settings, and the calls that change those wait for the waves in flight. */
lucent_status lucent_renderer_trace(lucent_renderer* r, uint32_t samples, void* stream);
/* Synchronises and reports the device error word. */
lucent_status lucent_renderer_check(lucent_renderer* r, void* stream);
/* Copies the accumulation targets to the host (each may be NULL):
 * color4 / albedo4 / normal4 as width*height*4 floats, history width*height.
 * Row 0 is the bottom row (gl_FragCoord convention). */
lucent_status lucent_renderer_read(lucent_renderer* r, float* color4, float* albedo4, float* normal4, float* history);
/* Queues a copy of the colour target (width*height*4 floats, as
 * lucent_renderer_read) to host memory on `stream` and returns without
 * waiting; color4 must stay valid until the stream reaches the copy (pinned
 * memory keeps the copy asynchronous). The counterpart of the reference's
 * asynchronous readback; lucent_renderer_check(stream) waits for it. */
lucent_status lucent_renderer_read_color_async(lucent_renderer* r, float* color4, void* stream);
lucent_status lucent_renderer_stats(lucent_renderer* r, lucent_render_stats* out);
/* Records CUDA events between the kernels of each trace (the counterpart of
 * the reference's GPU timer queries, renderer.ts:668-700); results appear in
 * lucent_render_stats.phase_ms after lucent_renderer_check. enabled = 2 also
 * counts the closest-hit traversal's binary64 decisions
 * (lucent_render_stats.traversal); the counters are atomics on a few words
 * and slow the closest-hit kernel down, so phase times taken with them are
 * not the kernel's own. */
lucent_status lucent_renderer_set_profiling(lucent_renderer* r, int32_t enabled);
/* Ray capture for parity checks of the traversal inside the renderer (no
 * reference counterpart; the reference's shader traversal cannot be read
 * back either). For every bounce b with bit b set in bounce_mask, the traces
 * that follow copy the bounce's closest-hit rays with their hits and its
 * shadow rays with their answers, at most max_rays of each per bounce, from
 * the last wave traced (a trace of W * H * samples <= 2^23 paths is one
 * wave). Waves launch directly while capture is on (no graph replay); images
 * are unchanged. bounce_mask = 0 turns capture off and frees its memory
 * (64 bytes per ray, two regions per bounce). */
lucent_status lucent_renderer_capture_rays(lucent_renderer* r, uint32_t bounce_mask, uint32_t max_rays);
/* Synchronises the legacy stream and copies the captured rays of `bounce`,
 * 16 floats per ray, in queue order (out16 may be NULL; at most cap rays);
 * *count = the bounce's queue length (may exceed what was captured).
 * shadow = 0: closest-hit rays (origin xyz, path id bits, direction xyz,
 * scene bits, hit t, u, v, BVH slot bits (-1 = no triangle hit), alpha key
 * bits, 0, 0, 0). shadow = 1: shadow rays (origin xyz, t_max, direction xyz,
 * alpha key bits, occluded (0/1), shadow slot bits, 0 x 6). */
lucent_status lucent_renderer_read_rays(lucent_renderer* r, uint32_t bounce, int32_t shadow, float* out16,
                                        uint32_t cap, uint32_t* count);
/* The texture arrays the scene's maps are sampled from (buildTextureArrays,
 * renderer.ts:314-333): *size = the layer size (0: no textures); color_out
 * and data_out (either may be NULL) receive color/data layer count x size x
 * size x 4 bytes (sRGB codes / linear codes), layers in packScene's order. */
lucent_status lucent_renderer_read_textures(lucent_renderer* r, uint32_t* size, uint8_t* color_out, uint8_t* data_out);
/* After bounces 0 and 1 (and 2 in waves of 2^21 paths or more), sort the
 * surviving rays by direction cell (cube-map face, 4 x 4 cells a face) and
 * origin cell (counting sort into a ray stream the closest-hit traversal
 * reads in order; default on). Paths are independent: images are the same
 * either way; only the traversal's coherence changes. */
lucent_status lucent_renderer_set_ray_sort(lucent_renderer* r, int32_t enabled);
/* Stage the top six BVH levels (63 nodes) in each traversal block's shared
 * memory (default on). Hits and images are the same either way; only where
 * the traversal reads those nodes changes. */
lucent_status lucent_renderer_set_top_levels(lucent_renderer* r, int32_t enabled);
/* Closest-hit rays over a four-wide view of the BVH (each inner step reads the
 * four grandchildren of a node; built at scene load, 128 bytes per binary
 * node; default on). Hits and images are the same either way: the
 * grandchildren's boxes lie inside their parents', so the reference's cull
 * decisions and visiting order are unchanged. */
lucent_status lucent_renderer_set_wide_bvh(lucent_renderer* r, int32_t enabled);
/* Pipelined waves (default on): successive waves (of one trace or of
 * successive traces) alternate between two path-state buffers and are traced
 * on the renderer's own streams, so one wave's last bounces (short launches
 * that leave most of the GPU idle) run beside the next wave's first bounces;
 * the accumulation stays on the caller's stream, in call order. Images are the
 * same either way. Costs a second path buffer (about 400 bytes per path of a
 * wave). Profiling and ray capture trace without it. */
lucent_status lucent_renderer_set_pipelining(lucent_renderer* r, int32_t enabled);
/* A renderer of width x height that renders `src`'s scene: geometry, BVH
 * and its wide view, triangle attributes, materials, spheres, lights and
 * texture arrays are read from src's device memory, not copied. The view
 * has its own targets, camera, settings, ground switch and lighting (call
 * lucent_renderer_upload_lighting on it). Materials are shared:
 * lucent_renderer_set_materials on src or any view changes them for all
 * (each renderer resets only its own average). src must keep its scene and
 * outlive its views; src cannot load another scene while views exist (a
 * view that loads a scene stops being a view). No reference counterpart:
 * the reference has one view per renderer; this serves many cameras of one
 * scene (multi-view inverse rendering, batches of views). */
lucent_status lucent_renderer_create_view(lucent_renderer* src, uint32_t width, uint32_t height, lucent_renderer** out);
/* ---------------------------------------------------------------------------
 * Differentiable rendering (path replay backpropagation). No reference
 * counterpart: the reference renders forward only.
 * ------------------------------------------------------------------------- */
/* Replaces the packed materials (count * 40 floats, packMaterials layout,
 * material.ts:121-149) of the loaded scene; count must equal the scene's
 * material count. Resets the accumulation. */
lucent_status lucent_renderer_set_materials(lucent_renderer* r, const float* materials, uint32_t count);
/* Gradient of  sum over pixels of dl_dimage[px] . I[px]  where I is the mean
 * of the `samples` samples starting at sample seed `seed` (what reset +
 * set_seed(seed) + trace(samples) renders), with respect to every material's
 * base colour (r, g, b), roughness, metallic and clearcoat (d_materials:
 * material_count * 6 floats, in that order) and, if d_env is non-NULL, to the
 * environment map's texels (env_width * env_height * 3 floats, rows top to
 * bottom). Both outputs are host buffers and are ADDED to. dl_dimage: host,
 * width * height * 4 floats (rgb used), rows bottom to top like the targets.
 * The samples are replayed from their seeds (twice: primal radiance, then the
 * adjoint), so memory is per wave, not per sample. Sampling is held fixed:
 * directions, pdfs, MIS weights, lobe and Russian-roulette choices, and the
 * firefly clamp's scale. The accumulation targets are left untouched.
 * Synchronous. */
lucent_status lucent_renderer_backward(lucent_renderer* r, uint32_t samples, uint32_t seed, const float* dl_dimage,
                                       float* d_materials, float* d_env, void* stream);
/* Frees the path-state buffers (about 315 bytes per path of the largest
 * wave traced so far); the next trace allocates them again. For hosts that
 * keep many renderers alive but trace one at a time. No reference
 * counterpart (WebGL owns the reference's render targets). */
lucent_status lucent_renderer_trim(lucent_renderer* r);

/* runDenoiser (renderer.ts:788-830; variance.frag, atrous.frag,
 * denoise.glsl): per-pixel variance of the demodulated illumination, then
 * `levels` (0..5) edge-avoiding a-trous iterations of spacing 1, 2, 4, 8, 16
 * guided by the albedo/normal/depth targets and the uploaded camera. The
 * reference passes levels = atrousLevels(frame) (renderer.ts:142) and sigma
 * L/N/P = 4, 64, 1.5. Asynchronous on `stream`; the result stays on the
 * device for lucent_renderer_display until the next reset or resize. */
lucent_status lucent_renderer_denoise(lucent_renderer* r, uint32_t levels, float sigma_l, float sigma_n,
                                      float sigma_p, void* stream);
/* Copies the last denoised illumination (width*height*4 floats: RGB,
 * variance) to the host; the filter targets the reference keeps in
 * `filtered`. */
lucent_status lucent_renderer_read_denoised(lucent_renderer* r, float* out4);
/* The display pass (renderer.ts:573-591, display.frag) at render size ==
 * view size: blend in the remodulated denoised image with `denoise_weight`
 * (denoiseWeight(frame), renderer.ts:144; 0 = raw), exposure, tone map
 * (0 ACES, 1 Reinhard, 2 none), sRGB, interleaved-gradient dither. Writes
 * the RGBA8 canvas (rows bottom to top) and/or the RGB floats before
 * quantization to host memory (either may be NULL); synchronous. */
lucent_status lucent_renderer_display(lucent_renderer* r, float denoise_weight, int32_t tonemap, float exposure,
                                      uint8_t* rgba8_out, float* rgb_out, void* stream);
/* The same display pass with the renderer's targets as the traced region
 * (uRenderSize) shown in a view_w x view_h canvas (uViewSize): when the sizes
 * differ, display.frag's Catmull-Rom upsampling (display.frag:44-60), the
 * reference's reduced-resolution preview while the camera moves
 * (renderer.ts:524-541). Outputs view_w * view_h pixels; otherwise as
 * lucent_renderer_display, which is this call at the renderer's size. */
lucent_status lucent_renderer_display_view(lucent_renderer* r, uint32_t view_w, uint32_t view_h, float denoise_weight,
                                           int32_t tonemap, float exposure, uint8_t* rgba8_out, float* rgb_out,
                                           void* stream);

/* ---------------------------------------------------------------------------
 * Multi-scene batches. No reference counterpart: the reference renders one
 * scene per WebGL context. A batch traces the next `samples` samples of
 * several renderers (each with its own scene, lighting, camera, settings and
 * targets) as one wavefront: every kernel of a bounce covers the paths of all
 * scenes, so small scenes and the short last bounces of each one share the
 * GPU. The result equals lucent_renderer_trace(r, samples) on each renderer
 * in turn, sample for sample and bit for bit (same kernels, same random
 * streams, same per-pixel accumulation order).
 * ------------------------------------------------------------------------- */
typedef struct lucent_batch lucent_batch;
typedef struct lucent_batch_options {
  uint32_t samples_per_wave; /* samples of every pixel per wave; 0 = as many as max_wave_paths allows */
  uint32_t max_wave_paths;   /* path-state budget of one wave (about 430 bytes of device memory per path) */
  int32_t use_graph;         /* capture a full wave once as a CUDA graph and replay it */
  uint32_t trace_blocks;     /* grid of the persistent traversal kernels; 0 = all resident blocks */
  uint32_t shade_blocks;     /* grid of the shade / resolve kernels; 0 = all resident blocks */
  int32_t sort_rays;         /* sort the rays of bounces 1 and 2 (see lucent_renderer_set_ray_sort) */
  int32_t top_levels;        /* top BVH levels of the first 8 scenes in shared memory (lucent_renderer_set_top_levels) */
  int32_t wide_bvh;          /* closest hit over the four-wide BVH views (lucent_renderer_set_wide_bvh) */
  uint32_t scenes_per_wave;  /* waves hold consecutive groups of this many scenes, each group traced for all
                                samples before the next (samples_per_wave / max_wave_paths then apply per
                                group); 0 = every scene in every wave */
  uint32_t streams;          /* 1..16: the renderers in this many consecutive parts, each traced as a batch
                                of its own (these options, path buffers of its own) on a stream of its own,
                                side by side; forked from and joined into the caller's stream */
} lucent_batch_options;
typedef struct lucent_batch_stats {
  uint64_t closest_rays, shadow_rays; /* traced by this batch since creation */
  uint32_t waves, graph_waves;        /* waves launched, of which replayed graphs */
  uint32_t wave_paths;                /* path capacity of a wave */
  uint64_t kernel_launches;           /* kernels its traces launched (replayed graphs count theirs) */
} lucent_batch_stats;
/* The renderers must stay alive (and keep their scenes loaded) while the
 * batch is used; they may be traced on their own in between. */
lucent_status lucent_batch_create(lucent_renderer* const* renderers, uint32_t n, lucent_batch** out);
void lucent_batch_destroy(lucent_batch* batch);
/* Defaults: samples_per_wave 0, max_wave_paths 2^25, use_graph 1, trace_blocks 0, shade_blocks 0,
 * sort_rays 1, top_levels 1, wide_bvh 1, scenes_per_wave 0, streams 1. */
lucent_status lucent_batch_set_options(lucent_batch* batch, const lucent_batch_options* options);
/* Asynchronous on `stream`. */
lucent_status lucent_batch_trace(lucent_batch* batch, uint32_t samples, void* stream);
/* Synchronises `stream`, reports the device error word and (if `stats` is
 * non-NULL) the batch's counters. */
lucent_status lucent_batch_check(lucent_batch* batch, void* stream, lucent_batch_stats* stats);

/* Diagnostic with no reference counterpart: evaluates the path tracer's
 * BSDF code (the device restatement of bsdf.glsl evalOpaque :114-166,
 * sampleOpaque :174-211, sampleDielectric :216-248) on `n` caller tuples of
 * 32 floats, writing 24 floats each; the layout is documented in
 * lucent_gb300/csrc/bsdf_tuples.cu. Host buffers; synchronous. */
lucent_status lucent_bsdf_eval_tuples(const float* tuples, uint32_t n, float* out);
/* Same tuples through the adjoint's BSDF derivative: 24 floats each, f (3)
 * then df/d(base colour r, g, b, roughness, metallic, clearcoat) (6 x 3). */
lucent_status lucent_bsdf_grad_tuples(const float* tuples, uint32_t n, float* out);

/* ---------------------------------------------------------------------------
 * Model ingestion helper. The reference leaves image decoding to the browser
 * (createImageBitmap, src/loaders/model.ts:43-72); this build decodes PNG
 * itself: the caller parses the chunks and inflates the data, this reverses
 * the per-scanline filters (PNG specification 9.2). `in` holds `rows` rows of
 * a filter-type byte plus `row_bytes` bytes; `bpp` is the bytes per complete
 * pixel (at least 1). Writes rows * row_bytes bytes; synchronous, host only. */
lucent_status lucent_png_unfilter(const uint8_t* in, uint32_t rows, uint32_t row_bytes, uint32_t bpp, uint8_t* out);

#ifdef __cplusplus
}
#endif
#endif /* LUCENT_H */
