/*
 * Oracle renderer: CPU restatement of the reference's path tracer
 * (src/shaders/trace.frag with common.glsl, scene.glsl, lights.glsl,
 * bsdf.glsl) and its denoise / display passes (variance.frag, atrous.frag,
 * denoise.glsl, display.frag). TEST INFRASTRUCTURE ONLY (the checker).
 *
 * Precision 32 evaluates the shading in binary32 like the GLSL; precision 64
 * evaluates it in binary64 (the FP64 reference render). Triangle hits use the
 * binary64 restatement of intersectBVH (src/math/bvh.ts:265-320) with
 * tMin = EPS (common.glsl:8) and tMax = INF (1e30), then analytic spheres and
 * the ground plane override them when closer, as traceScene does.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_scene {
  uint32_t tri_count;
  const float* positions;     /* 9 per triangle, original order (for intersectBVH) */
  const float* geo;           /* 12 per slot: packScene triGeometry (scene.ts:213-235) */
  const float* attr;          /* 16 per slot: packScene triAttributes */
  const float* nodes;         /* reference layout, 8 per node */
  uint32_t node_count;
  const uint32_t* tri_indices;
  const float* materials;     /* 40 per material (material.ts:121-131) */
  uint32_t material_count;
  const float* spheres;       /* 4 per sphere */
  const int32_t* sphere_materials;
  const int32_t* sphere_lights;
  uint32_t sphere_count;
  const float* lights;        /* 16 per light (scene.ts:88-95) */
  uint32_t light_count;
  int32_t ground_material;    /* -1: no ground */
  float ground_height;
  /* lighting uniforms (renderer.ts:355-413) */
  int32_t sun_enabled;
  float sun_dir[3], sun_radiance[3], sun_cos_angle, sun_pdf;
  uint32_t env_width, env_height;
  const float* env_rgb;       /* equirect RGB, rows top to bottom */
  uint32_t env_grid_w, env_grid_h;
  const float* env_alias;     /* 4 per cell */
  float env_rot_cos, env_rot_sin, env_intensity;
  int32_t env_sampling, env_background;
  float backdrop[3];
  const float* sheen_lut;     /* 16x16, already rounded to half precision */
  /* texture arrays (scene.glsl:17-18): tex_size^2 RGBA8 texels per layer, row 0 at v = 0;
   * colour layers hold sRGB codes. tex_size 0: no textures. */
  const uint8_t* color_maps;
  const uint8_t* data_maps;
  uint32_t tex_size;
} orc_scene;

typedef struct orc_camera {
  float pos[3], right[3], up[3], forward[3];
  float tan_half_fov, aperture, focus_dist;
} orc_camera;

/* Renders samples [seed0, seed0 + samples) into the crop [x0,x0+cw) x [y0,y0+ch)
 * of a width x height image (pixel y = 0 is the bottom row, like
 * gl_FragCoord), accumulating like trace.frag:324-354 with uReproject = 0.
 * Outputs per crop pixel: color4 (rgb mean, mean lum^2), albedo4, normal4,
 * history. albedo/normal are rounded to half precision at every store
 * (RGBA16F targets, renderer.ts:490) when precision == 32. */
int orc_render(const orc_scene* s, const orc_camera* cam, uint32_t max_bounces, float clamp_lum, uint32_t width,
               uint32_t height, uint32_t x0, uint32_t y0, uint32_t cw, uint32_t ch, uint32_t seed0,
               uint32_t samples, int precision, float* color4, float* albedo4, float* normal4, float* history,
               int threads);

/* orc_render (precision 32) that also counts the rays it traces and, when
 * `detailed`, the reference GLSL traversal work of each: work_out = [closest
 * rays, inner nodes visited, triangles tested, shadow rays, shadow nodes
 * visited, shadow triangles]. */
int orc_render_work(const orc_scene* s, const orc_camera* cam, uint32_t max_bounces, float clamp_lum,
                    uint32_t width, uint32_t height, uint32_t x0, uint32_t y0, uint32_t cw, uint32_t ch,
                    uint32_t seed0, uint32_t samples, float* color4, float* albedo4, float* normal4,
                    float* history, int threads, int detailed, uint64_t* work_out);

/* The triangle part of traceScene / occluded as orc_render decides it, ray by
 * ray (binary32 rays, binary64 decisions of intersectBVH over BVH slots with
 * the alpha test). orc_closest_slots: rays6 = 6 floats per ray, slot_out =
 * slot or -1 (miss) / -2 (stack overflow), t_out (may be NULL) = binary64 t.
 * orc_any_slots: rays7 = origin, direction, t_max; occluded_out = 1 / 0. keys:
 * per-ray alpha-blend hash keys (NULL: 0). */
int orc_closest_slots(const orc_scene* s, const float* rays6, const uint32_t* keys, uint64_t n, double t_min,
                      double t_max, int32_t* slot_out, double* t_out, int threads);
int orc_any_slots(const orc_scene* s, const float* rays7, const uint32_t* keys, uint64_t n, double t_min,
                  uint8_t* occluded_out, int threads);

/* One texture-array layer from a decoded RGBA8 image (rows top to bottom):
 * the resampling of buildTextureArrays (renderer.ts:314-333, resample.frag)
 * as the product defines it (box mip chain, level of detail log2(max(w, h) /
 * size) in binary64, bilinear with edge clamping, sRGB decoded before
 * filtering and re-encoded by code-value midpoints when srgb != 0). */
int orc_resample_layer(const uint8_t* rgba, uint32_t w, uint32_t h, uint32_t size, int srgb, uint8_t* out);
/* The shared layer size of buildTextureArrays for these image sizes. */
uint32_t orc_texture_size(const uint32_t* w, const uint32_t* h, uint32_t n);

/* BSDF tuples (bsdf.glsl): for each tuple evaluates evalOpaque, and
 * sampleOpaque / sampleDielectric driven by the given uniforms instead of the
 * RNG. Tuple layout and outputs documented in oracle_render.cpp. */
int orc_bsdf_tuples(const float* in, uint64_t n, int precision, double* out, int threads);
void orc_bsdf_set_lut(const float* lut);

/* Denoiser and display (variance.frag, atrous.frag, display.frag) on full
 * W x H images; see oracle_render.cpp for buffer layouts. */
int orc_denoise(const float* color4, const float* albedo4, const float* normal4, const float* history,
                uint32_t w, uint32_t h, const orc_camera* cam, uint32_t levels, float sigma_l, float sigma_n,
                float sigma_p, float* out4);
int orc_display(const float* color4, const float* albedo4, const float* denoised4, uint32_t w, uint32_t h,
                float denoise_weight, float exposure, int tonemap, float* out_rgb);
/* display.frag with the traced region rw x rh shown in a vw x vh view (Catmull-Rom when they differ). */
int orc_display_view(const float* color4, const float* albedo4, const float* denoised4, uint32_t rw, uint32_t rh,
                     uint32_t vw, uint32_t vh, float denoise_weight, float exposure, int tonemap, float* out_rgb);

/* The previous view of a temporal reprojection: its camera, size and
 * targets (w x h, albedo/normal as the RGBA16F values). */
typedef struct orc_history {
  const orc_camera* cam;
  uint32_t w, h;
  const float* color4;
  const float* albedo4;
  const float* normal4;
  const float* history;
} orc_history;

/* orc_render whose first sample per pixel starts from the history
 * reprojected from `hist` (trace.frag:310-322 with uReproject = 1). */
int orc_render_reproject(const orc_scene* s, const orc_camera* cam, const orc_history* hist, uint32_t max_bounces,
                         float clamp_lum, uint32_t width, uint32_t height, uint32_t x0, uint32_t y0, uint32_t cw,
                         uint32_t ch, uint32_t seed0, uint32_t samples, int precision, float* color4, float* albedo4,
                         float* normal4, float* history, int threads);

/* Finite-difference reference of the adjoint: sum over pixels of dl4[px].rgb
 * times the mean over samples [seed0, seed0 + samples) of the radiance traced
 * with sampling from s and BSDF values / environment radiance from
 * materials_eval / env_eval (NULL: s's own), in binary64. */
double orc_detached_dot(const orc_scene* s, const orc_camera* cam, uint32_t max_bounces, float clamp_lum,
                        uint32_t width, uint32_t height, uint32_t seed0, uint32_t samples, const float* materials_eval,
                        const float* env_eval, const float* dl4, int threads);

#ifdef __cplusplus
}
#endif
