// Device shading for the wavefront path tracer: the reference's surface,
// light and BSDF model (src/shaders/common.glsl, lights.glsl, bsdf.glsl,
// trace.frag) on packed device buffers. Binary32 throughout, like the GLSL.
#pragma once
#include <cuda_fp16.h>

#include "common.cuh"

namespace lucent {
namespace sh {

// The BSDF evaluation is called from four places of the shade kernel (three
// light samples and the BSDF sample); how it is compiled is set here.
#ifndef LUCENT_EVAL_FN
#define LUCENT_EVAL_FN LUCENT_DEV
#endif
#ifndef LUCENT_BSDF_FN
#define LUCENT_BSDF_FN LUCENT_DEV
#endif
#ifndef LUCENT_SAMPLE_FN
#define LUCENT_SAMPLE_FN LUCENT_DEV
#endif

constexpr float PI = 3.14159265358979323846f;
constexpr float INV_PI = 0.31830988618379067154f;
constexpr float TWO_PI = 6.28318530717958647692f;
constexpr float INF = 1e30f;
constexpr float EPS = 1e-6f;

// ------------------------------------------------------------ float3 helpers
LUCENT_DEV float3 f3(float a, float b, float c) { return make_float3(a, b, c); }
LUCENT_DEV float3 f3(float4 v) { return make_float3(v.x, v.y, v.z); }
LUCENT_DEV float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
LUCENT_DEV float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
LUCENT_DEV float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
LUCENT_DEV float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
LUCENT_DEV float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
LUCENT_DEV float3 operator*(float s, float3 a) { return f3(s * a.x, s * a.y, s * a.z); }
LUCENT_DEV float3 operator/(float3 a, float s) { return f3(a.x / s, a.y / s, a.z / s); }
LUCENT_DEV float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
LUCENT_DEV float3 cross3(float3 a, float3 b) {
  return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
LUCENT_DEV float len3(float3 a) { return sqrtf(dot3(a, a)); }
LUCENT_DEV float3 norm3(float3 a) { return a / len3(a); }
LUCENT_DEV float clampf(float x, float a, float b) { return fminf(fmaxf(x, a), b); }
LUCENT_DEV float mixf(float x, float y, float a) { return x * (1.f - a) + y * a; }
LUCENT_DEV float3 mix3(float3 x, float3 y, float a) { return x * (1.f - a) + y * a; }
LUCENT_DEV float max3(float3 v) { return fmaxf(v.x, fmaxf(v.y, v.z)); }
LUCENT_DEV float lum(float3 c) { return dot3(c, f3(0.2126f, 0.7152f, 0.0722f)); }
LUCENT_DEV float3 reflect3(float3 I, float3 N) { return I - 2.f * dot3(N, I) * N; }
LUCENT_DEV float3 refract3(float3 I, float3 N, float eta) {
  const float c = dot3(N, I);
  const float k = 1.f - eta * eta * (1.f - c * c);
  if (k < 0.f) return f3(0.f, 0.f, 0.f);
  return eta * I - (eta * c + sqrtf(k)) * N;
}
LUCENT_DEV float smooth(float e0, float e1, float x) {
  const float t = clampf((x - e0) / (e1 - e0), 0.f, 1.f);
  return t * t * (3.f - 2.f * t);
}

// ------------------------------------------------------------ RNG (common.glsl:13-25)
LUCENT_DEV uint32_t pcg(uint32_t& state) {
  const uint32_t s = state;
  state = s * 747796405u + 2891336453u;
  const uint32_t word = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
  return (word >> 22u) ^ word;
}
LUCENT_DEV float rnd(uint32_t& st) { return (float)pcg(st) * (1.0f / 4294967296.0f); }
// Alpha any-hit uniform from (path RNG state, slot): the path's own stream is
// never drawn inside a traversal.
LUCENT_DEV float alpha_rand(uint32_t key, uint32_t slot) {
  uint32_t s = key ^ (slot * 0x9E3779B9u);
  return (float)pcg(s) * (1.0f / 4294967296.0f);
}

// ------------------------------------------------------------ sampling helpers (common.glsl)
LUCENT_DEV void basis(float3 n, float3& t, float3& b) {
  const float s = n.z >= 0.f ? 1.f : -1.f;
  const float a = -1.f / (s + n.z);
  const float c = n.x * n.y * a;
  t = f3(1.f + s * n.x * n.x * a, s * c, -s * n.x);
  b = f3(c, s + n.y * n.y * a, -n.y);
}
LUCENT_DEV float3 to_world(float3 v, float3 t, float3 b, float3 n) { return t * v.x + b * v.y + n * v.z; }
LUCENT_DEV float3 to_local(float3 v, float3 t, float3 b, float3 n) { return f3(dot3(v, t), dot3(v, b), dot3(v, n)); }
LUCENT_DEV float3 cosine_hemisphere(float u0, float u1) {
  const float r = sqrtf(u0), phi = TWO_PI * u1;
  float sp, cp;
  sincosf(phi, &sp, &cp);
  return f3(r * cp, r * sp, sqrtf(fmaxf(0.f, 1.f - u0)));
}
LUCENT_DEV float3 uniform_cone(float u0, float u1, float cos_max) {
  const float ct = 1.f - u0 * (1.f - cos_max);
  const float st = sqrtf(fmaxf(0.f, 1.f - ct * ct));
  float sp, cp;
  sincosf(TWO_PI * u1, &sp, &cp);
  return f3(st * cp, st * sp, ct);
}
LUCENT_DEV float2 concentric_disk(float u0, float u1) {
  const float ox = 2.f * u0 - 1.f, oy = 2.f * u1 - 1.f;
  if (ox == 0.f && oy == 0.f) return make_float2(0.f, 0.f);
  float r, th;
  if (fabsf(ox) > fabsf(oy)) {
    r = ox;
    th = (PI / 4.f) * (oy / ox);
  } else {
    r = oy;
    th = (PI / 2.f) - (PI / 4.f) * (ox / oy);
  }
  float s, c;
  sincosf(th, &s, &c);
  return make_float2(r * c, r * s);
}
LUCENT_DEV float mis(float a, float b) {
  const float a2 = a * a, b2 = b * b;
  return a2 / fmaxf(a2 + b2, 1e-10f);
}
// Wachter-Binder offset (common.glsl:95-108): integer ULP nudge along n.
LUCENT_DEV float3 offset_ray(float3 p, float3 n) {
  const int ox = (int)(256.f * n.x), oy = (int)(256.f * n.y), oz = (int)(256.f * n.z);
  const float px = __int_as_float(__float_as_int(p.x) + (p.x < 0.f ? -ox : ox));
  const float py = __int_as_float(__float_as_int(p.y) + (p.y < 0.f ? -oy : oy));
  const float pz = __int_as_float(__float_as_int(p.z) + (p.z < 0.f ? -oz : oz));
  const float o = 1.f / 32.f, fs = 1.f / 65536.f;
  return f3(fabsf(p.x) < o ? p.x + fs * n.x : px, fabsf(p.y) < o ? p.y + fs * n.y : py,
            fabsf(p.z) < o ? p.z + fs * n.z : pz);
}

// ------------------------------------------------------------ device scene
struct SceneDev {
  const Node* nodes;
  uint32_t node_count;
  const float4* geo;        // 3 per slot: (v0, material), (v1, light), (v2, alpha flag)
  const float4* attr;       // 4 per slot: (n0, u0), (n1, u1), (n2, u2), (v0, v1, v2, 0)
  const float4* materials;  // 10 per material (material.ts:121-131)
  const float4* spheres;
  const int* sphere_materials;
  const int* sphere_lights;
  int sphere_count;
  const float4* lights;     // 4 per light (scene.ts:88-95)
  int light_count;
  int ground_material;      // -1: no ground plane
  float ground_height;
  int any_alpha;
  // Texture arrays (scene.glsl:17-18): tex_size^2 RGBA8 texels per layer,
  // row 0 at v = 0; colour layers hold sRGB codes. texel_lut: 512 floats,
  // sRGB code -> linear, then code / 255. tex_size 0: no textures.
  const uchar4* color_maps;
  const uchar4* data_maps;
  const float* texel_lut;
  int tex_size;
  const Node* wide;  // four-wide view of `nodes` (traverse_wide.cuh) or nullptr
};

// transformUV (scene.glsl:95-97): rows of a 2x3 affine map.
LUCENT_DEV float2 transform_uv(float2 uv, float4 row0, float4 row1) {
  return make_float2(row0.x * uv.x + row0.y * uv.y + row0.z, row1.x * uv.x + row1.y * uv.y + row1.z);
}

// textureLod(array, vec3(uv, layer), 0.0) with LINEAR filtering and REPEAT
// wrapping (context.ts:241-244); sRGB layers decode before filtering, alpha
// is linear.
LUCENT_DEV float4 sample_layer(const SceneDev& S, const uchar4* tex, int layer, float2 uv, bool srgb) {
  const int n = S.tex_size;
  float u = uv.x - floorf(uv.x), v = uv.y - floorf(uv.y);  // REPEAT
  if (!(u >= 0.f && u < 1.f)) u = 0.f;                     // NaN or infinite coordinates
  if (!(v >= 0.f && v < 1.f)) v = 0.f;
  const float x = u * (float)n - 0.5f, y = v * (float)n - 0.5f;
  const float x0 = floorf(x), y0 = floorf(y);
  const float fx = x - x0, fy = y - y0;
  const int ix = (int)x0, iy = (int)y0;
  const int xa = ix < 0 ? n - 1 : ix, xb = ix + 1 >= n ? 0 : ix + 1;
  const int ya = iy < 0 ? n - 1 : iy, yb = iy + 1 >= n ? 0 : iy + 1;
  const uchar4* L = tex + (size_t)layer * n * n;
  const uchar4 t00 = __ldg(L + (size_t)ya * n + xa), t10 = __ldg(L + (size_t)ya * n + xb);
  const uchar4 t01 = __ldg(L + (size_t)yb * n + xa), t11 = __ldg(L + (size_t)yb * n + xb);
  const float* rgb = S.texel_lut + (srgb ? 0 : 256);
  const float* lin = S.texel_lut + 256;
  auto mix4 = [&](float a, float b, float c, float d) {
    return (a * (1.f - fx) + b * fx) * (1.f - fy) + (c * (1.f - fx) + d * fx) * fy;
  };
  return make_float4(mix4(__ldg(rgb + t00.x), __ldg(rgb + t10.x), __ldg(rgb + t01.x), __ldg(rgb + t11.x)),
                     mix4(__ldg(rgb + t00.y), __ldg(rgb + t10.y), __ldg(rgb + t01.y), __ldg(rgb + t11.y)),
                     mix4(__ldg(rgb + t00.z), __ldg(rgb + t10.z), __ldg(rgb + t01.z), __ldg(rgb + t11.z)),
                     mix4(__ldg(lin + t00.w), __ldg(lin + t10.w), __ldg(lin + t01.w), __ldg(lin + t11.w)));
}

// triangleUV (scene.glsl:163-173): the slot's texture coordinates at barycentrics (bu, bv).
LUCENT_DEV float2 triangle_uv(const SceneDev& S, int slot, float bu, float bv) {
  const float4* a = S.attr + 4 * (size_t)slot;
  const float u0 = __ldg(&a[0].w), u1 = __ldg(&a[1].w), u2 = __ldg(&a[2].w);
  const float4 a3 = __ldg(&a[3]);
  const float w = 1.f - bu - bv;
  return make_float2(u0 * w + u1 * bu + u2 * bv, a3.x * w + a3.y * bu + a3.z * bv);
}

// alphaOpaque (scene.glsl:176-189): does a hit at barycentrics (bu, bv) on an
// alpha-tested slot block the ray? Constant alpha times the base colour map's
// alpha at the hit; mask mode compares with the cutoff, blend mode draws a
// uniform from (key, slot).
LUCENT_DEV bool alpha_opaque(const SceneDev& S, int slot, uint32_t key, float bu, float bv) {
  if (__ldg(&S.geo[3 * (size_t)slot + 2].w) < 0.5f) return true;
  const int m = (int)__ldg(&S.geo[3 * (size_t)slot].w);
  const float4* M = S.materials + (size_t)m * 10;
  float alpha = __ldg(&M[2].w);
  const int map = (int)__ldg(&M[4].x);
  if (map >= 0 && S.tex_size > 0) {
    const float2 tuv = transform_uv(triangle_uv(S, slot, bu, bv), __ldg(&M[8]), __ldg(&M[9]));
    alpha *= sample_layer(S, S.color_maps, map, tuv, true).w;
  }
  if ((int)__ldg(&M[3].w) == 1) return alpha >= __ldg(&M[5].w);
  return alpha_rand(key, (uint32_t)slot) < alpha;
}

// The alpha test without texture lookups, for the binary32 traversal
// kernels: kAlphaBlock or kAlphaPass as alpha_opaque decides, or kAlphaDefer
// when the answer needs the base colour map (the ray is then traced by the
// binary64 kernel, which samples it).
LUCENT_DEV AlphaAnswer alpha_fast(const SceneDev& S, int slot, uint32_t key) {
  if (__ldg(&S.geo[3 * (size_t)slot + 2].w) < 0.5f) return kAlphaBlock;
  const int m = (int)__ldg(&S.geo[3 * (size_t)slot].w);
  const float4* M = S.materials + (size_t)m * 10;
  if ((int)__ldg(&M[4].x) >= 0 && S.tex_size > 0) return kAlphaDefer;
  const float alpha = __ldg(&M[2].w);
  if ((int)__ldg(&M[3].w) == 1) return alpha >= __ldg(&M[5].w) ? kAlphaBlock : kAlphaPass;
  return alpha_rand(key, (uint32_t)slot) < alpha ? kAlphaBlock : kAlphaPass;
}

struct LightingDev {
  int sun_enabled;
  float3 sun_dir, sun_radiance;
  float sun_cos, sun_pdf;
  const float* env_rgb;  // equirect RGB f32, rows top to bottom
  int env_w, env_h;
  const float4* env_alias;  // per cell: keep probability, alias, pdfUV, alias pdfUV
  int grid_w, grid_h;
  float env_cos, env_sin, env_intensity;
  int env_sampling, env_background;
  float3 backdrop;
  const float* sheen_lut;  // 16 x 16, values already rounded to half precision
};

struct CameraDev {
  float3 pos, right, up, forward;
  float tan_half_fov, aperture, focus;
};

// Software GL LINEAR sample (the reference samples these with hardware
// bilinear filtering): u wraps (REPEAT) or clamps, v clamps.
LUCENT_DEV void bilinear(const float* img, int w, int h, int ch, float u, float v, bool repeat_s, float* out) {
  const float x = u * (float)w - 0.5f, y = v * (float)h - 0.5f;
  const float fx = floorf(x), fy = floorf(y);
  const float ax = x - fx, ay = y - fy;
  int x0 = (int)fx, y0 = (int)fy, x1 = x0 + 1, y1 = y0 + 1;
  if (repeat_s) {
    x0 %= w;
    x0 = x0 < 0 ? x0 + w : x0;
    x1 %= w;
    x1 = x1 < 0 ? x1 + w : x1;
  } else {
    x0 = min(max(x0, 0), w - 1);
    x1 = min(max(x1, 0), w - 1);
  }
  y0 = min(max(y0, 0), h - 1);
  y1 = min(max(y1, 0), h - 1);
  for (int c = 0; c < ch; c++) {
    const float a = __ldg(img + ((size_t)y0 * w + x0) * ch + c), b = __ldg(img + ((size_t)y0 * w + x1) * ch + c);
    const float cc = __ldg(img + ((size_t)y1 * w + x0) * ch + c), d = __ldg(img + ((size_t)y1 * w + x1) * ch + c);
    const float top = a * (1.f - ax) + b * ax, bot = cc * (1.f - ax) + d * ax;
    out[c] = top * (1.f - ay) + bot * ay;
  }
}

// The four texels and weights bilinear() blends (same clamping and wrap).
LUCENT_DEV void bilinear_taps(int w, int h, float u, float v, bool repeat_s, int idx[4], float wt[4]) {
  const float x = u * (float)w - 0.5f, y = v * (float)h - 0.5f;
  const float fx = floorf(x), fy = floorf(y);
  const float ax = x - fx, ay = y - fy;
  int x0 = (int)fx, y0 = (int)fy, x1 = x0 + 1, y1 = y0 + 1;
  if (repeat_s) {
    x0 %= w;
    x0 = x0 < 0 ? x0 + w : x0;
    x1 %= w;
    x1 = x1 < 0 ? x1 + w : x1;
  } else {
    x0 = min(max(x0, 0), w - 1);
    x1 = min(max(x1, 0), w - 1);
  }
  y0 = min(max(y0, 0), h - 1);
  y1 = min(max(y1, 0), h - 1);
  idx[0] = y0 * w + x0, idx[1] = y0 * w + x1, idx[2] = y1 * w + x0, idx[3] = y1 * w + x1;
  wt[0] = (1.f - ax) * (1.f - ay), wt[1] = ax * (1.f - ay), wt[2] = (1.f - ax) * ay, wt[3] = ax * ay;
}

// ------------------------------------------------------------ lights.glsl
LUCENT_DEV float3 env_to_local(const LightingDev& L, float3 d) {
  return f3(L.env_cos * d.x - L.env_sin * d.z, d.y, L.env_sin * d.x + L.env_cos * d.z);
}
LUCENT_DEV float3 env_to_world(const LightingDev& L, float3 l) {
  return f3(L.env_cos * l.x + L.env_sin * l.z, l.y, -L.env_sin * l.x + L.env_cos * l.z);
}
LUCENT_DEV float2 equirect_uv(float3 l) {
  return make_float2(atan2f(l.z, l.x) * (0.5f * INV_PI) + 0.5f, acosf(clampf(l.y, -1.f, 1.f)) * INV_PI);
}
LUCENT_DEV float3 env_tex(const LightingDev& L, float2 uv) {
  float o[3];
  bilinear(L.env_rgb, L.env_w, L.env_h, 3, uv.x, uv.y, true, o);
  return f3(o[0], o[1], o[2]);
}
LUCENT_DEV float3 env_radiance(const LightingDev& L, float3 d) {
  return env_tex(L, equirect_uv(env_to_local(L, d))) * L.env_intensity;
}
LUCENT_DEV float env_pdf(const LightingDev& L, float3 d) {
  const float3 l = env_to_local(L, d);
  const float st = sqrtf(fmaxf(0.f, 1.f - l.y * l.y));
  if (st < 1e-6f) return 0.f;
  const float2 uv = equirect_uv(l);
  const int cx = min((int)(uv.x * (float)L.grid_w), L.grid_w - 1);
  const int cy = min((int)(uv.y * (float)L.grid_h), L.grid_h - 1);
  return __ldg(&L.env_alias[(size_t)cy * L.grid_w + cx].z) / (2.f * PI * PI * st);
}

struct LightSample {
  float3 dir;
  float dist, pdf;
  float3 radiance;
  float2 uv;  // environment samples: the texture coordinate of the radiance lookup
};

LUCENT_DEV LightSample sample_environment(const LightingDev& L, uint32_t& rng) {
  LightSample ls;
  const int n = L.grid_w * L.grid_h;
  const int i = min((int)(rnd(rng) * (float)n), n - 1);
  const float4 e = __ldg(&L.env_alias[i]);
  int cell = i;
  float pdfUV = e.z;
  if (rnd(rng) >= e.x) {
    cell = (int)e.y;
    pdfUV = e.w;
  }
  const float j0 = rnd(rng), j1 = rnd(rng);
  const float u = ((float)(cell % L.grid_w) + j0) / (float)L.grid_w;
  const float v = ((float)(cell / L.grid_w) + j1) / (float)L.grid_h;
  const float phi = (u - 0.5f) * TWO_PI, theta = v * PI;
  float st, ct, sp, cp;
  sincosf(theta, &st, &ct);
  sincosf(phi, &sp, &cp);
  ls.dir = env_to_world(L, f3(st * cp, ct, st * sp));
  ls.dist = INF;
  ls.pdf = st > 1e-6f ? pdfUV / (2.f * PI * PI * st) : 0.f;
  ls.radiance = env_tex(L, make_float2(u, v)) * L.env_intensity;
  ls.uv = make_float2(u, v);
  return ls;
}

LUCENT_DEV float3 environment(const LightingDev& L, float3 d, bool specular, float bsdf_pdf) {
  float3 r = env_radiance(L, d);
  if (!specular && L.env_sampling) r = r * mis(bsdf_pdf, env_pdf(L, d));
  if (L.sun_enabled && dot3(d, L.sun_dir) >= L.sun_cos) {
    const float w = specular ? 1.f : mis(bsdf_pdf, L.sun_pdf);
    r = r + L.sun_radiance * w;
  }
  return r;
}

LUCENT_DEV float hit_sphere(float3 ro, float3 rd, float4 s, float tmax) {  // scene.glsl:132-144
  const float3 oc = ro - f3(s);
  const float b = dot3(oc, rd);
  const float c = dot3(oc, oc) - s.w * s.w;
  const float disc = b * b - c;
  if (disc < 0.f) return INF;
  const float sq = sqrtf(disc);
  float t = -b - sq;
  if (t > EPS && t < tmax) return t;
  t = -b + sq;
  if (t > EPS && t < tmax) return t;
  return INF;
}

LUCENT_DEV float hit_ground(const SceneDev& S, float3 ro, float3 rd, float tmax) {  // scene.glsl:146-150
  if (S.ground_material < 0 || fabsf(rd.y) < 1e-9f) return INF;
  const float t = (S.ground_height - ro.y) / rd.y;
  return t > EPS && t < tmax ? t : INF;
}

LUCENT_DEV LightSample sample_light(const SceneDev& S, int index, float3 p, float u0, float u1) {  // :99-138
  LightSample ls;
  ls.pdf = 0.f;
  ls.dir = f3(0.f, 0.f, 0.f);
  ls.dist = 0.f;
  const float4 l0 = __ldg(S.lights + index * 4), l1 = __ldg(S.lights + index * 4 + 1),
               l2 = __ldg(S.lights + index * 4 + 2), l3 = __ldg(S.lights + index * 4 + 3);
  ls.radiance = f3(l3);
  if (l0.w < 0.5f) {
    const float3 toC = f3(l0) - p;
    const float d2 = dot3(toC, toC);
    const float r = l1.w;
    if (d2 <= r * r) return ls;
    const float cos_max = sqrtf(fmaxf(0.f, 1.f - r * r / d2));
    const float3 axis = toC * rsqrtf(d2);
    float3 t, b;
    basis(axis, t, b);
    ls.dir = to_world(uniform_cone(u0, u1, cos_max), t, b, axis);
    ls.pdf = 1.f / (TWO_PI * (1.f - cos_max));
    const float t0 = hit_sphere(p, ls.dir, make_float4(l0.x, l0.y, l0.z, r), INF);
    ls.dist = t0 < INF ? t0 : sqrtf(d2);
  } else {
    const float3 e1 = f3(l1), e2 = f3(l2);
    const float3 q = f3(l0) + e1 * u0 + e2 * u1;
    const float3 toQ = q - p;
    const float d2 = dot3(toQ, toQ);
    const float d = sqrtf(d2);
    ls.dir = toQ / d;
    ls.dist = d;
    const float3 nc = cross3(e1, e2);
    const float area = len3(nc);
    const float cosL = fabsf(dot3(nc / area, ls.dir));
    if (cosL < 1e-4f) return ls;
    ls.pdf = d2 / (cosL * area);
  }
  return ls;
}

LUCENT_DEV float light_pdf(const SceneDev& S, int index, float3 p, float3 dir, float dist) {  // :141-158
  const float4 l0 = __ldg(S.lights + index * 4), l1 = __ldg(S.lights + index * 4 + 1),
               l2 = __ldg(S.lights + index * 4 + 2);
  if (l0.w < 0.5f) {
    const float3 toC = f3(l0) - p;
    const float d2 = dot3(toC, toC);
    const float r = l1.w;
    if (d2 <= r * r) return 0.f;
    const float cos_max = sqrtf(fmaxf(0.f, 1.f - r * r / d2));
    return 1.f / (TWO_PI * (1.f - cos_max));
  }
  const float3 nc = cross3(f3(l1), f3(l2));
  const float area = len3(nc);
  const float cosL = fabsf(dot3(nc / area, dir));
  if (cosL < 1e-4f) return 0.f;
  return dist * dist / (cosL * area);
}

// ------------------------------------------------------------ bsdf.glsl
struct Surface {
  float3 albedo;
  float metallic, roughness, ior, transmission;
  float clearcoat, clearcoat_roughness;
  float3 sheen_color;
  float sheen_roughness;
  bool thin;
  float3 absorption, n, nc;
};

LUCENT_DEV float d_ggx(float NdotH, float a) {
  const float a2 = a * a;
  const float d = NdotH * NdotH * (a2 - 1.f) + 1.f;
  return a2 / (PI * d * d);
}

// Error-free transformations (Knuth TwoSum; the FMA product residual;
// Kahan's difference of products), used where a binary32 formula cancels.
LUCENT_DEV void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
LUCENT_DEV float diff_of_products(float a, float b, float c, float d) {  // a*b - c*d to ~1.5 ulp
  const float w = c * d;
  const float e = fmaf(-c, d, w);
  return fmaf(a, b, -w) + e;
}

// The unnormalised half vector h = wo + wi as an exact pair (hs + he) and
// the pieces of the GGX denominator that cancel near the lobe's peak.
struct HalfVec {
  float3 hs, he;
  float hh;  // |h|^2
};
LUCENT_DEV HalfVec half_vec(float3 wo, float3 wi) {
  HalfVec h;
  two_sum(wo.x, wi.x, h.hs.x, h.he.x);
  two_sum(wo.y, wi.y, h.hs.y, h.he.y);
  two_sum(wo.z, wi.z, h.hs.z, h.he.z);
  h.hh = dot3(h.hs, h.hs) + 2.f * dot3(h.hs, h.he);
  return h;
}
// 1 - |n|^2 (a binary32 unit vector is unit only to ~1e-7).
LUCENT_DEV float one_minus_norm2(float3 n) {
  const float px = n.x * n.x, py = n.y * n.y, pz = n.z * n.z;
  const float ex = fmaf(n.x, n.x, -px), ey = fmaf(n.y, n.y, -py), ez = fmaf(n.z, n.z, -pz);
  float s, t1, t2;
  two_sum(px, py, s, t1);
  two_sum(s, pz, s, t2);
  return (1.f - s) - (ex + ey + ez + t1 + t2);
}
// D_GGX (bsdf.glsl:28-32) for n and H = h / |h|. Near the peak the
// shader's denominator NdotH^2 (a^2 - 1) + 1 cancels (a binary32 evaluation
// keeps ~1e-7 of absolute accuracy); below 1/4 it is evaluated as the equal
// sin^2 + (1 - |n|^2) + NdotH^2 a^2, sin^2 = |n x h|^2 / |h|^2 from exact
// cross products, which keeps full relative accuracy at any sharpness.
LUCENT_DEV float d_ggx_h(float3 n, float3 wo, float3 wi, float NdotH, float a) {
  const float a2 = a * a;
  const float d = NdotH * NdotH * (a2 - 1.f) + 1.f;
  if (!(NdotH > 0.f && d < 0.25f)) return a2 / (PI * d * d);
  const HalfVec h = half_vec(wo, wi);
  const float3 c = f3(diff_of_products(n.y, h.hs.z, n.z, h.hs.y) + (n.y * h.he.z - n.z * h.he.y),
                      diff_of_products(n.z, h.hs.x, n.x, h.hs.z) + (n.z * h.he.x - n.x * h.he.z),
                      diff_of_products(n.x, h.hs.y, n.y, h.hs.x) + (n.x * h.he.y - n.y * h.he.x));
  const float num = dot3(c, c) + h.hh * (one_minus_norm2(n) + NdotH * NdotH * a2);  // d |h|^2
  const float hn = h.hh / num;
  return a2 * hn * hn / PI;
}
LUCENT_DEV float g1_ggx(float NdotX, float a) {
  const float a2 = a * a;
  return 2.f * NdotX / (NdotX + sqrtf(a2 + (1.f - a2) * NdotX * NdotX));
}
LUCENT_DEV float schlick_w(float c) {
  const float m = 1.f - clampf(c, 0.f, 1.f);
  const float m2 = m * m;
  return m2 * m2 * m;  // pow(m, 5) for m in [0, 1]
}
LUCENT_DEV float3 fresnel3(float c, float3 F0) { return F0 + (f3(1.f, 1.f, 1.f) - F0) * schlick_w(c); }
LUCENT_DEV float fresnel1(float c, float F0) { return F0 + (1.f - F0) * schlick_w(c); }
LUCENT_DEV float dielectric_f0(float ior) {
  const float r = (ior - 1.f) / (ior + 1.f);
  return r * r;
}
LUCENT_DEV float alpha_of(float r) { return fmaxf(r * r, 1e-3f); }

// sampleGGXVNDF (Heitz 2018; bsdf.glsl:59-72). Three differences of the
// shader's form cancel in binary32 for sharp lobes (Vh.z -> 1) and samples
// at the rim of the projected disk (u0 -> 1): 1 - s, sqrt(1 - t1^2) and
// sqrt(1 - t1^2 - t2'^2). They are evaluated in rearranged forms with the
// same value:
//   1 - s = (1 - Vh.z) / 2,  1 - Vh.z = (v.x^2 + v.y^2) / (|v| (|v| + v.z))
//   q^2 = 1 - t1^2 = (1 - u0) + u0 sin^2(phi)            (1 - u0 exact, u0 >= 0.5)
//   1 - t1^2 - t2'^2 = s (q - t2)(q + t2'),  q^2 - t2^2 = 1 - u0, so
//   q - t2 = (1 - u0) / (q + t2) (t2 > 0),  q + t2' = (1-s)(q - t2) + (1 - u0) / (q - t2) (t2 <= 0).
LUCENT_BSDF_FN float3 sample_vndf(float3 Ve, float a, float u0, float u1) {
  const float3 v = f3(a * Ve.x, a * Ve.y, Ve.z);
  const float vl = len3(v);
  const float3 Vh = v / vl;
  const float lensq = Vh.x * Vh.x + Vh.y * Vh.y;
  const float3 T1 = lensq > 0.f ? f3(-Vh.y, Vh.x, 0.f) / sqrtf(lensq) : f3(1.f, 0.f, 0.f);
  const float3 T2 = cross3(Vh, T1);
  const float r = sqrtf(u0);
  float sp, cp;
  sincosf(TWO_PI * u1, &sp, &cp);
  const float t1 = r * cp;
  const float t2 = r * sp;
  const float s = 0.5f * (1.f + Vh.z);
  const float s1 = v.z > 0.f ? 0.5f * (v.x * v.x + v.y * v.y) / (vl * (vl + v.z)) : 1.f - s;
  const float om = 1.f - u0;
  const float q = sqrtf(fmaxf(0.f, om + u0 * sp * sp));
  const float t2b = s1 * q + s * t2;
  float qm, qp;  // q - t2 and q + t2'
  if (t2 > 0.f) {
    qm = om / (q + t2);
    qp = (1.f + s1) * q + s * t2;
  } else {
    qm = q - t2;
    qp = qm > 0.f ? s1 * qm + om / qm : 0.f;
  }
  const float z2 = s * qm * qp;
  const float3 Nh = t1 * T1 + t2b * T2 + sqrtf(fmaxf(0.f, z2)) * Vh;
  return norm3(f3(a * Nh.x, a * Nh.y, fmaxf(0.f, Nh.z)));
}

// Charlie sheen D (bsdf.glsl:79-83): (2 + 1/a) sin^(1/a) / 2pi with
// sin^2 = 1 - cos^2 evaluated as sin2 = (1 - c)(1 + c) to keep precision for
// exponents up to ~204.
LUCENT_DEV float d_charlie(float alpha, float NdotH) {
  const float inv = 1.f / alpha;
  const float sin2 = fmaxf((1.f - NdotH) * (1.f + NdotH), 0.f);
  return (2.f + inv) * powf(sin2, inv * 0.5f) / TWO_PI;
}
LUCENT_DEV float v_neubelt(float NdotL, float NdotV) { return 1.f / (4.f * (NdotL + NdotV - NdotL * NdotV)); }

LUCENT_DEV float sheen_albedo(const LightingDev& L, float NdotV, float r) {  // LINEAR-filtered 16x16 LUT
  float o;
  bilinear(L.sheen_lut, 16, 16, 1, (NdotV * 15.f + 0.5f) / 16.f, (r * 15.f + 0.5f) / 16.f, false, &o);
  return o;
}
LUCENT_DEV float spec_prob(float3 F0, float metallic, float NdotV) {
  const float f = lum(fresnel3(NdotV, F0));
  return mixf(clampf(f, 0.1f, 0.9f), 1.f, metallic);
}
LUCENT_DEV float coat_prob(const Surface& s, float3 wo) {
  if (s.clearcoat <= 0.f) return 0.f;
  const float Fc = s.clearcoat * fresnel1(fmaxf(dot3(s.nc, wo), 0.f), 0.04f);
  const float base = (1.f - Fc) * fmaxf(lum(s.albedo), 0.04f);
  return clampf(Fc / (Fc + base), 0.15f, 0.85f);
}
LUCENT_DEV float3 base_f0(const Surface& s) {
  const float d = dielectric_f0(s.ior);
  return mix3(f3(d, d, d), s.albedo, s.metallic);
}

// evalOpaque (bsdf.glsl:114-166): f (not cosine-weighted) and the mixture pdf.
LUCENT_EVAL_FN float3 eval_opaque(const LightingDev& L, const Surface& s, float3 wo, float3 wi, float& pdf) {
  const float3 n = s.n;
  const float NdotL = dot3(n, wi), NdotV = dot3(n, wo);
  pdf = 0.f;
  if (NdotL <= 0.f || NdotV <= 0.f) return f3(0.f, 0.f, 0.f);
  const float a = alpha_of(s.roughness);
  const float3 H = norm3(wo + wi);
  const float NdotH = fmaxf(dot3(n, H), 0.f), VdotH = fmaxf(dot3(wo, H), 0.f);
  const float3 F0 = base_f0(s);
  const float3 F = fresnel3(VdotH, F0);
  const float D = d_ggx_h(n, wo, wi, NdotH, a);
  const float G1v = g1_ggx(NdotV, a);
  const float G = G1v * g1_ggx(NdotL, a);
  const float3 spec = (D * G) * F / fmaxf(4.f * NdotV * NdotL, 1e-6f);
  const float3 diff = (f3(1.f, 1.f, 1.f) - F) * s.albedo * (1.f - s.metallic) * INV_PI;
  float3 f = diff + spec;
  const float pspec = spec_prob(F0, s.metallic, NdotV);
  pdf = mixf(NdotL * INV_PI, G1v * D / fmaxf(4.f * NdotV, 1e-6f), pspec);
  const float smax = max3(s.sheen_color);
  if (smax > 0.f) {
    const float sr = fmaxf(s.sheen_roughness, 0.07f);
    const float3 sheen = s.sheen_color * d_charlie(sr * sr, NdotH) * v_neubelt(NdotL, NdotV);
    const float scale = 1.f - smax * fmaxf(sheen_albedo(L, NdotV, sr), sheen_albedo(L, NdotL, sr));
    f = sheen + f * scale;
  }
  const float pcoat = coat_prob(s, wo);
  if (pcoat > 0.f) {
    const float cV = dot3(s.nc, wo), cL = dot3(s.nc, wi);
    float coat = 0.f, pdf_coat = 0.f;
    if (cV > 0.f && cL > 0.f) {
      const float ac = alpha_of(s.clearcoat_roughness);
      const float cH = fmaxf(dot3(s.nc, H), 0.f);
      const float Dc = d_ggx_h(s.nc, wo, wi, cH, ac), G1c = g1_ggx(cV, ac);
      coat = Dc * G1c * g1_ggx(cL, ac) * fresnel1(VdotH, 0.04f) / (4.f * cV * cL);
      pdf_coat = G1c * Dc / (4.f * cV);
    }
    const float Fcv = fresnel1(fmaxf(cV, 0.f), 0.04f);
    f = f * (1.f - s.clearcoat * Fcv) + f3(coat, coat, coat) * s.clearcoat;
    pdf = mixf(pdf, pdf_coat, pcoat);
  }
  return f;
}

// Derivatives of evalOpaque's f with respect to the material parameters an
// inverse renderer optimises: df[0..2] base colour r, g, b; df[3] roughness;
// df[4] metallic; df[5] clearcoat (each an RGB vector). The pdf, the lobe
// and coat probabilities and the sheen energy scale are sampling-side
// quantities and held fixed. The clearcoat derivative is the one-sided one
// at clearcoat = 0. Returns f as eval_opaque does.
LUCENT_DEV float3 eval_opaque_grad(const LightingDev& L, const Surface& s, float3 wo, float3 wi, float3 df[6]) {
  for (int k = 0; k < 6; k++) df[k] = f3(0.f, 0.f, 0.f);
  const float3 n = s.n;
  const float NdotL = dot3(n, wi), NdotV = dot3(n, wo);
  if (NdotL <= 0.f || NdotV <= 0.f) return f3(0.f, 0.f, 0.f);
  const float r = s.roughness, a = alpha_of(r), dadr = r * r > 1e-3f ? 2.f * r : 0.f;
  const float3 H = norm3(wo + wi);
  const float NdotH = fmaxf(dot3(n, H), 0.f), VdotH = fmaxf(dot3(wo, H), 0.f);
  const float d0 = dielectric_f0(s.ior), m = s.metallic, W = schlick_w(VdotH);
  const float3 F0 = base_f0(s);
  const float3 F = fresnel3(VdotH, F0);
  const float D = d_ggx_h(n, wo, wi, NdotH, a);
  const float dd = NdotH * NdotH * (a * a - 1.f) + 1.f;
  const float dDda = D * (2.f / a - 4.f * a * NdotH * NdotH / dd);
  auto g1 = [&](float N, float& dg) {
    const float q = sqrtf(a * a + (1.f - a * a) * N * N);
    const float g = 2.f * N / (N + q);
    dg = -2.f * N * (a * (1.f - N * N) / q) / ((N + q) * (N + q));
    return g;
  };
  float dG1v, dG1l;
  const float G1v = g1(NdotV, dG1v), G1l = g1(NdotL, dG1l);
  const float G = G1v * G1l, dGda = dG1v * G1l + G1v * dG1l;
  const float den = fmaxf(4.f * NdotV * NdotL, 1e-6f);
  const float3 spec = (D * G) * F / den;
  const float3 diff = (f3(1.f, 1.f, 1.f) - F) * s.albedo * (1.f - m) * INV_PI;
  float3 f1 = diff + spec;
  const float* Fp = &F.x;
  const float* alb = &s.albedo.x;
  float g_alb[3], g_r[3], g_m[3];
  for (int c = 0; c < 3; c++) {
    const float dFa = (1.f - W) * m, dFm = (1.f - W) * (alb[c] - d0);
    g_alb[c] = (-dFa * alb[c] + (1.f - Fp[c])) * (1.f - m) * INV_PI + D * G * dFa / den;
    g_r[c] = (dDda * G + D * dGda) * Fp[c] / den * dadr;
    g_m[c] = (-dFm * alb[c] * (1.f - m) - (1.f - Fp[c]) * alb[c]) * INV_PI + D * G * dFm / den;
  }
  float scale = 1.f;
  const float smax = max3(s.sheen_color);
  if (smax > 0.f) {
    const float sr = fmaxf(s.sheen_roughness, 0.07f);
    const float3 sheen = s.sheen_color * d_charlie(sr * sr, NdotH) * v_neubelt(NdotL, NdotV);
    scale = 1.f - smax * fmaxf(sheen_albedo(L, NdotV, sr), sheen_albedo(L, NdotL, sr));
    f1 = sheen + f1 * scale;
  }
  const float cV = dot3(s.nc, wo), cL = dot3(s.nc, wi);
  float coat = 0.f;
  if (cV > 0.f && cL > 0.f) {
    const float ac = alpha_of(s.clearcoat_roughness);
    const float cH = fmaxf(dot3(s.nc, H), 0.f);
    coat = d_ggx_h(s.nc, wo, wi, cH, ac) * g1_ggx(cV, ac) * g1_ggx(cL, ac) * fresnel1(VdotH, 0.04f) / (4.f * cV * cL);
  }
  const float Fcv = fresnel1(fmaxf(cV, 0.f), 0.04f);
  const float cc = s.clearcoat > 0.f ? s.clearcoat : 0.f;
  const float keep = 1.f - cc * Fcv;
  float3 f = cc > 0.f ? f1 * keep + f3(coat, coat, coat) * cc : f1;
  const float* f1p = &f1.x;
  float* dfp[6] = {&df[0].x, &df[1].x, &df[2].x, &df[3].x, &df[4].x, &df[5].x};
  for (int c = 0; c < 3; c++) {
    const float k = scale * (cc > 0.f ? keep : 1.f);
    dfp[c][c] = g_alb[c] * k;
    dfp[3][c] = g_r[c] * k;
    dfp[4][c] = g_m[c] * k;
    dfp[5][c] = coat - f1p[c] * Fcv;
  }
  return f;
}

struct BsdfSample {
  float3 dir, weight;
  float pdf;
};

// sampleOpaque (bsdf.glsl:174-211); `U` draws the uniforms in the GLSL order.
template <class UF>
LUCENT_SAMPLE_FN BsdfSample sample_opaque(const LightingDev& L, const Surface& s, float3 wo, UF&& U) {
  BsdfSample bs;
  bs.pdf = 0.f;
  bs.weight = f3(0.f, 0.f, 0.f);
  bs.dir = f3(0.f, 0.f, 0.f);
  float3 wi;
  const float uc = U();
  if (uc < coat_prob(s, wo)) {
    float3 t, b;
    basis(s.nc, t, b);
    const float3 woL = to_local(wo, t, b, s.nc);
    if (woL.z <= 0.f) return bs;
    const float a0 = U(), a1 = U();
    const float3 H = sample_vndf(woL, alpha_of(s.clearcoat_roughness), a0, a1);
    wi = to_world(reflect3(-woL, H), t, b, s.nc);
  } else {
    float3 t, b;
    basis(s.n, t, b);
    const float3 woL = to_local(wo, t, b, s.n);
    if (woL.z <= 0.f) return bs;
    float3 wiL;
    const float us = U();
    if (us < spec_prob(base_f0(s), s.metallic, woL.z)) {
      const float a0 = U(), a1 = U();
      wiL = reflect3(-woL, sample_vndf(woL, alpha_of(s.roughness), a0, a1));
    } else {
      const float a0 = U(), a1 = U();
      wiL = cosine_hemisphere(a0, a1);
    }
    wi = to_world(wiL, t, b, s.n);
  }
  const float NdotL = dot3(s.n, wi);
  if (NdotL <= 0.f) return bs;
  float pdf;
  const float3 f = eval_opaque(L, s, wo, wi, pdf);
  if (pdf <= 0.f) return bs;
  bs.dir = wi;
  bs.pdf = pdf;
  bs.weight = f * NdotL / pdf;
  return bs;
}

// sampleDielectric (bsdf.glsl:216-248).
template <class UF>
LUCENT_DEV bool sample_dielectric(const Surface& s, bool front, float3 ng, float3 wo, float3& wi, float3& weight,
                                  bool& reflected, UF&& U) {
  const float3 n = s.n;
  float3 t, b;
  basis(n, t, b);
  const float3 woL = to_local(wo, t, b, n);
  if (woL.z <= 0.f) return false;
  float3 H = n;
  if (s.roughness > 0.f) {
    const float a0 = U(), a1 = U();
    H = to_world(sample_vndf(woL, alpha_of(s.roughness), a0, a1), t, b, n);
  }
  float cosI = dot3(wo, H);
  if (cosI <= 0.f) {
    H = n;
    cosI = woL.z;
  }
  const float eta = front ? 1.f / s.ior : s.ior;
  const float sin2T = eta * eta * (1.f - cosI * cosI);
  float Fr = fresnel1(cosI, dielectric_f0(s.ior));
  if (s.thin)
    Fr = 2.f * Fr / (1.f + Fr);
  else if (sin2T > 1.f)
    Fr = 1.f;
  if (U() < Fr) {
    wi = reflect3(-wo, H);
    weight = f3(1.f, 1.f, 1.f);
    reflected = true;
    return dot3(wi, ng) > 0.f;
  }
  wi = s.thin ? -wo : refract3(-wo, H, eta);
  weight = s.albedo;
  reflected = false;
  return dot3(wi, ng) < 0.f;
}

}  // namespace sh
}  // namespace lucent
