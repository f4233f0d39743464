/*
 * Oracle renderer. TEST INFRASTRUCTURE ONLY: the checker for the CUDA path
 * tracer, denoiser and display kernels.
 *
 * A line-by-line restatement of the reference's GLSL (cited per function):
 *   src/shaders/common.glsl, scene.glsl, lights.glsl, bsdf.glsl, trace.frag,
 *   variance.frag, atrous.frag, denoise.glsl, display.frag.
 * Shading arithmetic is templated on the scalar R: float reproduces the GLSL's
 * binary32 evaluation, double gives the FP64 reference render. GLSL built-ins
 * use their specified formulas (mix = x(1-a)+ya, reflect, refract,
 * smoothstep, ...). Function arguments are evaluated left to right, as GLSL
 * ES 3.00 specifies, which fixes the order rand() values are drawn in.
 *
 * Deliberate, documented deviations shared with the CUDA product:
 *  - triangle hits come from the binary64 intersectBVH restatement (tMin =
 *    EPS, tMax = INF) instead of the GLSL's f32 traversal; spheres and the
 *    ground keep the GLSL's f32 tests and win when strictly closer;
 *  - shadow rays use the binary64 any-hit counterpart (any triangle the
 *    reference's Moller-Trumbore accepts in (EPS, tMax), boxes culled by its
 *    slab test at tMax);
 *  - alpha "blend" any-hit draws from a hash of (path RNG state, slot), not
 *    from the path's stream, so the stream does not depend on traversal order;
 *  - textures (colour/data map layers) are not supported (maps must be -1);
 *  - hardware bilinear filtering (env map, sheen LUT) is done in software in
 *    binary32 with the GL wrap rules.
 */
#include "oracle_render.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "oracle_core.h"

namespace {

template <class F>
void par_for(uint64_t n, int threads, F&& f) {
  if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
  if (threads == 1 || n < 64) {
    f(0, n);
    return;
  }
  std::vector<std::thread> pool;
  std::atomic<uint64_t> next(0);
  for (int k = 0; k < threads; k++)
    pool.emplace_back([&]() {
      for (;;) {
        const uint64_t b = next.fetch_add(16);
        if (b >= n) break;
        f(b, std::min(n, b + 16));
      }
    });
  for (auto& t : pool) t.join();
}

// ------------------------------------------------------------------ half floats
float half_round(float f) {  // binary32 -> binary16 (round to nearest even) -> binary32
  uint32_t x;
  std::memcpy(&x, &f, 4);
  const uint32_t sign = x & 0x80000000u;
  const uint32_t ax = x & 0x7fffffffu;
  uint32_t h;
  if (ax >= 0x7f800000u) {
    h = ax > 0x7f800000u ? 0x7e00u : 0x7c00u;
  } else if (ax >= 0x477ff000u) {  // rounds to >= 65520 -> inf
    h = 0x7c00u;
  } else if (ax < 0x38800000u) {  // subnormal half
    const float af = std::fabs(f);
    const float q = std::nearbyint(af * 16777216.0f);  // units of 2^-24
    h = (uint32_t)q;
  } else {
    const uint32_t e = (ax >> 23) - 112;
    uint32_t m = ax & 0x7fffffu;
    uint32_t r = (e << 10) | (m >> 13);
    const uint32_t rem = m & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (r & 1u))) r++;
    h = r;
  }
  // back to binary32
  const uint32_t hs = h & 0x7fffu;
  float out;
  if (hs >= 0x7c00u) {
    const uint32_t b = sign | 0x7f800000u | ((hs & 0x3ffu) << 13);
    std::memcpy(&out, &b, 4);
  } else if (hs < 0x400u) {
    out = (float)hs / 16777216.0f;
    if (sign) out = -out;
  } else {
    const uint32_t b = sign | ((((hs >> 10) + 112u) << 23) | ((hs & 0x3ffu) << 13));
    std::memcpy(&out, &b, 4);
  }
  return out;
}

// ------------------------------------------------------------------ vectors
template <class R>
struct Vec3 {
  R x, y, z;
};
template <class R>
struct Vec2 {
  R x, y;
};
template <class R> Vec3<R> v3(R a, R b, R c) { return {a, b, c}; }
template <class R> Vec3<R> operator+(Vec3<R> a, Vec3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> Vec3<R> operator-(Vec3<R> a, Vec3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R> Vec3<R> operator-(Vec3<R> a) { return {-a.x, -a.y, -a.z}; }
template <class R> Vec3<R> operator*(Vec3<R> a, Vec3<R> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class R> Vec3<R> operator*(Vec3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <class R> Vec3<R> operator*(R s, Vec3<R> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class R> Vec3<R> operator/(Vec3<R> a, R s) { return {a.x / s, a.y / s, a.z / s}; }
template <class R> Vec3<R> operator/(Vec3<R> a, Vec3<R> b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
template <class R> R dot(Vec3<R> a, Vec3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> Vec3<R> cross(Vec3<R> a, Vec3<R> b) {
  return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
template <class R> R length(Vec3<R> a) { return std::sqrt(dot(a, a)); }
template <class R> Vec3<R> normalize(Vec3<R> a) { return a / length(a); }
template <class R> Vec3<R> vmax(Vec3<R> a, R s) { return {std::max(a.x, s), std::max(a.y, s), std::max(a.z, s)}; }
template <class R> Vec3<R> vexp(Vec3<R> a) { return {std::exp(a.x), std::exp(a.y), std::exp(a.z)}; }
template <class R> Vec3<R> vlog(Vec3<R> a) { return {std::log(a.x), std::log(a.y), std::log(a.z)}; }
template <class R> R clampr(R x, R a, R b) { return std::min(std::max(x, a), b); }
template <class R> R mixr(R x, R y, R a) { return x * (R(1) - a) + y * a; }
template <class R> Vec3<R> mix3(Vec3<R> x, Vec3<R> y, R a) { return x * (R(1) - a) + y * a; }
template <class R> R smoothstep(R e0, R e1, R x) {
  const R t = clampr((x - e0) / (e1 - e0), R(0), R(1));
  return t * t * (R(3) - R(2) * t);
}
template <class R> Vec3<R> reflect(Vec3<R> I, Vec3<R> N) { return I - R(2) * dot(N, I) * N; }
template <class R> Vec3<R> refract(Vec3<R> I, Vec3<R> N, R eta) {
  const R k = R(1) - eta * eta * (R(1) - dot(N, I) * dot(N, I));
  if (k < R(0)) return {R(0), R(0), R(0)};
  return eta * I - (eta * dot(N, I) + std::sqrt(k)) * N;
}
template <class R> R max3(Vec3<R> v) { return std::max(v.x, std::max(v.y, v.z)); }
template <class R> R luminance(Vec3<R> c) { return dot(c, v3<R>(R(0.2126), R(0.7152), R(0.0722))); }

template <class R> struct K {  // common.glsl:4-8 constants at precision R
  static constexpr R PI = R(3.14159265358979323846);
  static constexpr R INV_PI = R(0.31830988618379067154);
  static constexpr R TWO_PI = R(6.28318530717958647692);
  static constexpr R INF = R(1e30);
  static constexpr R EPS = R(1e-6);
};

// ------------------------------------------------------------------ RNG (common.glsl:13-25)
inline uint32_t pcg(uint32_t& state) {
  const uint32_t s = state;
  state = s * 747796405u + 2891336453u;
  const uint32_t word = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
  return (word >> 22u) ^ word;
}

// Alpha any-hit uniform: hash of the path's RNG state and the slot (shared
// with the CUDA kernels), so traversal order never touches the path stream.
inline float alpha_rand(uint32_t key, uint32_t slot) {
  uint32_t s = key ^ (slot * 0x9E3779B9u);
  return (float)pcg(s) * (1.0f / 4294967296.0f);
}

// ------------------------------------------------------------------ scene access
inline const float* texel(const float* base, int i) { return base + (size_t)i * 4; }

struct Material {  // scene.glsl:140-201 fetchMaterial
  float albedo[3], metallic, roughness, ior, transmission, checkerScale, emission[3], alpha, albedo2[3];
  int alphaMode;
  int maps[4];
  float normalScale, clearcoat, clearcoatRoughness, alphaCutoff, sheenColor[3], sheenRoughness, attColor[3],
      attDist, uv0[3], uv1[3];
  bool thinWalled;
};

Material fetch_material_from(const float* mats, int index) {
  const float* t = mats + (size_t)index * 40;
  Material m;
  for (int k = 0; k < 3; k++) {
    m.albedo[k] = t[k];
    m.emission[k] = t[8 + k];
    m.albedo2[k] = t[12 + k];
    m.sheenColor[k] = t[24 + k];
    m.attColor[k] = t[28 + k];
    m.uv0[k] = t[32 + k];
    m.uv1[k] = t[36 + k];
  }
  m.metallic = t[3];
  m.roughness = t[4];
  m.ior = t[5];
  m.transmission = t[6];
  m.checkerScale = t[7];
  m.alpha = t[11];
  m.alphaMode = (int)t[15];
  for (int k = 0; k < 4; k++) m.maps[k] = (int)t[16 + k];
  m.normalScale = t[20];
  m.clearcoat = t[21];
  m.clearcoatRoughness = t[22];
  m.alphaCutoff = t[23];
  m.sheenRoughness = t[27];
  m.attDist = t[31];
  m.thinWalled = t[35] > 0.5f;
  return m;
}

// ------------------------------------------------------------------ textures
// Decode tables of the texture arrays: sRGB code -> linear (IEC 61966-2-1,
// binary64 rounded to binary32), code / 255, and the linear values of the
// code-value midpoints (the sRGB encoder's thresholds).
struct TexelTables {
  float srgb[256], unorm[256], mid[255];
  TexelTables() {
    auto eotf = [](double c) { return c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4); };
    for (int v = 0; v < 256; v++) {
      srgb[v] = (float)eotf(v / 255.0);
      unorm[v] = (float)v / 255.f;
    }
    for (int k = 0; k < 255; k++) mid[k] = (float)eotf((k + 0.5) / 255.0);
  }
};
const TexelTables& texel_tables() {
  static const TexelTables t;
  return t;
}

// textureLod(array, vec3(uv, layer), 0) with LINEAR filtering and REPEAT
// wrapping; sRGB layers decode before filtering, alpha is linear.
template <class R>
void sample_layer(const orc_scene* s, const uint8_t* tex, int layer, R u_in, R v_in, bool srgb, R out[4]) {
  const TexelTables& T = texel_tables();
  const int n = (int)s->tex_size;
  R u = u_in - std::floor(u_in), v = v_in - std::floor(v_in);
  if (!(u >= R(0) && u < R(1))) u = R(0);
  if (!(v >= R(0) && v < R(1))) v = R(0);
  const R x = u * R(n) - R(0.5), y = v * R(n) - R(0.5);
  const R x0 = std::floor(x), y0 = std::floor(y);
  const R fx = x - x0, fy = y - y0;
  const int ix = (int)x0, iy = (int)y0;
  const int xa = ix < 0 ? n - 1 : ix, xb = ix + 1 >= n ? 0 : ix + 1;
  const int ya = iy < 0 ? n - 1 : iy, yb = iy + 1 >= n ? 0 : iy + 1;
  const uint8_t* L = tex + (size_t)layer * n * n * 4;
  const uint8_t* t00 = L + ((size_t)ya * n + xa) * 4;
  const uint8_t* t10 = L + ((size_t)ya * n + xb) * 4;
  const uint8_t* t01 = L + ((size_t)yb * n + xa) * 4;
  const uint8_t* t11 = L + ((size_t)yb * n + xb) * 4;
  for (int c = 0; c < 4; c++) {
    const float* d = (srgb && c < 3) ? T.srgb : T.unorm;
    const R a = R(d[t00[c]]), b = R(d[t10[c]]), e = R(d[t01[c]]), f = R(d[t11[c]]);
    out[c] = (a * (R(1) - fx) + b * fx) * (R(1) - fy) + (e * (R(1) - fx) + f * fx) * fy;
  }
}

// alphaOpaque (scene.glsl:176-189): constant alpha times the base colour
// map's alpha at the hit's texture coordinates (barycentrics bu, bv).
bool alpha_opaque(const orc_scene* s, int slot, uint32_t key, float bu, float bv) {
  const float* g = s->geo + (size_t)slot * 12;
  const float* t = s->materials + (size_t)(int)g[3] * 40;
  float alpha = t[11];
  const int map = (int)t[16];
  if (map >= 0 && s->tex_size > 0) {
    const float* a = s->attr + (size_t)slot * 16;
    const float w = 1.f - bu - bv;
    const float u = a[3] * w + a[7] * bu + a[11] * bv, v = a[12] * w + a[13] * bu + a[14] * bv;
    const float tu = t[32] * u + t[33] * v + t[34], tv = t[36] * u + t[37] * v + t[38];
    float c[4];
    sample_layer<float>(s, s->color_maps, map, tu, tv, true, c);
    alpha *= c[3];
  }
  const int mode = (int)t[15];
  if (mode == 1) return alpha >= t[23];
  return alpha_rand(key, (uint32_t)slot) < alpha;
}

// Binary64 closest hit in intersectBVH's order (bvh.ts:265-320) over slots,
// with the alpha test applied before a hit may update `closest`.
struct TriHit {
  int slot;
  double t, u, v;
};

bool closest_tri(const orc_scene* s, orc::V3 o, orc::V3 d, double tMin, double tMax, uint32_t key, TriHit& h) {
  using namespace orc;
  h.slot = -1;
  if (s->tri_count == 0) return true;
  const double org[3] = {o.x, o.y, o.z};
  const double inv[3] = {1.0 / d.x, 1.0 / d.y, 1.0 / d.z};
  int stack[64];
  int sp = 0;
  stack[sp++] = 0;
  double closest = tMax;
  while (sp > 0) {
    const int n = stack[--sp];
    const float* nd = s->nodes + (size_t)n * 8;
    const double mn[3] = {nd[0], nd[1], nd[2]}, mx[3] = {nd[4], nd[5], nd[6]};
    if (slab(mn, mx, org, inv, closest) == INF) continue;
    if (nd[7] > 0) {
      for (int i = 0; i < (int)nd[7]; i++) {
        const int slot = (int)nd[3] + i;
        const float* g = s->geo + (size_t)slot * 12;
        double th, uh, vh;
        if (!tri_hit(o, d, {g[0], g[1], g[2]}, {g[4], g[5], g[6]}, {g[8], g[9], g[10]}, tMin, closest, th, uh, vh))
          continue;
        if (g[11] >= 0.5f && !alpha_opaque(s, slot, key, (float)uh, (float)vh)) continue;
        closest = th;
        h = {slot, th, uh, vh};
      }
    } else {
      if (sp + 2 > 64) return false;
      stack[sp++] = (int)nd[3] + 1;
      stack[sp++] = (int)nd[3];
    }
  }
  return true;
}

// Any-hit counterpart: some triangle accepted in (tMin, tMax) whose leaf the
// reference's slab test (at tMax) reaches. Independent of visiting order.
bool any_tri(const orc_scene* s, orc::V3 o, orc::V3 d, double tMin, double tMax, uint32_t key) {
  using namespace orc;
  if (s->tri_count == 0) return false;
  const double org[3] = {o.x, o.y, o.z};
  const double inv[3] = {1.0 / d.x, 1.0 / d.y, 1.0 / d.z};
  int stack[64];
  int sp = 0;
  stack[sp++] = 0;
  while (sp > 0) {
    const int n = stack[--sp];
    const float* nd = s->nodes + (size_t)n * 8;
    const double mn[3] = {nd[0], nd[1], nd[2]}, mx[3] = {nd[4], nd[5], nd[6]};
    if (slab(mn, mx, org, inv, tMax) == INF) continue;
    if (nd[7] > 0) {
      for (int i = 0; i < (int)nd[7]; i++) {
        const int slot = (int)nd[3] + i;
        const float* g = s->geo + (size_t)slot * 12;
        double th, uh, vh;
        if (!tri_hit(o, d, {g[0], g[1], g[2]}, {g[4], g[5], g[6]}, {g[8], g[9], g[10]}, tMin, tMax, th, uh, vh))
          continue;
        if (g[11] >= 0.5f && !alpha_opaque(s, slot, key, (float)uh, (float)vh)) continue;
        return true;
      }
    } else if (sp + 2 <= 64) {
      stack[sp++] = (int)nd[3] + 1;
      stack[sp++] = (int)nd[3];
    }
  }
  return false;
}

// Work counts of the reference's GLSL traversals (scene.glsl:218-267 closest,
// near-first, both child boxes read per inner node; :347-375 occluded,
// left-first, one box per visited node), used for algorithmic bytes.
struct WorkCounts {
  uint64_t closest_rays = 0, closest_inner = 0, closest_tris = 0;
  uint64_t shadow_rays = 0, shadow_nodes = 0, shadow_tris = 0;
};

inline float glsl_hit_aabb(const float* ro, const float* inv, const float* mn, const float* mx, float tmax) {
  float tmn[3], tmx[3];
  for (int i = 0; i < 3; i++) {
    const float t0 = (mn[i] - ro[i]) * inv[i], t1 = (mx[i] - ro[i]) * inv[i];
    tmn[i] = std::min(t0, t1);
    tmx[i] = std::max(t0, t1);
  }
  const float tn = std::max(std::max(tmn[0], tmn[1]), std::max(tmn[2], 0.0f));
  const float tf = std::min(std::min(tmx[0], tmx[1]), std::min(tmx[2], tmax));
  return tf >= tn ? tn : 1e30f;
}

inline bool glsl_hit_tri(const float* ro, const float* rd, const float* g, float tmax, float& t) {
  const float e1[3] = {g[4] - g[0], g[5] - g[1], g[6] - g[2]};
  const float e2[3] = {g[8] - g[0], g[9] - g[1], g[10] - g[2]};
  const float p[3] = {rd[1] * e2[2] - rd[2] * e2[1], rd[2] * e2[0] - rd[0] * e2[2], rd[0] * e2[1] - rd[1] * e2[0]};
  const float det = e1[0] * p[0] + e1[1] * p[1] + e1[2] * p[2];
  if (std::fabs(det) < 1e-12f) return false;
  const float invDet = 1.0f / det;
  const float s[3] = {ro[0] - g[0], ro[1] - g[1], ro[2] - g[2]};
  const float u = (s[0] * p[0] + s[1] * p[1] + s[2] * p[2]) * invDet;
  if (u < 0.0f || u > 1.0f) return false;
  const float q[3] = {s[1] * e1[2] - s[2] * e1[1], s[2] * e1[0] - s[0] * e1[2], s[0] * e1[1] - s[1] * e1[0]};
  const float v = (rd[0] * q[0] + rd[1] * q[1] + rd[2] * q[2]) * invDet;
  if (v < 0.0f || u + v > 1.0f) return false;
  t = (e2[0] * q[0] + e2[1] * q[1] + e2[2] * q[2]) * invDet;
  return t > 1e-6f && t < tmax;
}

void count_closest(const orc_scene* s, const float* ro, const float* rd, WorkCounts& w) {
  w.closest_rays++;
  if (s->tri_count == 0) return;
  const float inv[3] = {1.0f / rd[0], 1.0f / rd[1], 1.0f / rd[2]};
  float closest = 1e30f;
  int stack[40], sp = 0, node = 0;
  for (int iter = 0; iter < 8192; iter++) {
    const float* nd = s->nodes + (size_t)node * 8;
    const int first = (int)nd[3], count = (int)nd[7];
    if (count > 0) {
      for (int k = 0; k < count; k++) {
        w.closest_tris++;
        float t;
        if (glsl_hit_tri(ro, rd, s->geo + (size_t)(first + k) * 12, closest, t)) closest = t;
      }
      if (sp == 0) break;
      node = stack[--sp];
      continue;
    }
    w.closest_inner++;
    int l = first, r = first + 1;
    const float* L = s->nodes + (size_t)l * 8;
    const float* R = s->nodes + (size_t)r * 8;
    float tl = glsl_hit_aabb(ro, inv, L, L + 4, closest), tr = glsl_hit_aabb(ro, inv, R, R + 4, closest);
    if (tl > tr) {
      std::swap(tl, tr);
      std::swap(l, r);
    }
    if (tl == 1e30f) {
      if (sp == 0) break;
      node = stack[--sp];
    } else {
      node = l;
      if (tr != 1e30f && sp < 40) stack[sp++] = r;
    }
  }
}

void count_shadow(const orc_scene* s, const float* ro, const float* rd, float tmax, WorkCounts& w) {
  w.shadow_rays++;
  if (s->tri_count == 0) return;
  const float inv[3] = {1.0f / rd[0], 1.0f / rd[1], 1.0f / rd[2]};
  int stack[40], sp = 0, node = 0;
  for (int iter = 0; iter < 8192; iter++) {
    const float* nd = s->nodes + (size_t)node * 8;
    w.shadow_nodes++;
    if (glsl_hit_aabb(ro, inv, nd, nd + 4, tmax) == 1e30f) {
      if (sp == 0) return;
      node = stack[--sp];
      continue;
    }
    const int first = (int)nd[3], count = (int)nd[7];
    if (count > 0) {
      for (int k = 0; k < count; k++) {
        w.shadow_tris++;
        float t;
        if (glsl_hit_tri(ro, rd, s->geo + (size_t)(first + k) * 12, tmax, t)) return;
      }
      if (sp == 0) return;
      node = stack[--sp];
    } else {
      node = first;
      if (sp < 40) stack[sp++] = first + 1;
    }
  }
}

// Software bilinear sample (GL LINEAR) of an RGB/1-channel f32 image.
template <class R>
void bilinear(const float* img, int w, int h, int ch, R u, R v, bool repeat_s, R* out) {
  const R x = u * R(w) - R(0.5), y = v * R(h) - R(0.5);
  const R fx = std::floor(x), fy = std::floor(y);
  const R ax = x - fx, ay = y - fy;
  int x0 = (int)fx, y0 = (int)fy, x1 = x0 + 1, y1 = y0 + 1;
  auto wrap = [&](int i, int n, bool rep) {
    if (rep) {
      i %= n;
      return i < 0 ? i + n : i;
    }
    return i < 0 ? 0 : (i >= n ? n - 1 : i);
  };
  x0 = wrap(x0, w, repeat_s);
  x1 = wrap(x1, w, repeat_s);
  y0 = wrap(y0, h, false);
  y1 = wrap(y1, h, false);
  for (int c = 0; c < ch; c++) {
    const R a = img[((size_t)y0 * w + x0) * ch + c], b = img[((size_t)y0 * w + x1) * ch + c];
    const R cc = img[((size_t)y1 * w + x0) * ch + c], d = img[((size_t)y1 * w + x1) * ch + c];
    const R top = a * (R(1) - ax) + b * ax, bot = cc * (R(1) - ax) + d * ax;
    out[c] = top * (R(1) - ay) + bot * ay;
  }
}

// ------------------------------------------------------------------ the tracer
template <class R>
struct Tracer {
  using V = Vec3<R>;
  using V2 = Vec2<R>;
  using C = K<R>;
  const orc_scene* s;
  const orc_camera* cam;
  uint32_t W, H, maxBounces;
  R uClamp;
  uint32_t g_seed = 0;
  WorkCounts* wc = nullptr;  // when set, counts rays (and, if `detailed`, their GLSL traversal work)
  bool detailed = true;
  // Detached evaluation (tracePathDetached): materials and environment texels
  // whose values are used for every BSDF value and emitted radiance, while
  // sampling keeps s's (nullptr: s's own).
  const float* mev = nullptr;
  const float* eev = nullptr;

  R rand() { return R(pcg(g_seed)) * (R(1) / R(4294967296.0)); }
  V2 rand2() {
    const R a = rand();
    const R b = rand();
    return {a, b};
  }
  static V f3(const float* p) { return {R(p[0]), R(p[1]), R(p[2])}; }

  // common.glsl:29-35
  static void basis(V n, V& t, V& b) {
    const R sg = n.z >= R(0) ? R(1) : R(-1);
    const R a = R(-1) / (sg + n.z);
    const R c = n.x * n.y * a;
    t = {R(1) + sg * n.x * n.x * a, sg * c, -sg * n.x};
    b = {c, sg + n.y * n.y * a, -n.y};
  }
  static V toWorld(V v, V t, V b, V n) { return t * v.x + b * v.y + n * v.z; }
  static V toLocal(V v, V t, V b, V n) { return {dot(v, t), dot(v, b), dot(v, n)}; }
  static V cosineHemisphere(V2 u) {  // :46-52
    const R r = std::sqrt(u.x), phi = C::TWO_PI * u.y;
    return {r * std::cos(phi), r * std::sin(phi), std::sqrt(std::max(R(0), R(1) - u.x))};
  }
  static V uniformCone(V2 u, R cosThetaMax) {  // :55-60
    const R cosTheta = R(1) - u.x * (R(1) - cosThetaMax);
    const R sinTheta = std::sqrt(std::max(R(0), R(1) - cosTheta * cosTheta));
    const R phi = C::TWO_PI * u.y;
    return {sinTheta * std::cos(phi), sinTheta * std::sin(phi), cosTheta};
  }
  static V2 concentricDisk(V2 u) {  // :63-75
    const V2 o = {R(2) * u.x - R(1), R(2) * u.y - R(1)};
    if (o.x == R(0) && o.y == R(0)) return {R(0), R(0)};
    R r, theta;
    if (std::fabs(o.x) > std::fabs(o.y)) {
      r = o.x;
      theta = (C::PI / R(4)) * (o.y / o.x);
    } else {
      r = o.y;
      theta = (C::PI / R(2)) - (C::PI / R(4)) * (o.x / o.y);
    }
    return {r * std::cos(theta), r * std::sin(theta)};
  }
  static R misWeight(R a, R b) {  // :82-86
    const R a2 = a * a, b2 = b * b;
    return a2 / std::max(a2 + b2, R(1e-10));
  }
  // offsetRay (:95-108) works on binary32 bit patterns in both precisions.
  static V offsetRay(V pR, V nR) {
    const float p[3] = {(float)pR.x, (float)pR.y, (float)pR.z}, n[3] = {(float)nR.x, (float)nR.y, (float)nR.z};
    float out[3];
    for (int k = 0; k < 3; k++) {
      const int o = (int)(256.0f * n[k]);
      int32_t bits;
      std::memcpy(&bits, &p[k], 4);
      bits += p[k] < 0.0f ? -o : o;
      float pi;
      std::memcpy(&pi, &bits, 4);
      out[k] = std::fabs(p[k]) < (1.0f / 32.0f) ? p[k] + (1.0f / 65536.0f) * n[k] : pi;
    }
    return {R(out[0]), R(out[1]), R(out[2])};
  }

  // ---------------------------------------------------------------- scene.glsl
  R hitSphere(V ro, V rd, const float* sp, R tMax) const {  // :132-144
    const V oc = ro - f3(sp);
    const R b = dot(oc, rd);
    const R c = dot(oc, oc) - R(sp[3]) * R(sp[3]);
    const R disc = b * b - c;
    if (disc < R(0)) return C::INF;
    const R sq = std::sqrt(disc);
    R t = -b - sq;
    if (t > C::EPS && t < tMax) return t;
    t = -b + sq;
    if (t > C::EPS && t < tMax) return t;
    return C::INF;
  }
  R hitGround(V ro, V rd, R tMax) const {  // :146-150
    if (s->ground_material < 0 || std::fabs(rd.y) < R(1e-9)) return C::INF;
    const R t = (R(s->ground_height) - ro.y) / rd.y;
    return t > C::EPS && t < tMax ? t : C::INF;
  }

  struct Hit {
    R t;
    V position, normal, geomNormal;
    bool frontFace;
    int material, light;
    Vec2<R> uv;
    V dpdu, dpdv;  // zero without texture coordinates (scene.glsl:108-109)
  };

  // traceScene (:192-333), triangle part replaced by the binary64 closest hit.
  bool traceScene(V ro, V rd, Hit& hit) {
    R closest = C::INF;
    int bestSphere = -1;
    bool ground = false;
    for (uint32_t i = 0; i < s->sphere_count; i++) {
      const R t = hitSphere(ro, rd, s->spheres + 4 * i, closest);
      if (t < closest) {
        closest = t;
        bestSphere = (int)i;
      }
    }
    const R tg = hitGround(ro, rd, closest);
    if (tg < closest) {
      closest = tg;
      bestSphere = -1;
      ground = true;
    }
    if (wc && detailed) {
      const float rf[3] = {(float)ro.x, (float)ro.y, (float)ro.z}, df[3] = {(float)rd.x, (float)rd.y, (float)rd.z};
      count_closest(s, rf, df, *wc);
    } else if (wc) {
      wc->closest_rays++;
    }
    TriHit th;
    closest_tri(s, {(double)ro.x, (double)ro.y, (double)ro.z}, {(double)rd.x, (double)rd.y, (double)rd.z}, 1e-6,
                1e30, g_seed, th);
    int bestTri = -1;
    Vec2<R> bary = {R(0), R(0)};
    if (th.slot >= 0 && R(th.t) < closest) {
      closest = R(th.t);
      bestTri = th.slot;
      bary = {R(th.u), R(th.v)};
      bestSphere = -1;
      ground = false;
    }
    if (bestTri < 0 && bestSphere < 0 && !ground) return false;
    hit.t = closest;
    hit.position = ro + rd * closest;
    hit.uv = {R(0), R(0)};
    hit.dpdu = hit.dpdv = {R(0), R(0), R(0)};
    hit.light = -1;
    if (ground) {
      hit.frontFace = rd.y < R(0);
      hit.normal = {R(0), hit.frontFace ? R(1) : R(-1), R(0)};
      hit.geomNormal = hit.normal;
      hit.material = s->ground_material;
      hit.uv = {hit.position.x, hit.position.z};
      return true;
    }
    if (bestSphere >= 0) {
      const float* sp = s->spheres + 4 * bestSphere;
      const V n = (hit.position - f3(sp)) / R(sp[3]);
      hit.frontFace = dot(rd, n) < R(0);
      hit.normal = hit.frontFace ? n : -n;
      hit.geomNormal = hit.normal;
      hit.material = s->sphere_materials[bestSphere];
      hit.light = s->sphere_lights[bestSphere];
      return true;
    }
    const float* g = s->geo + (size_t)bestTri * 12;
    const float* a = s->attr + (size_t)bestTri * 16;
    const V p0 = f3(g), p1 = f3(g + 4), p2 = f3(g + 8);
    const V n0 = f3(a), n1 = f3(a + 4), n2 = f3(a + 8);
    const Vec2<R> uv0 = {R(a[3]), R(a[12])}, uv1 = {R(a[7]), R(a[13])}, uv2 = {R(a[11]), R(a[14])};
    const R w = R(1) - bary.x - bary.y;
    hit.uv = {uv0.x * w + uv1.x * bary.x + uv2.x * bary.y, uv0.y * w + uv1.y * bary.x + uv2.y * bary.y};
    const V e1 = p1 - p0, e2 = p2 - p0;
    const Vec2<R> d1 = {uv1.x - uv0.x, uv1.y - uv0.y}, d2 = {uv2.x - uv0.x, uv2.y - uv0.y};
    const R det = d1.x * d2.y - d1.y * d2.x;
    if (std::fabs(det) > R(1e-12)) {  // scene.glsl:314-319
      const R r = R(1) / det;
      hit.dpdu = (e1 * d2.y - e2 * d1.y) * r;
      hit.dpdv = (e2 * d1.x - e1 * d2.x) * r;
    }
    V ng = normalize(cross(e1, e2));
    V ns = normalize(n0 * w + n1 * bary.x + n2 * bary.y);
    hit.frontFace = dot(rd, ng) < R(0);
    if (!hit.frontFace) {
      ng = -ng;
      ns = -ns;
    }
    if (dot(ns, ng) < R(0.05)) ns = ng;
    hit.normal = ns;
    hit.geomNormal = ng;
    hit.material = (int)g[3];
    hit.light = (int)g[7];
    return true;
  }

  bool occluded(V ro, V rd, R tMax) {  // :336-377
    for (uint32_t i = 0; i < s->sphere_count; i++)
      if (hitSphere(ro, rd, s->spheres + 4 * i, tMax) < tMax) return true;
    if (hitGround(ro, rd, tMax) < tMax) return true;
    if (s->tri_count == 0) return false;
    if (wc && detailed) {
      const float rf[3] = {(float)ro.x, (float)ro.y, (float)ro.z}, df[3] = {(float)rd.x, (float)rd.y, (float)rd.z};
      count_shadow(s, rf, df, (float)tMax, *wc);
    } else if (wc) {
      wc->shadow_rays++;
    }
    return any_tri(s, {(double)ro.x, (double)ro.y, (double)ro.z}, {(double)rd.x, (double)rd.y, (double)rd.z}, 1e-6,
                   (double)tMax, g_seed);
  }

  // ---------------------------------------------------------------- lights.glsl
  V envToLocal(V d) const {
    const R c = R(s->env_rot_cos), sn = R(s->env_rot_sin);
    return {c * d.x - sn * d.z, d.y, sn * d.x + c * d.z};
  }
  V envToWorld(V l) const {
    const R c = R(s->env_rot_cos), sn = R(s->env_rot_sin);
    return {c * l.x + sn * l.z, l.y, -sn * l.x + c * l.z};
  }
  static Vec2<R> equirectUV(V l) {
    return {std::atan2(l.z, l.x) * (R(0.5) * C::INV_PI) + R(0.5), std::acos(clampr(l.y, R(-1), R(1))) * C::INV_PI};
  }
  V envTex(Vec2<R> uv) const {
    R out[3];
    bilinear<R>(s->env_rgb, (int)s->env_width, (int)s->env_height, 3, uv.x, uv.y, true, out);
    return {out[0], out[1], out[2]};
  }
  V envTexEv(Vec2<R> uv) const {
    if (!eev) return envTex(uv);
    R out[3];
    bilinear<R>(eev, (int)s->env_width, (int)s->env_height, 3, uv.x, uv.y, true, out);
    return {out[0], out[1], out[2]};
  }
  V envRadiance(V d) const { return envTex(equirectUV(envToLocal(d))) * R(s->env_intensity); }
  const float* aliasTexel(int cx, int cy) const { return s->env_alias + ((size_t)cy * s->env_grid_w + cx) * 4; }
  R envPdf(V d) const {  // :50-56
    const V l = envToLocal(d);
    const R sinTheta = std::sqrt(std::max(R(0), R(1) - l.y * l.y));
    if (sinTheta < R(1e-6)) return R(0);
    const Vec2<R> uv = equirectUV(l);
    const int cx = std::min((int)(uv.x * R(s->env_grid_w)), (int)s->env_grid_w - 1);
    const int cy = std::min((int)(uv.y * R(s->env_grid_h)), (int)s->env_grid_h - 1);
    return R(aliasTexel(cx, cy)[2]) / (R(2) * C::PI * C::PI * sinTheta);
  }
  struct LightSample {
    V dir;
    R dist, pdf;
    V radiance;
    Vec2<R> uv;  // environment samples: texture coordinate of the radiance lookup
  };
  LightSample sampleEnvironment() {  // :59-79
    LightSample ls;
    const int gw = (int)s->env_grid_w, gh = (int)s->env_grid_h;
    const int n = gw * gh;
    const int i = std::min((int)(rand() * R(n)), n - 1);
    const float* e = aliasTexel(i % gw, i / gw);
    int cell = i;
    R pdfUV = R(e[2]);
    if (rand() >= R(e[0])) {
      cell = (int)e[1];
      pdfUV = R(e[3]);
    }
    const V2 j = rand2();
    const Vec2<R> uv = {(R(cell % gw) + j.x) / R(gw), (R(cell / gw) + j.y) / R(gh)};
    const R phi = (uv.x - R(0.5)) * C::TWO_PI, theta = uv.y * C::PI;
    const R sinTheta = std::sin(theta);
    ls.dir = envToWorld({sinTheta * std::cos(phi), std::cos(theta), sinTheta * std::sin(phi)});
    ls.dist = C::INF;
    ls.pdf = sinTheta > R(1e-6) ? pdfUV / (R(2) * C::PI * C::PI * sinTheta) : R(0);
    ls.radiance = envTex(uv) * R(s->env_intensity);
    ls.uv = uv;
    return ls;
  }
  V environment(V d, bool specularBounce, R bsdfPdf) const {  // :83-91
    V L = envRadiance(d);
    if (!specularBounce && s->env_sampling != 0) L = L * misWeight(bsdfPdf, envPdf(d));
    if (s->sun_enabled != 0 && dot(d, f3(s->sun_dir)) >= R(s->sun_cos_angle)) {
      const R w = specularBounce ? R(1) : misWeight(bsdfPdf, R(s->sun_pdf));
      L = L + f3(s->sun_radiance) * w;
    }
    return L;
  }
  V environmentEv(V d, bool specularBounce, R bsdfPdf) const {  // environment() with eev's radiance
    V L = envTexEv(equirectUV(envToLocal(d))) * R(s->env_intensity);
    if (!specularBounce && s->env_sampling != 0) L = L * misWeight(bsdfPdf, envPdf(d));
    if (s->sun_enabled != 0 && dot(d, f3(s->sun_dir)) >= R(s->sun_cos_angle)) {
      const R w = specularBounce ? R(1) : misWeight(bsdfPdf, R(s->sun_pdf));
      L = L + f3(s->sun_radiance) * w;
    }
    return L;
  }
  V sampleSunDirection(V2 u) const {  // :93-97
    V t, b;
    const V sd = f3(s->sun_dir);
    basis(sd, t, b);
    return toWorld(uniformCone(u, R(s->sun_cos_angle)), t, b, sd);
  }
  LightSample sampleLight(int index, V p, V2 u) const {  // :99-138
    LightSample ls;
    ls.pdf = R(0);
    const float* l0 = s->lights + (size_t)index * 16;
    const float *l1 = l0 + 4, *l2 = l0 + 8;
    ls.radiance = f3(l0 + 12);
    ls.dir = {R(0), R(0), R(0)};
    ls.dist = R(0);
    if (l0[3] < 0.5f) {
      const V toC = f3(l0) - p;
      const R d2 = dot(toC, toC);
      const R r = R(l1[3]);
      if (d2 <= r * r) return ls;
      const R cosMax = std::sqrt(std::max(R(0), R(1) - r * r / d2));
      const V axis = toC * (R(1) / std::sqrt(d2));
      V t, b;
      basis(axis, t, b);
      ls.dir = toWorld(uniformCone(u, cosMax), t, b, axis);
      ls.pdf = R(1) / (C::TWO_PI * (R(1) - cosMax));
      const float sp[4] = {l0[0], l0[1], l0[2], l1[3]};
      const R t0 = hitSphere(p, ls.dir, sp, C::INF);
      ls.dist = t0 < C::INF ? t0 : std::sqrt(d2);
    } else {
      const V e1 = f3(l1), e2 = f3(l2);
      const V q = f3(l0) + e1 * u.x + e2 * u.y;
      const V toQ = q - p;
      const R d2 = dot(toQ, toQ);
      const R d = std::sqrt(d2);
      ls.dir = toQ / d;
      ls.dist = d;
      const V nCross = cross(e1, e2);
      const R area = length(nCross);
      const R cosL = std::fabs(dot(nCross / area, ls.dir));
      if (cosL < R(1e-4)) return ls;
      ls.pdf = d2 / (cosL * area);
    }
    return ls;
  }
  R lightPdf(int index, V p, V dir, R dist) const {  // :141-158
    const float* l0 = s->lights + (size_t)index * 16;
    const float *l1 = l0 + 4, *l2 = l0 + 8;
    if (l0[3] < 0.5f) {
      const V toC = f3(l0) - p;
      const R d2 = dot(toC, toC);
      const R r = R(l1[3]);
      if (d2 <= r * r) return R(0);
      const R cosMax = std::sqrt(std::max(R(0), R(1) - r * r / d2));
      return R(1) / (C::TWO_PI * (R(1) - cosMax));
    }
    const V nCross = cross(f3(l1), f3(l2));
    const R area = length(nCross);
    const R cosL = std::fabs(dot(nCross / area, dir));
    if (cosL < R(1e-4)) return R(0);
    return dist * dist / (cosL * area);
  }

  // ---------------------------------------------------------------- bsdf.glsl
  struct Surface {
    V albedo;
    R metallic, roughness, ior, transmission;
    V emission;
    R clearcoat, clearcoatRoughness;
    V sheenColor;
    R sheenRoughness;
    bool thinWalled;
    V absorption, n, nc;
  };
  static R D_GGX(R NdotH, R a) {
    const R a2 = a * a;
    const R d = NdotH * NdotH * (a2 - R(1)) + R(1);
    return a2 / (C::PI * d * d);
  }
  static R G1_GGX(R NdotX, R a) {
    const R a2 = a * a;
    return R(2) * NdotX / (NdotX + std::sqrt(a2 + (R(1) - a2) * NdotX * NdotX));
  }
  static V fresnelSchlick3(R cosTheta, V F0) {
    const R f = std::pow(R(1) - clampr(cosTheta, R(0), R(1)), R(5));
    return F0 + (V{R(1), R(1), R(1)} - F0) * f;
  }
  static R fresnelSchlick1(R cosTheta, R F0) {
    return F0 + (R(1) - F0) * std::pow(R(1) - clampr(cosTheta, R(0), R(1)), R(5));
  }
  static R dielectricF0(R ior) {
    const R r = (ior - R(1)) / (ior + R(1));
    return r * r;
  }
  static V sampleGGXVNDF(V Ve, R a, V2 u) {  // :59-72
    const V Vh = normalize(V{a * Ve.x, a * Ve.y, Ve.z});
    const R lensq = Vh.x * Vh.x + Vh.y * Vh.y;
    const V T1 = lensq > R(0) ? V{-Vh.y, Vh.x, R(0)} * (R(1) / std::sqrt(lensq)) : V{R(1), R(0), R(0)};
    const V T2 = cross(Vh, T1);
    const R r = std::sqrt(u.x), phi = C::TWO_PI * u.y;
    const R t1 = r * std::cos(phi);
    R t2 = r * std::sin(phi);
    const R sv = R(0.5) * (R(1) + Vh.z);
    t2 = (R(1) - sv) * std::sqrt(std::max(R(0), R(1) - t1 * t1)) + sv * t2;
    const V Nh = t1 * T1 + t2 * T2 + std::sqrt(std::max(R(0), R(1) - t1 * t1 - t2 * t2)) * Vh;
    return normalize(V{a * Nh.x, a * Nh.y, std::max(R(0), Nh.z)});
  }
  static R alphaFromRoughness(R roughness) { return std::max(roughness * roughness, R(1e-3)); }
  static R D_Charlie(R alpha, R NdotH) {
    const R inv = R(1) / alpha;
    const R sin2 = std::max(R(1) - NdotH * NdotH, R(0));
    return (R(2) + inv) * std::pow(sin2, inv * R(0.5)) / C::TWO_PI;
  }
  static R V_Neubelt(R NdotL, R NdotV) { return R(1) / (R(4) * (NdotL + NdotV - NdotL * NdotV)); }
  R sheenAlbedo(R NdotV, R roughness) const {  // :89-92, LINEAR filter on the 16x16 R16F LUT
    const R u = (NdotV * R(15) + R(0.5)) / R(16), v = (roughness * R(15) + R(0.5)) / R(16);
    R out;
    bilinear<R>(s->sheen_lut, 16, 16, 1, u, v, false, &out);
    return out;
  }
  static R specularProbability(V F0, R metallic, R NdotV) {
    const R f = luminance(fresnelSchlick3(NdotV, F0));
    return mixr(clampr(f, R(0.1), R(0.9)), R(1), metallic);
  }
  static R coatProbability(const Surface& sf, V wo) {
    if (sf.clearcoat <= R(0)) return R(0);
    const R Fc = sf.clearcoat * fresnelSchlick1(std::max(dot(sf.nc, wo), R(0)), R(0.04));
    const R base = (R(1) - Fc) * std::max(luminance(sf.albedo), R(0.04));
    return clampr(Fc / (Fc + base), R(0.15), R(0.85));
  }
  static V baseF0(const Surface& sf) {
    const R d = dielectricF0(sf.ior);
    return mix3(V{d, d, d}, sf.albedo, sf.metallic);
  }
  V evalOpaque(const Surface& sf, V wo, V wi, R& pdf) const {  // :114-166
    const V n = sf.n;
    const R NdotL = dot(n, wi), NdotV = dot(n, wo);
    pdf = R(0);
    if (NdotL <= R(0) || NdotV <= R(0)) return {R(0), R(0), R(0)};
    const R a = alphaFromRoughness(sf.roughness);
    const V Hh = normalize(wo + wi);
    const R NdotH = std::max(dot(n, Hh), R(0)), VdotH = std::max(dot(wo, Hh), R(0));
    const V F0 = baseF0(sf);
    const V F = fresnelSchlick3(VdotH, F0);
    const R D = D_GGX(NdotH, a);
    const R G1v = G1_GGX(NdotV, a);
    const R G = G1v * G1_GGX(NdotL, a);
    const V specular = (F * (D * G)) / std::max(R(4) * NdotV * NdotL, R(1e-6));
    const V diffuse = (V{R(1), R(1), R(1)} - F) * sf.albedo * (R(1) - sf.metallic) * C::INV_PI;
    V f = diffuse + specular;
    const R pSpec = specularProbability(F0, sf.metallic, NdotV);
    pdf = mixr(NdotL * C::INV_PI, G1v * D / std::max(R(4) * NdotV, R(1e-6)), pSpec);
    const R sheenMax = max3(sf.sheenColor);
    if (sheenMax > R(0)) {
      const R sr = std::max(sf.sheenRoughness, R(0.07));
      const V sheen = sf.sheenColor * D_Charlie(sr * sr, NdotH) * V_Neubelt(NdotL, NdotV);
      const R scale = R(1) - sheenMax * std::max(sheenAlbedo(NdotV, sr), sheenAlbedo(NdotL, sr));
      f = sheen + f * scale;
    }
    const R pCoat = coatProbability(sf, wo);
    if (pCoat > R(0)) {
      const R cV = dot(sf.nc, wo), cL = dot(sf.nc, wi);
      V coat = {R(0), R(0), R(0)};
      R pdfCoat = R(0);
      if (cV > R(0) && cL > R(0)) {
        const R ac = alphaFromRoughness(sf.clearcoatRoughness);
        const R cH = std::max(dot(sf.nc, Hh), R(0));
        const R Dc = D_GGX(cH, ac);
        const R G1c = G1_GGX(cV, ac);
        const R cv = Dc * G1c * G1_GGX(cL, ac) * fresnelSchlick1(VdotH, R(0.04)) / (R(4) * cV * cL);
        coat = {cv, cv, cv};
        pdfCoat = G1c * Dc / (R(4) * cV);
      }
      const R Fcv = fresnelSchlick1(std::max(cV, R(0)), R(0.04));
      f = f * (R(1) - sf.clearcoat * Fcv) + coat * sf.clearcoat;
      pdf = mixr(pdf, pdfCoat, pCoat);
    }
    return f;
  }
  struct BSDFSample {
    V dir, weight;
    R pdf;
  };
  // sampleOpaque (:174-211); `u` supplies the uniforms in the order the GLSL draws them.
  template <class U>
  BSDFSample sampleOpaque(const Surface& sf, V wo, U&& u) const {
    BSDFSample bs;
    bs.pdf = R(0);
    bs.weight = {R(0), R(0), R(0)};
    bs.dir = {R(0), R(0), R(0)};
    V wi;
    if (u() < coatProbability(sf, wo)) {
      V t, b;
      basis(sf.nc, t, b);
      const V woL = toLocal(wo, t, b, sf.nc);
      if (woL.z <= R(0)) return bs;
      const R a0 = u();
      const R a1 = u();
      const V Hh = sampleGGXVNDF(woL, alphaFromRoughness(sf.clearcoatRoughness), V2{a0, a1});
      wi = toWorld(reflect(-woL, Hh), t, b, sf.nc);
    } else {
      V t, b;
      basis(sf.n, t, b);
      const V woL = toLocal(wo, t, b, sf.n);
      if (woL.z <= R(0)) return bs;
      V wiL;
      if (u() < specularProbability(baseF0(sf), sf.metallic, woL.z)) {
        const R a0 = u();
        const R a1 = u();
        const V Hh = sampleGGXVNDF(woL, alphaFromRoughness(sf.roughness), V2{a0, a1});
        wiL = reflect(-woL, Hh);
      } else {
        const R a0 = u();
        const R a1 = u();
        wiL = cosineHemisphere(V2{a0, a1});
      }
      wi = toWorld(wiL, t, b, sf.n);
    }
    const R NdotL = dot(sf.n, wi);
    if (NdotL <= R(0)) return bs;
    R pdf;
    const V f = evalOpaque(sf, wo, wi, pdf);
    if (pdf <= R(0)) return bs;
    bs.dir = wi;
    bs.pdf = pdf;
    bs.weight = f * NdotL / pdf;
    return bs;
  }
  // sampleDielectric (:216-248).
  template <class U>
  bool sampleDielectric(const Surface& sf, bool frontFace, V ng, V wo, V& wi, V& weight, bool& reflected,
                        U&& u) const {
    const V n = sf.n;
    V t, b;
    basis(n, t, b);
    const V woL = toLocal(wo, t, b, n);
    if (woL.z <= R(0)) return false;
    V Hh = n;
    if (sf.roughness > R(0)) {
      const R a0 = u();
      const R a1 = u();
      const V HL = sampleGGXVNDF(woL, alphaFromRoughness(sf.roughness), V2{a0, a1});
      Hh = toWorld(HL, t, b, n);
    }
    R cosI = dot(wo, Hh);
    if (cosI <= R(0)) {
      Hh = n;
      cosI = woL.z;
    }
    const R eta = frontFace ? R(1) / sf.ior : sf.ior;
    const R sin2T = eta * eta * (R(1) - cosI * cosI);
    R Fr = fresnelSchlick1(cosI, dielectricF0(sf.ior));
    if (sf.thinWalled)
      Fr = R(2) * Fr / (R(1) + Fr);
    else if (sin2T > R(1))
      Fr = R(1);
    if (u() < Fr) {
      wi = reflect(-wo, Hh);
      weight = {R(1), R(1), R(1)};
      reflected = true;
      return dot(wi, ng) > R(0);
    }
    wi = sf.thinWalled ? -wo : refract(-wo, Hh, eta);
    weight = sf.albedo;
    reflected = false;
    return dot(wi, ng) < R(0);
  }

  // ---------------------------------------------------------------- trace.frag
  V clampContribution(V c, int bounce) const {  // :65-69
    if (bounce == 0 || uClamp <= R(0)) return c;
    const R l = luminance(c);
    return l > uClamp ? c * (uClamp / l) : c;
  }
  Surface surfaceAt(const Hit& hit, V wo, V& emission) const { return surfaceAtFrom(s->materials, hit, wo, emission); }
  Surface surfaceAtFrom(const float* mats, const Hit& hit, V wo, V& emission) const {  // :72-124
    const Material m = fetch_material_from(mats, hit.material);
    Surface sf;
    sf.albedo = f3(m.albedo);
    if (m.checkerScale > 0.0f) {
      const V q = {std::floor(hit.position.x * R(m.checkerScale) + R(0.5)),
                   std::floor(hit.position.y * R(m.checkerScale) + R(0.5)),
                   std::floor(hit.position.z * R(m.checkerScale) + R(0.5))};
      const R sum = q.x + q.y + q.z;
      const R md = sum - R(2) * std::floor(sum / R(2));
      if (md >= R(0.5)) sf.albedo = f3(m.albedo2);
    }
    sf.metallic = R(m.metallic);
    sf.roughness = R(m.roughness);
    emission = f3(m.emission);
    sf.nc = hit.normal;
    sf.n = hit.normal;
    if (s->tex_size > 0 && std::max(std::max(m.maps[0], m.maps[1]), std::max(m.maps[2], m.maps[3])) >= 0) {
      const R tu = R(m.uv0[0]) * hit.uv.x + R(m.uv0[1]) * hit.uv.y + R(m.uv0[2]);
      const R tv = R(m.uv1[0]) * hit.uv.x + R(m.uv1[1]) * hit.uv.y + R(m.uv1[2]);
      R c[4];
      if (m.maps[0] >= 0) {
        sample_layer<R>(s, s->color_maps, m.maps[0], tu, tv, true, c);
        sf.albedo = sf.albedo * V{c[0], c[1], c[2]};
      }
      if (m.maps[1] >= 0) {
        sample_layer<R>(s, s->data_maps, m.maps[1], tu, tv, false, c);
        sf.roughness = sf.roughness * c[1];
        sf.metallic = sf.metallic * c[2];
      }
      if (m.maps[3] >= 0) {
        sample_layer<R>(s, s->color_maps, m.maps[3], tu, tv, true, c);
        emission = emission * V{c[0], c[1], c[2]};
      }
      if (m.maps[2] >= 0 && dot(hit.dpdu, hit.dpdu) > R(0)) {  // :98-110
        const V N = hit.frontFace ? hit.normal : -hit.normal;
        const V T = normalize(hit.dpdu - N * dot(N, hit.dpdu));
        V B = cross(N, T);
        if (dot(B, -hit.dpdv) < R(0)) B = -B;
        sample_layer<R>(s, s->data_maps, m.maps[2], tu, tv, false, c);
        const R tx = (c[0] * R(2) - R(1)) * R(m.normalScale), ty = (c[1] * R(2) - R(1)) * R(m.normalScale);
        const R tz = c[2] * R(2) - R(1);
        V mapped = normalize(T * tx + B * ty + N * std::max(tz, R(1e-3)));
        mapped = hit.frontFace ? mapped : -mapped;
        if (dot(mapped, wo) > R(1e-3) && dot(mapped, hit.geomNormal) > R(0)) sf.n = mapped;
      }
    }
    sf.ior = R(m.ior);
    sf.transmission = R(m.transmission) * (R(1) - sf.metallic);
    sf.emission = emission;
    sf.clearcoat = R(m.clearcoat);
    sf.clearcoatRoughness = R(m.clearcoatRoughness);
    sf.sheenColor = f3(m.sheenColor);
    sf.sheenRoughness = R(m.sheenRoughness);
    sf.thinWalled = m.thinWalled;
    sf.absorption = m.attDist > 0.0f ? (-vlog(vmax(f3(m.attColor), R(1e-4)))) / R(m.attDist) : V{R(0), R(0), R(0)};
    return sf;
  }

  struct Guide {
    V albedo, normal;
    R depth, coverage;
    bool done;
    V position;  // primary hit (trace.frag:131-132)
    R reuse;
  };

  // cameraRay (:53-62).
  void cameraRay(Vec2<R> fragCoord, V& ro, V& rd) {
    const V2 j = rand2();
    const Vec2<R> uv = {(fragCoord.x + j.x) / R(W) * R(2) - R(1), (fragCoord.y + j.y) / R(H) * R(2) - R(1)};
    const R aspect = R(W) / R(H);
    const R th = R(cam->tan_half_fov);
    const V F = f3(cam->forward), Rt = f3(cam->right), U = f3(cam->up), P = f3(cam->pos);
    const V dir = normalize(F + Rt * (uv.x * aspect * th) + U * (uv.y * th));
    const V focus = P + dir * (R(cam->focus_dist) / dot(dir, F));
    const V2 dk = concentricDisk(rand2());
    const V2 lens = {dk.x * R(cam->aperture), dk.y * R(cam->aperture)};
    ro = P + Rt * lens.x + U * lens.y;
    rd = normalize(focus - ro);
  }

  // tracePath (:136-272).
  V tracePath(V ro, V rd, Guide& guide) {
    V radiance = {R(0), R(0), R(0)};
    V throughput = {R(1), R(1), R(1)};
    bool specularBounce = true;
    R bsdfPdf = R(0);
    V guideTint = {R(1), R(1), R(1)};
    guide = {{R(1), R(1), R(1)}, -rd, R(1e4), R(0), false, {R(0), R(0), R(0)}, R(1)};
    auto U = [this]() { return rand(); };
    for (int bounce = 0; bounce <= (int)maxBounces; bounce++) {
      Hit hit;
      if (!traceScene(ro, rd, hit)) {
        const V env = bounce == 0 && s->env_background == 0 ? f3(s->backdrop) : environment(rd, specularBounce, bsdfPdf);
        radiance = radiance + clampContribution(throughput * env, bounce);
        if (!guide.done) {
          guide.albedo = guideTint;
          guide.normal = -rd;
          guide.done = true;
        }
        break;
      }
      if (bounce == 0) {
        guide.depth = hit.t;
        guide.coverage = R(1);
        guide.position = hit.position;
      }
      const V wo = -rd;
      V emission;
      const Surface sf = surfaceAt(hit, wo, emission);
      const V ng = hit.geomNormal;
      if (!hit.frontFace && !sf.thinWalled && sf.transmission > R(0))
        throughput = throughput * vexp(-sf.absorption * hit.t);
      if (emission.x > R(0) || emission.y > R(0) || emission.z > R(0)) {
        R w = R(1);
        if (!specularBounce && hit.light >= 0) {
          const R pl = lightPdf(hit.light, ro, rd, hit.t) / R(s->light_count);
          w = misWeight(bsdfPdf, pl);
        }
        radiance = radiance + clampContribution(throughput * emission * w, bounce);
        if (!guide.done) {
          guide.albedo = guideTint;
          guide.normal = sf.n;
          guide.done = true;
        }
        if (hit.light >= 0) break;
      }
      const bool glass = sf.transmission > R(0) && rand() < sf.transmission;
      if (bounce == 0) {  // :187-193
        const R sharp = R(1) - smoothstep(R(0.1), R(0.7), sf.roughness);
        R glossy = std::max(sharp * mixr<R>(R(0.5), R(1), sf.metallic), sf.transmission);
        glossy = std::max(glossy, sf.clearcoat * R(0.5) * (R(1) - smoothstep(R(0.08), R(0.5), sf.clearcoatRoughness)));
        guide.reuse = R(1) - glossy;
      }
      const bool mirror = !glass && sf.metallic > R(0.9) && sf.roughness < R(0.1);
      if (!guide.done && !((glass || mirror) && bounce < 3)) {
        guide.albedo = guideTint * sf.albedo;
        guide.normal = sf.n;
        guide.done = true;
      }
      if (glass) {
        V wi, weight;
        bool reflected;
        if (!sampleDielectric(sf, hit.frontFace, ng, wo, wi, weight, reflected, U)) break;
        throughput = throughput * weight;
        if (!guide.done) guideTint = guideTint * weight;
        ro = offsetRay(hit.position, reflected ? ng : -ng);
        rd = wi;
        specularBounce = true;
      } else {
        if (!guide.done) guideTint = guideTint * sf.albedo;
        const V shadowOrigin = offsetRay(hit.position, ng);
        const V n = sf.n;
        if (s->sun_enabled != 0) {
          const V wi = sampleSunDirection(rand2());
          const R NdotL = dot(n, wi);
          if (NdotL > R(0) && dot(ng, wi) > R(0) && !occluded(shadowOrigin, wi, C::INF)) {
            R pb;
            const V f = evalOpaque(sf, wo, wi, pb);
            const R w = misWeight(R(s->sun_pdf), pb);
            radiance = radiance + clampContribution(throughput * f * NdotL * f3(s->sun_radiance) * (w / R(s->sun_pdf)), bounce);
          }
        }
        if (s->env_sampling != 0) {
          const LightSample ls = sampleEnvironment();
          const R NdotL = dot(n, ls.dir);
          if (ls.pdf > R(0) && NdotL > R(0) && dot(ng, ls.dir) > R(0) && !occluded(shadowOrigin, ls.dir, C::INF)) {
            R pb;
            const V f = evalOpaque(sf, wo, ls.dir, pb);
            const R w = misWeight(ls.pdf, pb);
            radiance = radiance + clampContribution(throughput * f * NdotL * ls.radiance * (w / ls.pdf), bounce);
          }
        }
        if (s->light_count > 0) {
          const int li = std::min((int)(rand() * R(s->light_count)), (int)s->light_count - 1);
          const LightSample ls = sampleLight(li, hit.position, rand2());
          const R NdotL = dot(n, ls.dir);
          if (ls.pdf > R(0) && NdotL > R(0) && dot(ng, ls.dir) > R(0) &&
              !occluded(shadowOrigin, ls.dir, ls.dist * (R(1) - R(1e-4)))) {
            const R pl = ls.pdf / R(s->light_count);
            R pb;
            const V f = evalOpaque(sf, wo, ls.dir, pb);
            const R w = misWeight(pl, pb);
            radiance = radiance + clampContribution(throughput * f * NdotL * ls.radiance * (w / pl), bounce);
          }
        }
        const BSDFSample bs = sampleOpaque(sf, wo, U);
        if (bs.pdf <= R(0) || dot(bs.dir, ng) <= R(0)) break;
        throughput = throughput * bs.weight;
        bsdfPdf = bs.pdf;
        specularBounce = false;
        ro = shadowOrigin;
        rd = bs.dir;
      }
      if (bounce >= 2) {  // :265-269
        const R p = std::min(R(0.95), max3(throughput));
        if (rand() >= p) break;
        throughput = throughput / p;
      }
    }
    return radiance;
  }

  // tracePath with sampling detached from evaluation: every sampling
  // decision, direction, pdf, MIS weight, Russian-roulette probability and
  // firefly-clamp scale comes from s (the primal parameters); every BSDF value
  // and emitted environment radiance comes from mev / eev. At mev = s's
  // materials and eev = s's map this returns tracePath's radiance; its
  // derivative in mev / eev is what path replay backpropagation computes.
  R clampScale(V c, int bounce) const {
    if (bounce == 0 || uClamp <= R(0)) return R(1);
    const R l = luminance(c);
    return l > uClamp ? uClamp / l : R(1);
  }
  V tracePathDetached(V ro, V rd) {
    V radiance = {R(0), R(0), R(0)};
    V thr = {R(1), R(1), R(1)};  // sampling (primal) throughput
    V tev = {R(1), R(1), R(1)};  // evaluated throughput
    bool specularBounce = true;
    R bsdfPdf = R(0);
    auto U = [this]() { return rand(); };
    const float* mats = mev ? mev : s->materials;
    for (int bounce = 0; bounce <= (int)maxBounces; bounce++) {
      Hit hit;
      if (!traceScene(ro, rd, hit)) {
        const bool backdrop = bounce == 0 && s->env_background == 0;
        const V env0 = backdrop ? f3(s->backdrop) : environment(rd, specularBounce, bsdfPdf);
        const V enve = backdrop ? f3(s->backdrop) : environmentEv(rd, specularBounce, bsdfPdf);
        radiance = radiance + tev * enve * clampScale(thr * env0, bounce);
        break;
      }
      const V wo = -rd;
      V emission, emission_e;
      const Surface sf = surfaceAt(hit, wo, emission);
      const Surface se = surfaceAtFrom(mats, hit, wo, emission_e);
      const V ng = hit.geomNormal;
      if (!hit.frontFace && !sf.thinWalled && sf.transmission > R(0)) {
        thr = thr * vexp(-sf.absorption * hit.t);
        tev = tev * vexp(-se.absorption * hit.t);
      }
      if (emission.x > R(0) || emission.y > R(0) || emission.z > R(0)) {
        R w = R(1);
        if (!specularBounce && hit.light >= 0) {
          const R pl = lightPdf(hit.light, ro, rd, hit.t) / R(s->light_count);
          w = misWeight(bsdfPdf, pl);
        }
        radiance = radiance + tev * emission * w * clampScale(thr * emission * w, bounce);
        if (hit.light >= 0) break;
      }
      const bool glass = sf.transmission > R(0) && rand() < sf.transmission;
      if (glass) {
        V wi, weight;
        bool reflected;
        if (!sampleDielectric(sf, hit.frontFace, ng, wo, wi, weight, reflected, U)) break;
        thr = thr * weight;
        tev = reflected ? tev : tev * se.albedo;
        ro = offsetRay(hit.position, reflected ? ng : -ng);
        rd = wi;
        specularBounce = true;
      } else {
        const V shadowOrigin = offsetRay(hit.position, ng);
        const V n = sf.n;
        if (s->sun_enabled != 0) {
          const V wi = sampleSunDirection(rand2());
          const R NdotL = dot(n, wi);
          if (NdotL > R(0) && dot(ng, wi) > R(0) && !occluded(shadowOrigin, wi, C::INF)) {
            R pb, pe;
            const V f = evalOpaque(sf, wo, wi, pb);
            const V fe = evalOpaque(se, wo, wi, pe);
            const R w = misWeight(R(s->sun_pdf), pb);
            const V le = f3(s->sun_radiance) * (NdotL * w / R(s->sun_pdf));
            radiance = radiance + tev * fe * le * clampScale(thr * f * le, bounce);
          }
        }
        if (s->env_sampling != 0) {
          const LightSample ls = sampleEnvironment();
          const R NdotL = dot(n, ls.dir);
          if (ls.pdf > R(0) && NdotL > R(0) && dot(ng, ls.dir) > R(0) && !occluded(shadowOrigin, ls.dir, C::INF)) {
            R pb, pe;
            const V f = evalOpaque(sf, wo, ls.dir, pb);
            const V fe = evalOpaque(se, wo, ls.dir, pe);
            const R w = misWeight(ls.pdf, pb);
            const R k = NdotL * w / ls.pdf;
            const V le = envTexEv(ls.uv) * R(s->env_intensity);
            radiance = radiance + tev * fe * le * k * clampScale(thr * f * ls.radiance * k, bounce);
          }
        }
        if (s->light_count > 0) {
          const int li = std::min((int)(rand() * R(s->light_count)), (int)s->light_count - 1);
          const LightSample ls = sampleLight(li, hit.position, rand2());
          const R NdotL = dot(n, ls.dir);
          if (ls.pdf > R(0) && NdotL > R(0) && dot(ng, ls.dir) > R(0) &&
              !occluded(shadowOrigin, ls.dir, ls.dist * (R(1) - R(1e-4)))) {
            const R pl = ls.pdf / R(s->light_count);
            R pb, pe;
            const V f = evalOpaque(sf, wo, ls.dir, pb);
            const V fe = evalOpaque(se, wo, ls.dir, pe);
            const R w = misWeight(pl, pb);
            const V le = ls.radiance * (NdotL * w / pl);
            radiance = radiance + tev * fe * le * clampScale(thr * f * le, bounce);
          }
        }
        const BSDFSample bs = sampleOpaque(sf, wo, U);
        if (bs.pdf <= R(0) || dot(bs.dir, ng) <= R(0)) break;
        R pe;
        const V fe = evalOpaque(se, wo, bs.dir, pe);
        thr = thr * bs.weight;
        tev = tev * fe * (dot(n, bs.dir) / bs.pdf);
        bsdfPdf = bs.pdf;
        specularBounce = false;
        ro = shadowOrigin;
        rd = bs.dir;
      }
      if (bounce >= 2) {
        const R p = std::min(R(0.95), max3(thr));
        if (rand() >= p) break;
        thr = thr / p;
        tev = tev / p;
      }
    }
    return radiance;
  }
};

}  // namespace

extern "C" {

}  // extern "C"

// reprojectHistory + projectToPrevious (trace.frag:274-322): the previous
// view's averages where this sample's primary surface (or sky direction) was
// seen, bilinear over the taps that saw the same surface; false if none.
template <class R>
static bool reproject_history(const orc_history* h, const typename Tracer<R>::Guide& g, Vec3<R> rd, R out_c[4],
                              R out_a[4], R out_n[4], R& n) {
  using V = Vec3<R>;
  auto f3 = [](const float* p) { return V{R(p[0]), R(p[1]), R(p[2])}; };
  for (int c = 0; c < 4; c++) out_c[c] = out_a[c] = out_n[c] = R(0);
  n = R(0);
  const bool surface = g.coverage > R(0.5);
  const V d = surface ? g.position - f3(h->cam->pos) : rd;
  const R z = dot(d, f3(h->cam->forward));
  if (z <= R(1e-6)) return false;
  const R pw = R(h->w), ph = R(h->h), aspect = pw / ph, th = R(h->cam->tan_half_fov);
  const R px = (dot(d, f3(h->cam->right)) / (z * th * aspect) * R(0.5) + R(0.5)) * pw;
  const R py = (dot(d, f3(h->cam->up)) / (z * th) * R(0.5) + R(0.5)) * ph;
  if (!(px >= R(0) && py >= R(0) && px < pw && py < ph)) return false;
  const R expected = length(d);
  const R fx = px - R(0.5), fy = py - R(0.5);
  const int bx = (int)std::floor(fx), by = (int)std::floor(fy);
  const R tx = fx - std::floor(fx), ty = fy - std::floor(fy);
  R wsum = R(0);
  for (int i = 0; i < 4; i++) {
    const int ox = i & 1, oy = i >> 1, qx = bx + ox, qy = by + oy;
    if (qx < 0 || qy < 0 || qx >= (int)h->w || qy >= (int)h->h) continue;
    const size_t q = (size_t)qy * h->w + qx;
    const float* a = h->albedo4 + q * 4;
    const float* nq = h->normal4 + q * 4;
    const V nn = normalize(V{R(nq[0]) + R(1e-6), R(nq[1]) + R(1e-6), R(nq[2]) + R(1e-6)});
    const bool same = surface ? R(a[3]) > R(0.5) && std::fabs(R(nq[3]) - expected) < R(0.02) * expected &&
                                    dot(nn, g.normal) > R(0.85)
                              : R(a[3]) < R(0.5);
    if (!same) continue;
    const R w = (ox == 1 ? tx : R(1) - tx) * (oy == 1 ? ty : R(1) - ty);
    for (int c = 0; c < 4; c++) {
      out_c[c] += R(h->color4[q * 4 + c]) * w;
      out_a[c] += R(a[c]) * w;
      out_n[c] += R(nq[c]) * w;
    }
    n += R(h->history[q]) * w;
    wsum += w;
  }
  if (wsum < R(1e-3)) return false;
  for (int c = 0; c < 4; c++) {
    out_c[c] /= wsum;
    out_a[c] /= wsum;
    out_n[c] /= wsum;
  }
  n = std::min(n / wsum, R(8) * g.reuse);  // uHistoryCap = HISTORY_CAP (renderer.ts:139, 250)
  return true;
}

extern "C" {

static int render_impl(const orc_scene* s, const orc_camera* cam, uint32_t max_bounces, float clamp_lum,
                       uint32_t width, uint32_t height, uint32_t x0, uint32_t y0, uint32_t cw, uint32_t ch,
                       uint32_t seed0, uint32_t samples, int precision, float* color4, float* albedo4,
                       float* normal4, float* history, int threads, uint64_t* work_out, bool detailed,
                       const orc_history* hist = nullptr) {
  // One counter set per par_for chunk (chunks start at multiples of 16), so
  // no two threads ever share one.
  std::vector<WorkCounts> counts(work_out ? (size_t)cw * ch / 16 + 2 : 1);
  if (x0 + cw > width || y0 + ch > height) return 1;
  std::memset(color4, 0, (size_t)cw * ch * 16);
  std::memset(albedo4, 0, (size_t)cw * ch * 16);
  std::memset(normal4, 0, (size_t)cw * ch * 16);
  std::memset(history, 0, (size_t)cw * ch * 4);
  auto run = [&](auto tag) {
    using R = decltype(tag);
    par_for((uint64_t)cw * ch, threads, [&](uint64_t b, uint64_t e) {
      Tracer<R> tr{s, cam, width, height, max_bounces, R(clamp_lum)};
      if (work_out) tr.wc = &counts[b / 16];
      tr.detailed = detailed;
      for (uint64_t q = b; q < e; q++) {
        const uint32_t px = x0 + (uint32_t)(q % cw), py = y0 + (uint32_t)(q / cw);
        const uint32_t pixelIndex = px + py * width;
        float* col = color4 + q * 4;
        float* alb = albedo4 + q * 4;
        float* nrm = normal4 + q * 4;
        for (uint32_t k = 0; k < samples; k++) {  // trace.frag:324-354, one draw per sample
          const uint32_t seed = seed0 + k;
          tr.g_seed = pixelIndex * 1973u + seed * 9277u + 26699u;
          pcg(tr.g_seed);
          Vec3<R> ro, rd;
          tr.cameraRay({R(px) + R(0.5), R(py) + R(0.5)}, ro, rd);
          typename Tracer<R>::Guide guide;
          Vec3<R> color = tr.tracePath(ro, rd, guide);
          if (std::isnan(color.x) || std::isnan(color.y) || std::isnan(color.z) || std::isinf(color.x) ||
              std::isinf(color.y) || std::isinf(color.z))
            color = {R(0), R(0), R(0)};
          const R lum = luminance(color);
          if (k == 0 && hist) {  // the first sample after a camera move starts from the reprojected history
            R pc[4], pa[4], pn[4], n0;
            reproject_history<R>(hist, guide, rd, pc, pa, pn, n0);  // zeros and 0 samples when disoccluded
            for (int c = 0; c < 4; c++) col[c] = (float)pc[c], alb[c] = (float)pa[c], nrm[c] = (float)pn[c];
            history[q] = (float)n0;
          }
          const float n = history[q];
          const R kk = R(1) / (R(n) + R(1));
          const R nc[4] = {color.x, color.y, color.z, lum * lum};
          const R na[4] = {guide.albedo.x, guide.albedo.y, guide.albedo.z, guide.coverage};
          const R nn[4] = {guide.normal.x, guide.normal.y, guide.normal.z, guide.depth};
          for (int c = 0; c < 4; c++) {
            col[c] = (float)mixr<R>(R(col[c]), nc[c], kk);
            const float a = (float)mixr<R>(R(alb[c]), na[c], kk);
            const float nv = (float)mixr<R>(R(nrm[c]), nn[c], kk);
            alb[c] = precision == 32 ? half_round(a) : a;
            nrm[c] = precision == 32 ? half_round(nv) : nv;
          }
          history[q] = n + 1.0f;
        }
      }
    });
  };
  if (precision == 64)
    run(double(0));
  else
    run(float(0));
  if (work_out) {
    for (int k = 0; k < 6; k++) work_out[k] = 0;
    for (const WorkCounts& w : counts) {
      work_out[0] += w.closest_rays, work_out[1] += w.closest_inner, work_out[2] += w.closest_tris;
      work_out[3] += w.shadow_rays, work_out[4] += w.shadow_nodes, work_out[5] += w.shadow_tris;
    }
  }
  return 0;
}

// The triangle part of traceScene and occluded as the oracle decides it,
// ray by ray: closest_tri (intersectBVH's binary64 order over slots with the
// alpha test, bvh.ts:265-320, scene.glsl:176-189) for closest rays, any_tri for
// shadow rays (t_max per ray in rays6's 7th float when stride is 7). Rays are
// binary32 (origin xyz, direction xyz); keys are the alpha-blend hash keys.
// Outputs: slot (-1 miss, -2 stack overflow) and binary64 t for closest rays;
// 1/0 occluded for shadow rays.
int orc_closest_slots(const orc_scene* s, const float* rays6, const uint32_t* keys, uint64_t n, double t_min,
                      double t_max, int32_t* slot_out, double* t_out, int threads) {
  par_for(n, threads, [&](uint64_t b, uint64_t e) {
    for (uint64_t i = b; i < e; i++) {
      const float* r = rays6 + i * 6;
      TriHit h{-1, 0, 0, 0};
      const bool ok = closest_tri(s, {(double)r[0], (double)r[1], (double)r[2]}, {(double)r[3], (double)r[4], (double)r[5]},
                                  t_min, t_max, keys ? keys[i] : 0u, h);
      slot_out[i] = ok ? h.slot : -2;
      if (t_out) t_out[i] = h.slot >= 0 ? h.t : INFINITY;
    }
  });
  return 0;
}

int orc_any_slots(const orc_scene* s, const float* rays7, const uint32_t* keys, uint64_t n, double t_min,
                  uint8_t* occluded_out, int threads) {
  par_for(n, threads, [&](uint64_t b, uint64_t e) {
    for (uint64_t i = b; i < e; i++) {
      const float* r = rays7 + i * 7;
      occluded_out[i] = any_tri(s, {(double)r[0], (double)r[1], (double)r[2]}, {(double)r[3], (double)r[4], (double)r[5]},
                                t_min, (double)r[6], keys ? keys[i] : 0u) ? 1 : 0;
    }
  });
  return 0;
}

int orc_render(const orc_scene* s, const orc_camera* cam, uint32_t max_bounces, float clamp_lum, uint32_t width,
               uint32_t height, uint32_t x0, uint32_t y0, uint32_t cw, uint32_t ch, uint32_t seed0,
               uint32_t samples, int precision, float* color4, float* albedo4, float* normal4, float* history,
               int threads) {
  return render_impl(s, cam, max_bounces, clamp_lum, width, height, x0, y0, cw, ch, seed0, samples, precision,
                     color4, albedo4, normal4, history, threads, nullptr, false);
}

int orc_render_reproject(const orc_scene* s, const orc_camera* cam, const orc_history* hist, uint32_t max_bounces,
                         float clamp_lum, uint32_t width, uint32_t height, uint32_t x0, uint32_t y0, uint32_t cw,
                         uint32_t ch, uint32_t seed0, uint32_t samples, int precision, float* color4, float* albedo4,
                         float* normal4, float* history, int threads) {
  return render_impl(s, cam, max_bounces, clamp_lum, width, height, x0, y0, cw, ch, seed0, samples, precision,
                     color4, albedo4, normal4, history, threads, nullptr, false, hist);
}

int orc_render_work(const orc_scene* s, const orc_camera* cam, uint32_t max_bounces, float clamp_lum,
                    uint32_t width, uint32_t height, uint32_t x0, uint32_t y0, uint32_t cw, uint32_t ch,
                    uint32_t seed0, uint32_t samples, float* color4, float* albedo4, float* normal4,
                    float* history, int threads, int detailed, uint64_t* work_out) {
  return render_impl(s, cam, max_bounces, clamp_lum, width, height, x0, y0, cw, ch, seed0, samples, 32, color4,
                     albedo4, normal4, history, threads, work_out, detailed != 0);
}

// sum over pixels and channels of dl4[px].rgb * (mean of the samples' detached
// radiance), in binary64 with a fixed reduction order (finite-difference
// reference for the adjoint). NaN/inf samples count as 0, like the
// accumulation.
double orc_detached_dot(const orc_scene* s, const orc_camera* cam, uint32_t max_bounces, float clamp_lum,
                        uint32_t width, uint32_t height, uint32_t seed0, uint32_t samples, const float* materials_eval,
                        const float* env_eval, const float* dl4, int threads) {
  const uint64_t npx = (uint64_t)width * height;
  const uint64_t chunk = 64;
  std::vector<double> part((npx + chunk - 1) / chunk, 0.0);
  par_for((npx + chunk - 1) / chunk, threads, [&](uint64_t b, uint64_t e) {
    Tracer<double> tr{s, cam, width, height, max_bounces, double(clamp_lum)};
    tr.mev = materials_eval;
    tr.eev = env_eval;
    for (uint64_t ci = b; ci < e; ci++) {
      double acc = 0.0;
      for (uint64_t q = ci * chunk; q < std::min(npx, (ci + 1) * chunk); q++) {
        const uint32_t px = (uint32_t)(q % width), py = (uint32_t)(q / width);
        const uint32_t pixelIndex = px + py * width;
        double sum[3] = {0, 0, 0};
        for (uint32_t k = 0; k < samples; k++) {
          tr.g_seed = pixelIndex * 1973u + (seed0 + k) * 9277u + 26699u;
          pcg(tr.g_seed);
          Vec3<double> ro, rd;
          tr.cameraRay({double(px) + 0.5, double(py) + 0.5}, ro, rd);
          const Vec3<double> c = tr.tracePathDetached(ro, rd);
          if (std::isnan(c.x) || std::isnan(c.y) || std::isnan(c.z) || std::isinf(c.x) || std::isinf(c.y) ||
              std::isinf(c.z))
            continue;
          sum[0] += c.x, sum[1] += c.y, sum[2] += c.z;
        }
        const float* d = dl4 + q * 4;
        acc += (d[0] * sum[0] + d[1] * sum[1] + d[2] * sum[2]) / samples;
      }
      part[ci] = acc;
    }
  });
  double total = 0.0;
  for (double v : part) total += v;
  return total;
}

// ---------------------------------------------------------------------------
// Denoiser: variance.frag :15-55, atrous.frag :77-137, denoise.glsl :10-25;
// driven as runDenoiser (renderer.ts:788-830). Binary32 like the GLSL.
// Buffers are W x H, row 0 = bottom; color4/out4 RGBA, albedo4/normal4 RGBA.
// ---------------------------------------------------------------------------
static inline float lumf(float r, float g, float b) { return r * 0.2126f + g * 0.7152f + b * 0.0722f; }

static inline void unit_normal(const float* n, float* o) {  // denoise.glsl:21-24
  const float l = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
  if (l > 1e-6f) {
    o[0] = n[0] / l, o[1] = n[1] / l, o[2] = n[2] / l;
  } else {
    o[0] = 0.f, o[1] = 0.f, o[2] = 1.f;
  }
}

int orc_denoise(const float* color4, const float* albedo4, const float* normal4, const float* history, uint32_t w,
                uint32_t h, const orc_camera* cam, uint32_t levels, float sigma_l, float sigma_n, float sigma_p,
                float* out4) {
  const int W = (int)w, H = (int)h;
  std::vector<float> a((size_t)W * H * 4), b((size_t)W * H * 4);
  auto inside = [&](int x, int y) { return x >= 0 && y >= 0 && x < W && y < H; };
  // variance.frag
  for (int y = 0; y < H; y++)
    for (int x = 0; x < W; x++) {
      const size_t p = (size_t)y * W + x;
      const float* c = color4 + 4 * p;
      const float* al = albedo4 + 4 * p;
      float* o = a.data() + 4 * p;
      if (al[3] < 0.5f) {
        o[0] = c[0], o[1] = c[1], o[2] = c[2], o[3] = 0.f;
        continue;
      }
      const float illum[3] = {c[0] / std::max(al[0], 1e-3f), c[1] / std::max(al[1], 1e-3f), c[2] / std::max(al[2], 1e-3f)};
      const float samples = std::max(history[p], 1.0f);
      const float la = std::max(lumf(al[0], al[1], al[2]), 1e-3f);
      float variance;
      if (samples >= 4.0f) {
        const float l = lumf(c[0], c[1], c[2]);
        variance = std::max(0.0f, c[3] - l * l) / (la * la) / samples;
      } else {
        const float* np = normal4 + 4 * p;
        float n[3];
        unit_normal(np, n);
        float s1 = 0, s2 = 0, ws = 0;
        for (int dy = -3; dy <= 3; dy++)
          for (int dx = -3; dx <= 3; dx++) {
            const int qx = x + dx, qy = y + dy;
            if (!inside(qx, qy)) continue;
            const size_t q = (size_t)qy * W + qx;
            const float* aq = albedo4 + 4 * q;
            if (aq[3] < 0.5f) continue;
            const float* nq = normal4 + 4 * q;
            float un[3];
            unit_normal(nq, un);
            const float cosn = std::max(0.0f, n[0] * un[0] + n[1] * un[1] + n[2] * un[2]);
            const float stepv = (0.1f * np[3] < std::fabs(np[3] - nq[3])) ? 0.0f : 1.0f;  // step(|dz|, 0.1 z)
            const float wgt = std::pow(cosn, 32.0f) * stepv;
            const float* cq = color4 + 4 * q;
            const float l = lumf(cq[0] / std::max(aq[0], 1e-3f), cq[1] / std::max(aq[1], 1e-3f), cq[2] / std::max(aq[2], 1e-3f));
            s1 += wgt * l;
            s2 += wgt * l * l;
            ws += wgt;
          }
        const float m1 = s1 / std::max(ws, 1e-6f);
        variance = std::max(0.0f, s2 / std::max(ws, 1e-6f) - m1 * m1) / samples;
      }
      o[0] = illum[0], o[1] = illum[1], o[2] = illum[2], o[3] = variance;
    }
  // atrous.frag, steps 1, 2, 4, 8, 16 (renderer.ts:140)
  const float F[3] = {cam->forward[0], cam->forward[1], cam->forward[2]};
  const float Rt[3] = {cam->right[0], cam->right[1], cam->right[2]};
  const float U[3] = {cam->up[0], cam->up[1], cam->up[2]};
  const float CP[3] = {cam->pos[0], cam->pos[1], cam->pos[2]};
  const float th = cam->tan_half_fov;
  auto primary_dir = [&](int x, int y, float* d) {  // atrous.frag:77-81
    const float ux = ((float)x + 0.5f) / (float)W * 2.0f - 1.0f, uy = ((float)y + 0.5f) / (float)H * 2.0f - 1.0f;
    const float aspect = (float)W / (float)H;
    float v[3];
    for (int k = 0; k < 3; k++) v[k] = F[k] + Rt[k] * (ux * aspect * th) + U[k] * (uy * th);
    const float l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int k = 0; k < 3; k++) d[k] = v[k] / l;
  };
  const float hk[3] = {0.375f, 0.25f, 0.0625f};
  float* in = a.data();
  float* outb = b.data();
  for (uint32_t lv = 0; lv < levels; lv++) {
    const int stepv = 1 << lv;
    for (int y = 0; y < H; y++)
      for (int x = 0; x < W; x++) {
        const size_t p = (size_t)y * W + x;
        const float* cp = in + 4 * p;
        float* o = outb + 4 * p;
        if (albedo4[4 * p + 3] < 0.5f) {
          o[0] = cp[0], o[1] = cp[1], o[2] = cp[2], o[3] = cp[3];
          continue;
        }
        const float* np = normal4 + 4 * p;
        float n[3], dp[3], P[3];
        unit_normal(np, n);
        primary_dir(x, y, dp);
        for (int k = 0; k < 3; k++) P[k] = CP[k] + dp[k] * np[3];
        const float footprint = 2.0f * th * np[3] / (float)H;
        float var = 0, wv = 0;
        for (int dy = -1; dy <= 1; dy++)
          for (int dx = -1; dx <= 1; dx++) {
            const int qx = x + dx, qy = y + dy;
            if (!inside(qx, qy)) continue;
            const float k = (dx == 0 ? 0.5f : 0.25f) * (dy == 0 ? 0.5f : 0.25f);
            var += in[4 * ((size_t)qy * W + qx) + 3] * k;
            wv += k;
          }
        const float denom = sigma_l * std::sqrt(std::max(var / wv, 0.0f)) + 1e-6f;
        const float lp = lumf(cp[0], cp[1], cp[2]);
        float sum[3] = {cp[0] * (hk[0] * hk[0]), cp[1] * (hk[0] * hk[0]), cp[2] * (hk[0] * hk[0])};
        float sumVar = cp[3] * (hk[0] * hk[0]) * (hk[0] * hk[0]);
        float wsum = hk[0] * hk[0];
        for (int dy = -2; dy <= 2; dy++)
          for (int dx = -2; dx <= 2; dx++) {
            if (dx == 0 && dy == 0) continue;
            const int qx = x + dx * stepv, qy = y + dy * stepv;
            if (!inside(qx, qy)) continue;
            const size_t q = (size_t)qy * W + qx;
            if (albedo4[4 * q + 3] < 0.5f) continue;
            const float* cq = in + 4 * q;
            const float* nq = normal4 + 4 * q;
            const float k = hk[std::abs(dx)] * hk[std::abs(dy)];
            float un[3], dq[3], Q[3];
            unit_normal(nq, un);
            const float wn = std::pow(std::max(0.0f, n[0] * un[0] + n[1] * un[1] + n[2] * un[2]), sigma_n);
            primary_dir(qx, qy, dq);
            for (int c = 0; c < 3; c++) Q[c] = CP[c] + dq[c] * nq[3];
            const float reach = sigma_p * footprint * (float)stepv * std::sqrt((float)(dx * dx + dy * dy));
            const float pd = n[0] * (Q[0] - P[0]) + n[1] * (Q[1] - P[1]) + n[2] * (Q[2] - P[2]);
            const float wp = std::exp(-std::fabs(pd) / (reach + 1e-6f));
            const float wl = std::exp(-std::fabs(lp - lumf(cq[0], cq[1], cq[2])) / denom);
            const float wgt = k * wn * wp * wl;
            for (int c = 0; c < 3; c++) sum[c] += cq[c] * wgt;
            sumVar += cq[3] * wgt * wgt;
            wsum += wgt;
          }
        o[0] = sum[0] / wsum, o[1] = sum[1] / wsum, o[2] = sum[2] / wsum, o[3] = sumVar / (wsum * wsum);
      }
    std::swap(in, outb);
  }
  std::memcpy(out4, in, (size_t)W * H * 16);
  return 0;
}

// display.frag :42-67 with uRenderSize == uViewSize. out_rgb: the value
// written to the RGBA8 target before quantization (dither included).
// display.frag:42-67: the traced region (rw x rh, at the start of the
// targets) shown in a vw x vh view; Catmull-Rom upsampling (:47-60) when the
// sizes differ. `radiance` is display.frag:33-40 (coordinates clamped to the
// region, denoised blend).
int orc_display_view(const float* color4, const float* albedo4, const float* denoised4, uint32_t rw, uint32_t rh,
                     uint32_t vw, uint32_t vh, float denoise_weight, float exposure, int tonemap, float* out_rgb) {
  auto radiance = [&](int px, int py, float* c) {
    px = std::min(std::max(px, 0), (int)rw - 1);
    py = std::min(std::max(py, 0), (int)rh - 1);
    const size_t p = (size_t)py * rw + px;
    for (int k = 0; k < 3; k++) c[k] = color4[4 * p + k];
    if (denoise_weight > 0.0f) {
      const float* a = albedo4 + 4 * p;
      if (a[3] >= 0.5f)
        for (int k = 0; k < 3; k++) {
          const float dn = denoised4[4 * p + k] * std::max(a[k], 1e-3f);
          c[k] = c[k] * (1.0f - denoise_weight) + dn * denoise_weight;
        }
    }
  };
  const bool same = rw == vw && rh == vh;
  const float sx = (float)rw / (float)vw, sy = (float)rh / (float)vh;  // uRenderSize / uViewSize
  for (uint32_t y = 0; y < vh; y++)
    for (uint32_t x = 0; x < vw; x++) {
      const float fx = (float)x + 0.5f, fy = (float)y + 0.5f;  // gl_FragCoord.xy
      float c[3];
      if (same) {
        radiance((int)x, (int)y, c);
      } else {
        const float srx = fx * sx - 0.5f, sry = fy * sy - 0.5f;
        const int ix = (int)std::floor(srx), iy = (int)std::floor(sry);
        const float f[2] = {srx - std::floor(srx), sry - std::floor(sry)};
        float w[4][2];
        for (int a = 0; a < 2; a++) {
          const float t = f[a];
          w[0][a] = t * (-0.5f + t * (1.0f - 0.5f * t));
          w[1][a] = 1.0f + t * t * (-2.5f + 1.5f * t);
          w[2][a] = t * (0.5f + t * (2.0f - 1.5f * t));
          w[3][a] = t * t * (-0.5f + 0.5f * t);
        }
        c[0] = c[1] = c[2] = 0.0f;
        for (int yy = 0; yy < 4; yy++)
          for (int xx = 0; xx < 4; xx++) {
            float r[3];
            radiance(ix + xx - 1, iy + yy - 1, r);
            const float wt = w[xx][0] * w[yy][1];
            for (int k = 0; k < 3; k++) c[k] += r[k] * wt;
          }
        for (int k = 0; k < 3; k++) c[k] = std::max(c[k], 0.0f);
      }
      const float t = 0.06711056f * fx + 0.00583715f * fy;
      const float u = 52.9829189f * (t - std::floor(t));
      const float ign = u - std::floor(u);
      const size_t p = (size_t)y * vw + x;
      for (int k = 0; k < 3; k++) {
        float v = c[k] * exposure;
        if (tonemap == 0)
          v = std::min(std::max((v * (2.51f * v + 0.03f)) / (v * (2.43f * v + 0.59f) + 0.14f), 0.0f), 1.0f);
        else if (tonemap == 1)
          v = v / (1.0f + v);
        v = std::min(std::max(v, 0.0f), 1.0f);
        const float lo = v * 12.92f, hi = 1.055f * std::pow(v, 1.0f / 2.4f) - 0.055f;
        v = v < 0.0031308f ? lo : hi;  // mix(lo, hi, step(0.0031308, c))
        out_rgb[3 * p + k] = v + (ign - 0.5f) / 255.0f;
      }
    }
  return 0;
}

int orc_display(const float* color4, const float* albedo4, const float* denoised4, uint32_t w, uint32_t h,
                float denoise_weight, float exposure, int tonemap, float* out_rgb) {
  return orc_display_view(color4, albedo4, denoised4, w, h, w, h, denoise_weight, exposure, tonemap, out_rgb);
}

// BSDF tuples. in: 32 floats per tuple
//   0-2 albedo, 3 metallic, 4 roughness, 5 ior, 6 clearcoat, 7 clearcoatRoughness,
//   8-10 sheenColor, 11 sheenRoughness, 12 thinWalled, 13-15 n, 16-18 nc,
//   19-21 wo, 22-24 wi, 25-30 six uniforms, 31 frontFace (ng = n)
// out: 24 doubles per tuple
//   0-2 evalOpaque f, 3 pdf, 4-6 sampleOpaque dir, 7-9 weight, 10 pdf,
//   11 sampleDielectric ok, 12-14 wi, 15-17 weight, 18 reflected.
// The sheen LUT comes from `lut` (16x16, half-rounded) supplied in in-tuple
// order via orc_bsdf_set_lut.
static float g_lut[256];

void orc_bsdf_set_lut(const float* lut) { std::memcpy(g_lut, lut, sizeof g_lut); }

int orc_bsdf_tuples(const float* in, uint64_t n, int precision, double* out, int threads) {
  orc_scene sc{};
  sc.sheen_lut = g_lut;
  auto run = [&](auto tag) {
    using R = decltype(tag);
    using T = Tracer<R>;
    par_for(n, threads, [&](uint64_t b, uint64_t e) {
      T tr{&sc, nullptr, 1, 1, 0, R(0)};
      for (uint64_t i = b; i < e; i++) {
        const float* t = in + i * 32;
        typename T::Surface sf;
        sf.albedo = {R(t[0]), R(t[1]), R(t[2])};
        sf.metallic = R(t[3]);
        sf.roughness = R(t[4]);
        sf.ior = R(t[5]);
        sf.transmission = R(0);
        sf.clearcoat = R(t[6]);
        sf.clearcoatRoughness = R(t[7]);
        sf.sheenColor = {R(t[8]), R(t[9]), R(t[10])};
        sf.sheenRoughness = R(t[11]);
        sf.thinWalled = t[12] > 0.5f;
        sf.n = {R(t[13]), R(t[14]), R(t[15])};
        sf.nc = {R(t[16]), R(t[17]), R(t[18])};
        sf.emission = {R(0), R(0), R(0)};
        sf.absorption = {R(0), R(0), R(0)};
        const Vec3<R> wo = {R(t[19]), R(t[20]), R(t[21])}, wi = {R(t[22]), R(t[23]), R(t[24])};
        double* o = out + i * 24;
        R pdf;
        const Vec3<R> f = tr.evalOpaque(sf, wo, wi, pdf);
        o[0] = f.x, o[1] = f.y, o[2] = f.z, o[3] = pdf;
        int k = 0;
        auto U = [&]() { return R(t[25 + (k++ % 6)]); };
        const auto bs = tr.sampleOpaque(sf, wo, U);
        o[4] = bs.dir.x, o[5] = bs.dir.y, o[6] = bs.dir.z;
        o[7] = bs.weight.x, o[8] = bs.weight.y, o[9] = bs.weight.z, o[10] = bs.pdf;
        k = 0;
        Vec3<R> dwi = {R(0), R(0), R(0)}, dw = {R(0), R(0), R(0)};
        bool refl = false;
        const bool ok = tr.sampleDielectric(sf, t[31] > 0.5f, sf.n, wo, dwi, dw, refl, U);
        o[11] = ok, o[12] = dwi.x, o[13] = dwi.y, o[14] = dwi.z;
        o[15] = dw.x, o[16] = dw.y, o[17] = dw.z, o[18] = refl;
        for (int q = 19; q < 24; q++) o[q] = 0;
      }
    });
  };
  if (precision == 64)
    run(double(0));
  else
    run(float(0));
  return 0;
}

}  // extern "C"

// ------------------------------------------------------------------ texture arrays
// buildTextureArrays (renderer.ts:314-333) as the product defines its
// resampling: box mip chain (2x2 averages, edges clamped, each level stored as
// 8-bit codes), level of detail log2(max(w, h) / size) in binary64, bilinear
// taps with edge clamping at ((x + 0.5) / size, (y + 0.5) / size), sRGB
// decoded before filtering and encoded by the code-value midpoints.
namespace {

struct TexLevel {
  std::vector<uint8_t> texels;
  int w, h;
};

float tex_decode(uint8_t v, int ch, bool srgb) {
  const TexelTables& T = texel_tables();
  return (srgb && ch < 3) ? T.srgb[v] : T.unorm[v];
}

uint8_t tex_encode(float c, int ch, bool srgb) {
  if (!(c > 0.f)) return 0;
  if (srgb && ch < 3) {
    const float* mid = texel_tables().mid;  // number of midpoints <= c (increasing table)
    return (uint8_t)(std::upper_bound(mid, mid + 255, c) - mid);
  }
  const float v = c * 255.f + 0.5f;
  return v >= 255.f ? 255 : (uint8_t)v;
}

float tex_fetch(const TexLevel& L, int x, int y, int ch, bool srgb) {
  x = x < 0 ? 0 : (x >= L.w ? L.w - 1 : x);
  y = y < 0 ? 0 : (y >= L.h ? L.h - 1 : y);
  return tex_decode(L.texels[((size_t)y * L.w + x) * 4 + ch], ch, srgb);
}

float tex_bilinear(const TexLevel& L, float u, float v, int ch, bool srgb) {
  const float x = u * (float)L.w - 0.5f, y = v * (float)L.h - 0.5f;
  const float x0 = std::floor(x), y0 = std::floor(y);
  const float fx = x - x0, fy = y - y0;
  const int ix = (int)x0, iy = (int)y0;
  const float a = tex_fetch(L, ix, iy, ch, srgb), b = tex_fetch(L, ix + 1, iy, ch, srgb);
  const float c = tex_fetch(L, ix, iy + 1, ch, srgb), d = tex_fetch(L, ix + 1, iy + 1, ch, srgb);
  const float top = a * (1.f - fx) + b * fx, bottom = c * (1.f - fx) + d * fx;
  return top * (1.f - fy) + bottom * fy;
}

}  // namespace

extern "C" {

uint32_t orc_texture_size(const uint32_t* w, const uint32_t* h, uint32_t n) {
  if (n == 0) return 0;
  uint32_t largest = 1;
  for (uint32_t i = 0; i < n; i++) largest = std::max(largest, std::max(w[i], h[i]));
  uint32_t size = 1;
  while (size < largest) size <<= 1;
  size = std::min<uint32_t>(size, 2048);
  while (size > 256 && (uint64_t)n * size * size * 4 > (256ull << 20)) size /= 2;
  return size;
}

int orc_resample_layer(const uint8_t* rgba, uint32_t w, uint32_t h, uint32_t size, int srgb, uint8_t* out) {
  if (!rgba || !out || !w || !h || !size) return 1;
  const bool sr = srgb != 0;
  const double rho = (double)std::max(w, h) / size;
  const double lambda = rho > 1.0 ? std::log2(rho) : 0.0;
  const int d1 = (int)std::floor(lambda);
  std::vector<TexLevel> L(1);
  L[0].texels.assign(rgba, rgba + (size_t)w * h * 4);
  L[0].w = (int)w;
  L[0].h = (int)h;
  for (int k = 1; k <= d1 + 1; k++) {
    const TexLevel& src = L[k - 1];
    if (src.w == 1 && src.h == 1) break;
    TexLevel dst;
    dst.w = src.w > 1 ? src.w / 2 : 1;
    dst.h = src.h > 1 ? src.h / 2 : 1;
    dst.texels.resize((size_t)dst.w * dst.h * 4);
    for (int y = 0; y < dst.h; y++)
      for (int x = 0; x < dst.w; x++)
        for (int ch = 0; ch < 4; ch++) {
          const float s4 = tex_fetch(src, 2 * x, 2 * y, ch, sr) + tex_fetch(src, 2 * x + 1, 2 * y, ch, sr) +
                           tex_fetch(src, 2 * x, 2 * y + 1, ch, sr) + tex_fetch(src, 2 * x + 1, 2 * y + 1, ch, sr);
          dst.texels[((size_t)y * dst.w + x) * 4 + ch] = tex_encode(s4 * 0.25f, ch, sr);
        }
    L.push_back(std::move(dst));
  }
  const int nlev = (int)L.size();
  const int a = std::min(d1, nlev - 1), b = std::min(a + 1, nlev - 1);
  const float blend = b > a ? (float)(lambda - d1) : 0.f;
  for (uint32_t i = 0; i < size * size; i++) {
    const float u = ((float)(i % size) + 0.5f) / (float)size, v = ((float)(i / size) + 0.5f) / (float)size;
    for (int ch = 0; ch < 4; ch++) {
      float c = tex_bilinear(L[a], u, v, ch, sr);
      if (blend > 0.f) c = c * (1.f - blend) + tex_bilinear(L[b], u, v, ch, sr) * blend;
      out[(size_t)i * 4 + ch] = tex_encode(c, ch, sr);
    }
  }
  return 0;
}

}  // extern "C"
