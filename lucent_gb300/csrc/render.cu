// Wavefront path tracer: the reference's trace.frag (src/shaders/trace.frag)
// restructured as kernels over queues of paths.
//
// One batch holds S samples of every pixel (path p = s * W * H + pixel). Each
// path keeps the reference's per-pixel PCG stream (trace.frag:326-328, seed =
// pixel * 1973 + sampleSeed * 9277 + 26699) and draws its numbers in the
// reference's order, so a path makes the reference's choices. Per bounce:
//   closest  -> triangle hit per active path (traverse.cuh, hit ids equal to
//               the reference's CPU intersector with tMin = EPS, tMax = INF)
//   shade    -> spheres / ground, surface, emission + MIS, dielectric or
//               opaque: next-event estimation (sun, environment, one light)
//               into per-path shadow slots, BSDF sample, Russian roulette
//   any-hit  -> shadow rays
//   resolve  -> unoccluded NEE added in the reference's order (sun, env, light):
//               at the start of the next shade, or in the accumulation for a
//               path that ends (the backward replays keep a resolve kernel)
// Accumulation replays the running mean (trace.frag:350-354) sample by
// sample per pixel, so a batch equals S sequential draws.
#include <cuda_fp16.h>

#include "internal.h"
#include "render_internal.h"
#include "shade.cuh"
#include "traverse.cuh"
#include "traverse_wide.cuh"

namespace lucent {

using namespace sh;

// ------------------------------------------------------------ traversal policies
// Policies for waves holding the paths of several scenes: a path's scene is
// sid[path]; its BVH, triangles and materials come from the scene table.

// Closest-hit rays of a wave, read in order from a ray stream: ray k of the
// bounce's queue (origin + path id, direction + scene), written by the
// camera or shade kernel at the path's queue position (`nray`), or by the
// ray sort in sorted order (`sray`). The hit of ray k is written to hits[k]:
// the shade kernel walks the same queue and reads it at the same position.
struct PathClosestMulti {
  const uint32_t* cnt;
  const float4* rays;  // 2 float4 per ray: origin + path id, direction + scene
  PathField ro;  // path records: the RNG state is origin.w
  float4* hits;
  const SceneRec* recs;
  int any_alpha;
  static constexpr bool kMultiScene = true;
  static constexpr int kThreads = 256, kMinBlocks = 3;  // closest-hit block shape
  // Lanes of a wide-kernel warp that wait before it fetches new rays: a refill
  // stalls the warp on the atomic and the new rays' loads (path tracing's
  // short rays: 24 measured best of 1, 4, 8, 16, 24, 32).
  static constexpr int kRefillMin = 24;
  __device__ uint32_t count() const { return *cnt; }
  __device__ uint32_t path(uint32_t k) const { return __float_as_uint(rays[2 * (size_t)k].w); }
  __device__ void ray(uint32_t k, float3& o, float3& d) const {
    const float4 a = rays[2 * (size_t)k], b = rays[2 * (size_t)k + 1];
    o = make_float3(a.x, a.y, a.z);
    d = make_float3(b.x, b.y, b.z);
  }
  __device__ BvhView bvh(uint32_t k) const { return scene_bvh(__float_as_int(rays[2 * (size_t)k + 1].w)); }
  __device__ BvhView scene_bvh(int sc) const {
    const SceneDev& S = recs[sc].scene;
    return {S.nodes, S.geo, S.node_count, sc, S.wide};
  }
  __device__ uint32_t key(uint32_t k) const { return __float_as_uint(ro[path(k)].w); }
  __device__ bool alpha_any() const { return any_alpha != 0; }
  __device__ bool alpha(int sc, int slot, uint32_t key, float bu, float bv) const {
    return alpha_opaque(recs[sc].scene, slot, key, bu, bv);
  }
  __device__ AlphaAnswer alpha_fast(int sc, int slot, uint32_t key) const {
    return sh::alpha_fast(recs[sc].scene, slot, key);
  }
  // The triangle only: the shade kernel computes t, u, v (hit_values).
  __device__ void finish(uint32_t k, int slot) const { hits[k] = make_float4(0.f, 0.f, 0.f, __int_as_float(slot)); }
  __device__ void hit(uint32_t k, int slot, double t, double u, double v) const {
    hits[k] = make_float4(__double2float_rn(t), __double2float_rn(u), __double2float_rn(v), __int_as_float(slot));
  }
  __device__ void miss(uint32_t k) const { hits[k] = make_float4(INF, 0.f, 0.f, __int_as_float(-1)); }
  __device__ void fail(uint32_t k) const { miss(k); }
};

struct PathShadowMulti {
  const uint32_t* cnt;
  const uint32_t* queue;
  const float4* so;
  const float4* sd;
  float4* sh_c;  // per shadow slot: contribution, w = 1 until the ray is found occluded
  const SceneRec* recs;
  const uint16_t* sid;
  int any_alpha;
  static constexpr bool kMultiScene = true;
  __device__ uint32_t count() const { return *cnt; }
  __device__ void ray(uint32_t k, float3& o, float3& d) const {  // rays are stored in queue order
    const float4 a = so[k], b = sd[k];
    o = make_float3(a.x, a.y, a.z);
    d = make_float3(b.x, b.y, b.z);
  }
  __device__ BvhView bvh(uint32_t k) const { return scene_bvh(__ldg(sid + queue[k] / 3)); }  // slot 3 * path + j
  __device__ BvhView scene_bvh(int sc) const {
    const SceneDev& S = recs[sc].scene;
    return {S.nodes, S.geo, S.node_count, sc, S.wide};
  }
  __device__ float tmax32(uint32_t k) const { return so[k].w; }
  __device__ uint32_t key(uint32_t k) const { return __float_as_uint(sd[k].w); }
  __device__ bool alpha_any() const { return any_alpha != 0; }
  __device__ bool alpha(int sc, int slot, uint32_t key, float bu, float bv) const {
    return alpha_opaque(recs[sc].scene, slot, key, bu, bv);
  }
  __device__ AlphaAnswer alpha_fast(int sc, int slot, uint32_t key) const {
    return sh::alpha_fast(recs[sc].scene, slot, key);
  }
  __device__ void shadow(uint32_t k, bool occluded) const {
    if (occluded) sh_c[queue[k]].w = 0.f;
  }
};

// ------------------------------------------------------------ kernels
// Path flags (guide tint .w). Bits kPendShift.. mark the path's next-event
// slots (sun, environment, light) whose shadow rays the last shade emitted:
// the contributions that resolve (the next shade, or the accumulation)
// still has to add.
constexpr unsigned kSpecular = 1u, kGuideDone = 2u;
constexpr int kPendShift = 2;

// cameraRay (trace.frag:53-62) and the path's initial state; sample s of
// pixel `pixel` draws from the stream seeded with (pixel, seed0 + s). Path p
// takes position k of the first queue.
__device__ __forceinline__ void camera_path(const Paths& P, uint32_t p, uint32_t k, uint32_t pixel, uint32_t s,
                                            const CameraDev& cam, int W, int H, uint32_t seed0, int scene) {
  const uint32_t x = pixel % W, y = pixel / W;
  uint32_t st = pixel * 1973u + (seed0 + s) * 9277u + 26699u;  // trace.frag:327-328
  pcg(st);
  const float j0 = rnd(st), j1 = rnd(st);
  const float ux = ((float)x + 0.5f + j0) / (float)W * 2.f - 1.f;
  const float uy = ((float)y + 0.5f + j1) / (float)H * 2.f - 1.f;
  const float aspect = (float)W / (float)H;
  const float3 dir = norm3(cam.forward + cam.right * (ux * aspect * cam.tan_half_fov) + cam.up * (uy * cam.tan_half_fov));
  const float3 focus = cam.pos + dir * (cam.focus / dot3(dir, cam.forward));
  const float l0 = rnd(st), l1 = rnd(st);
  const float2 lens = concentric_disk(l0, l1);
  const float3 ro = cam.pos + cam.right * (lens.x * cam.aperture) + cam.up * (lens.y * cam.aperture);
  const float3 rd = norm3(focus - ro);
  // The rest of the record starts as constants that the bounce-0 shade
  // takes without reading them (first_record_field).
  P.ro[p] = make_float4(ro.x, ro.y, ro.z, __uint_as_float(st));
  P.rd[p] = make_float4(rd.x, rd.y, rd.z, 0.f);
  P.q[0][k] = p;
  P.nray[2 * (size_t)k] = make_float4(ro.x, ro.y, ro.z, __uint_as_float(p));
  P.nray[2 * (size_t)k + 1] = make_float4(rd.x, rd.y, rd.z, __int_as_float(scene));
}

// A path record field as the bounce-0 shade starts from it: throughput 1
// (no BSDF pdf yet), no radiance, guide tint 1 with the specular flag, guide
// albedo 1, guide normal -rd at depth 1e4; later bounces read the record.
__device__ __forceinline__ float4 first_record_field(int f, float3 rd) {
  switch (f) {
    case 2: return make_float4(1.f, 1.f, 1.f, 0.f);                                  // throughput + pdf
    case 3: return make_float4(1.f, 1.f, 1.f, __uint_as_float(kSpecular));           // tint + flags
    case 4: return make_float4(1.f, 1.f, 1.f, 0.f);                                  // guide albedo
    case 5: return make_float4(-rd.x, -rd.y, -rd.z, 1e4f);                           // guide normal + depth
    default: return make_float4(0.f, 0.f, 0.f, 0.f);                                 // radiance
  }
}

// Index of the scene whose range [base[i], base[i + 1]) holds v (n scenes).
__device__ __forceinline__ int find_scene(const uint32_t* __restrict__ base, int n, uint32_t v) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(base + mid) <= v) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Several scenes in one wave: scene i owns paths [path_base[i], path_base[i + 1]).
// Path base + s * W * H + pixel is sample s of the pixel; the first queue
// holds a scene's paths pixel-major (position base + pixel * S + s), so a
// warp's primary rays are the samples of one or two pixels: nearly the same
// ray, the same nodes, the same triangles. Paths are independent, so the
// queue order changes no result.
__global__ void k_camera_multi(Paths P, const SceneRec* __restrict__ recs, const uint32_t* __restrict__ path_base,
                               int n, uint16_t* __restrict__ sid, int S) {
  const uint32_t total = __ldg(path_base + n);
  // One thread per path, in path order: the 128-byte path records are written
  // coalesced; the queue entry and the 32-byte ray go to the path's queue
  // position.
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < total; p += gridDim.x * blockDim.x) {
    const int sc = find_scene(path_base, n, p);
    const SceneRec& R = recs[sc];
    const uint32_t base = __ldg(path_base + sc), WH = (uint32_t)R.W * R.H, local = p - base;
    const uint32_t pixel = local % WH, s = local / WH, k = base + pixel * (uint32_t)S + s;
    camera_path(P, p, k, pixel, s, R.cam, R.W, R.H, R.seed0, sc);
    sid[p] = (uint16_t)sc;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) P.ctr[kCtrQ0] = total;
}

__device__ __forceinline__ float3 clamp_c(float3 c, int bounce, float uclamp) {  // trace.frag:65-69
  if (bounce == 0 || uclamp <= 0.f) return c;
  const float l = lum(c);
  return l > uclamp ? c * (uclamp / l) : c;
}

// Shadow ray j of path p: its slot s = 3p + j holds the contribution and a
// flag (w) that the any-hit kernels clear when the ray is occluded, read by
// resolve per path (the path's flags say which slots are pending); the ray
// itself (origin + tmax, direction + alpha key) is stored at its position in
// the shadow queue, so the any-hit kernel reads the rays in order.
__device__ __forceinline__ void emit_shadow(const Paths& P, uint32_t p, int j, float3 o, float3 d, float tmax,
                                            uint32_t key, float3 c) {
  const uint32_t s = 3 * p + j;
  P.sh_c[s] = make_float4(c.x, c.y, c.z, 1.f);
  const uint32_t pos = atomicAdd(&P.ctr[kCtrShadow], 1u);
  P.sh_o[pos] = make_float4(o.x, o.y, o.z, tmax);
  P.sh_d[pos] = make_float4(d.x, d.y, d.z, __uint_as_float(key));
  P.qs[pos] = s;
}

__device__ __forceinline__ bool analytic_occluded(const SceneDev& S, float3 ro, float3 rd, float tmax) {
  for (int i = 0; i < S.sphere_count; i++)  // scene.glsl:337-340
    if (hit_sphere(ro, rd, __ldg(&S.spheres[i]), tmax) < tmax) return true;
  return hit_ground(S, ro, rd, tmax) < tmax;
}

// Path-replay adjoint state (used by the ADJ instantiation of k_shade_t).
// Gradients are of sum_pixels dl[pixel] . (mean radiance of the replayed
// samples) with respect to each material's base colour (3), roughness,
// metallic and clearcoat (dmat, 6 floats per material) and to the
// environment texels (denv, RGB + one pad float per texel, 16-byte aligned, so
// that a tap is one vector atomic). Sampling (directions,
// pdfs, MIS weights, lobe and Russian-roulette choices, the firefly clamp's
// scale) is held fixed, as in path replay backpropagation.
struct AdjointDev {
  const float4* dl;  // per pixel: dL/dI (rgb) / samples
  float4* lrem;      // per path: radiance still to come (primal total minus what is accounted for)
  float4* gcont;     // per path, 5 float4: dl_c * df_c/dtheta_p / f_c at the BSDF-sampled direction (18), material
  float4* gslot;     // per shadow slot, 2 float4: dl . c * df/f for its light direction (6), material
  float4* genv;      // per path: environment sample uv and scale (rgb) of its env shadow slot
  float* dmat;
  float* denv;       // nullptr: no environment gradient
  uint32_t WH;
  int primal;        // 1: the primal replay (paths only, no adjoint work)
};

// Adds g[0..5] to dmat[mat * 6 ..], one atomic per distinct material per warp.
__device__ __forceinline__ void add_material_grad(float* dmat, int mat, const float g[6]) {
  const unsigned act = __activemask();
  const unsigned peers = __match_any_sync(act, mat);
  const int leader = __ffs(peers) - 1;
  const int lane = threadIdx.x & 31;
  float sum[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  for (unsigned b = peers; b; b &= b - 1) {
    const int src = __ffs(b) - 1;
#pragma unroll
    for (int k = 0; k < 6; k++) sum[k] += __shfl_sync(peers, g[k], src);
  }
  if (lane == leader && mat >= 0)
#pragma unroll
    for (int k = 0; k < 6; k++)
      if (sum[k] != 0.f) atomicAdd(dmat + (size_t)mat * 6 + k, sum[k]);
}

// Environment texel gradient: sv_c * bilinear weight into each of 4 texels,
// one float4 atomic per tap (the texels' RGB gradients are float4s).
__device__ __forceinline__ void add_env_grad(const AdjointDev& A, const LightingDev& L, float2 uv, float3 dl, float3 sv) {
  int idx[4];
  float wt[4];
  bilinear_taps(L.env_w, L.env_h, uv.x, uv.y, true, idx, wt);
  const float g[3] = {dl.x * sv.x, dl.y * sv.y, dl.z * sv.z};
  float4* const d4 = reinterpret_cast<float4*>(A.denv);
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const float4 v = make_float4(g[0] * wt[k], g[1] * wt[k], g[2] * wt[k], 0.f);
    if (v.x != 0.f || v.y != 0.f || v.z != 0.f) atomicAdd(d4 + idx[k], v);
  }
}

// The clamp_c scale factor (1 when unclamped).
__device__ __forceinline__ float clamp_scale(float3 c, int bounce, float uclamp) {
  if (bounce == 0 || uclamp <= 0.f) return 1.f;
  const float l = lum(c);
  return l > uclamp ? uclamp / l : 1.f;
}

// dl . (c (.) df_p / f) for p = 0..5 (zero where f is zero).
__device__ __forceinline__ void contract_grad(float3 dl, float3 c, float3 f, const float3 df[6], float g[6]) {
  const float w[3] = {f.x != 0.f ? dl.x * c.x / f.x : 0.f, f.y != 0.f ? dl.y * c.y / f.y : 0.f,
                      f.z != 0.f ? dl.z * c.z / f.z : 0.f};
#pragma unroll
  for (int k = 0; k < 6; k++) g[k] = w[0] * df[k].x + w[1] * df[k].y + w[2] * df[k].z;
}

// Gradient of one next-event contribution c (light direction wi) with respect
// to the vertex's material, stored in its shadow slot until occlusion is known.
__device__ __forceinline__ void nee_grad(const AdjointDev& A, const LightingDev& L, const Surface& s, float3 wo,
                                         float3 wi, float3 dl, float3 c, int material, uint32_t slot) {
  float3 df[6];
  const float3 fg = eval_opaque_grad(L, s, wo, wi, df);
  float g[6];
  contract_grad(dl, c, fg, df, g);
  A.gslot[2 * (size_t)slot] = make_float4(g[0], g[1], g[2], g[3]);
  A.gslot[2 * (size_t)slot + 1] = make_float4(g[4], g[5], __int_as_float(material), 0.f);
}

// Where the shade kernel finds a path's scene, lighting and settings: a
// per-path scene index into a table of SceneRec.
struct SceneTable {
  const SceneRec* recs;
  const uint16_t* sid;
  __device__ int index(uint32_t p) const { return __ldg(sid + p); }
  __device__ const SceneRec& rec(uint32_t p) const { return recs[index(p)]; }
  __device__ const SceneDev& scene(uint32_t p) const { return rec(p).scene; }
  __device__ const LightingDev& light(uint32_t p) const { return rec(p).light; }
  __device__ int bounces(uint32_t p) const { return rec(p).max_bounces; }
  __device__ float uclamp(uint32_t p) const { return rec(p).clamp; }
};

// The texture-map part of surfaceAt (trace.frag:72-110): multipliers of the
// base colour, roughness, metallic and emission, and the normal-mapped
// shading normal. Only the TEX instantiation of the shade kernel contains
// it. `slot`: the triangle, -1 for the ground plane, -2 for a sphere.
struct MapSample {
  float3 albedo, emission, n;
  float roughness, metallic;
  bool mapped;
};
static __device__ __forceinline__ MapSample sample_maps(const SceneDev& S, const float4* M, float4 maps, int slot,
                                                        float4 hit, float3 pos, float3 rd, float3 normal, float3 gn,
                                                        bool front) {
  MapSample out{f3(1.f, 1.f, 1.f), f3(1.f, 1.f, 1.f), normal, 1.f, 1.f, false};
  // hit.uv and the surface derivatives (scene.glsl:274-320)
  float2 huv = make_float2(0.f, 0.f);
  float3 dpdu = f3(0.f, 0.f, 0.f), dpdv = f3(0.f, 0.f, 0.f);
  if (slot == -1) {
    huv = make_float2(pos.x, pos.z);
  } else if (slot >= 0) {
    const float4 h = hit;
    const float4* a = S.attr + 4 * (size_t)slot;
    const float4* g = S.geo + 3 * (size_t)slot;
    const float4 a3 = __ldg(a + 3), p0 = __ldg(g), p1 = __ldg(g + 1), p2 = __ldg(g + 2);
    const float2 uv0 = make_float2(__ldg(&a[0].w), a3.x), uv1 = make_float2(__ldg(&a[1].w), a3.y),
                 uv2 = make_float2(__ldg(&a[2].w), a3.z);
    const float hw = 1.f - h.y - h.z;
    huv = make_float2(uv0.x * hw + uv1.x * h.y + uv2.x * h.z, uv0.y * hw + uv1.y * h.y + uv2.y * h.z);
    const float2 d1 = make_float2(uv1.x - uv0.x, uv1.y - uv0.y), d2 = make_float2(uv2.x - uv0.x, uv2.y - uv0.y);
    const float det = d1.x * d2.y - d1.y * d2.x;
    if (fabsf(det) > 1e-12f) {
      const float r = 1.f / det;
      const float3 e1 = f3(p1) - f3(p0), e2 = f3(p2) - f3(p0);
      dpdu = (e1 * d2.y - e2 * d1.y) * r;
      dpdv = (e2 * d1.x - e1 * d2.x) * r;
    }
  }
  const float2 tuv = transform_uv(huv, __ldg(M + 8), __ldg(M + 9));
  if (maps.x >= 0.f) out.albedo = f3(sample_layer(S, S.color_maps, (int)maps.x, tuv, true));
  if (maps.y >= 0.f) {
    const float4 mr = sample_layer(S, S.data_maps, (int)maps.y, tuv, false);
    out.roughness = mr.y;
    out.metallic = mr.z;
  }
  if (maps.w >= 0.f) out.emission = f3(sample_layer(S, S.color_maps, (int)maps.w, tuv, true));
  if (maps.z >= 0.f && dot3(dpdu, dpdu) > 0.f) {
    // Tangent frame from the UV derivatives on the outward normal, so back
    // faces see the mirrored perturbation; glTF's +Y points to decreasing v.
    const float3 N = front ? normal : -normal;
    const float3 T = norm3(dpdu - N * dot3(N, dpdu));
    float3 B = cross3(N, T);
    if (dot3(B, -dpdv) < 0.f) B = -B;
    const float4 t4 = sample_layer(S, S.data_maps, (int)maps.z, tuv, false);
    const float scale = __ldg(&M[5].x);
    const float tx = (t4.x * 2.f - 1.f) * scale, ty = (t4.y * 2.f - 1.f) * scale, tz = t4.z * 2.f - 1.f;
    float3 mapped = norm3(T * tx + B * ty + N * fmaxf(tz, 1e-3f));
    mapped = front ? mapped : -mapped;
    if (dot3(mapped, -rd) > 1e-3f && dot3(mapped, gn) > 0.f) {
      out.n = mapped;
      out.mapped = true;
    }
  }
  return out;
}

// The t, u, v the renderer shades with: the binary32 estimates of the
// triangle's binary32 test at c = tMax (mt_classify; every triangle accepted
// in binary32 has them), like the GLSL's own hitTriangle, else the binary64
// values rounded. A function of the ray and the triangle alone, whatever
// decisions the traversal took; computed one path per thread.
static __device__ __forceinline__ float4 hit_values(const float4* __restrict__ geo, float3 ro, float3 rd, int slot) {
  const float4 a = __ldg(geo + 3 * (size_t)slot), b = __ldg(geo + 3 * (size_t)slot + 1),
               c = __ldg(geo + 3 * (size_t)slot + 2);
  const Ray32 r = make_ray32(ro, rd);
  float tl, th;
  float3 est;
  // tMin = 1e-6 and tMax = 1e30 (binary64) rounded down and up to binary32.
  const float tmin_lo = __int_as_float(0x358637bd), tmin_hi = __int_as_float(0x358637be);
  const float cmax_lo = __int_as_float(0x7149f2c9), cmax_hi = __int_as_float(0x7149f2ca);
  if (mt_classify(r, a, b, c, tmin_lo, tmin_hi, cmax_lo, cmax_hi, tl, th, est) == kTriAccept)
    return make_float4(est.x, est.y, est.z, __int_as_float(slot));
  const Tri64 h = tri_f64(ro, rd, a, b, c, 1e-6, __longlong_as_double(0x7ff0000000000000ll));
  return make_float4(__double2float_rn(h.t), __double2float_rn(h.u), __double2float_rn(h.v), __int_as_float(slot));
}

// One bounce of every path in queue `cur`. Hits on texture-mapped materials
// are shaded by a second instantiation, TEX: the first appends them to the
// textured-hit queue untouched, so untextured shading carries none of the
// texture code; the TEX launch then shades exactly those paths. Which
// instantiation shades a hit depends on the hit alone, never on the launch,
// so a scene renders the same alone and in a batch. Four blocks of 128 per
// SM: 128 registers a thread, no spills (measured faster than five blocks
// at 96 registers with spills, and than six).
template <class Src, bool ADJ = false, bool TEX = false>
__global__ void __launch_bounds__(128, 4) k_shade_t(Paths P, const __grid_constant__ Src src, int cur, int bounce,
                                                    const __grid_constant__ AdjointDev A = AdjointDev{}) {
  const uint32_t n = TEX ? P.ctr[kCtrTex] : P.ctr[kCtrQ0 + cur];
  const uint32_t* q = P.q[cur];
  uint32_t* qn = P.q[cur ^ 1];
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const uint32_t kq = TEX ? P.qtex[k] : k;  // position in queue `cur`, which also indexes the hits
    const uint32_t p = q[kq];
    const SceneDev& S = src.scene(p);
    const LightingDev& L = src.light(p);
    const int max_bounces = src.bounces(p);
    const float uclamp = src.uclamp(p);
    const float4 ro4 = P.ro[p];
    float3 ro = f3(ro4), rd = f3(P.rd[p]);
    const bool first = bounce == 0;  // the camera wrote only origin and direction
    const float4 thr4 = first ? first_record_field(2, rd) : P.thr[p];
    const float4 tint4 = first ? first_record_field(3, rd) : P.tint[p];
    float3 thr = f3(thr4), rad = f3(first ? first_record_field(7, rd) : P.rad[p]), tint = f3(tint4);
    // The forward render and the backward's primal replay resolve the
    // previous bounce's next-event contributions here (the adjoint replay
    // keeps its resolve kernel, which also gathers gradients): the unoccluded
    // ones join the radiance first, in the reference's order (sun,
    // environment, light), as a separate resolve pass would add them.
    unsigned emitted = 0u;
    const unsigned flags = __float_as_uint(tint4.w);
    if (!ADJ || A.primal) {
      const unsigned pending = flags >> kPendShift & 7u;
#pragma unroll
      for (int j = 0; j < 3; j++) {
        if (!(pending >> j & 1u)) continue;
        const float4 c = P.sh_c[3 * (size_t)p + j];
        if (c.w != 0.f) rad = rad + f3(c);  // unoccluded
      }
    }
    float bsdf_pdf = thr4.w;
    bool spec = flags & kSpecular, done = flags & kGuideDone;
    float4 galb = first ? first_record_field(4, rd) : P.galb[p];
    float4 gnrm = first ? first_record_field(5, rd) : P.gnrm[p];
    uint32_t st = __float_as_uint(ro4.w);  // the path's RNG state
    float4 hv = P.hit[kq];
    if (__float_as_int(hv.w) >= 0) hv = hit_values(S.geo, ro, rd, __float_as_int(hv.w));
    bool alive = false, deferred = false;
    float3 dl = f3(0.f, 0.f, 0.f), lrem = f3(0.f, 0.f, 0.f);
    int cont_mat = -1;
    const bool adj = ADJ && !A.primal;
    if (adj) {
      const float4 l4 = A.lrem[p];
      dl = l4.w == 0.f ? f3(A.dl[p % A.WH]) : f3(0.f, 0.f, 0.f);  // w != 0: the sample was dropped (NaN)
      lrem = f3(l4);
    }

    // traceScene (scene.glsl:192-333): spheres, ground, then the triangle hit.
    float closest = INF;
    int best_sphere = -1;
    bool ground = false;
    for (int i = 0; i < S.sphere_count; i++) {
      const float t = hit_sphere(ro, rd, __ldg(&S.spheres[i]), closest);
      if (t < closest) {
        closest = t;
        best_sphere = i;
      }
    }
    const float tg = hit_ground(S, ro, rd, closest);
    if (tg < closest) {
      closest = tg;
      best_sphere = -1;
      ground = true;
    }
    const int slot = __float_as_int(hv.w);
    bool tri = false;
    if (slot >= 0 && hv.x < closest) {
      closest = hv.x;
      tri = true;
      best_sphere = -1;
      ground = false;
    }
    do {
      if (!tri && best_sphere < 0 && !ground) {  // miss (trace.frag:146-155)
        if (bounce == 0) P.gpos[p] = make_float4(0.f, 0.f, 0.f, 1.f);  // no guide position: full reuse
        const float3 env = bounce == 0 && !L.env_background ? L.backdrop : environment(L, rd, spec, bsdf_pdf);
        rad = rad + clamp_c(thr * env, bounce, uclamp);
        if (adj) {
          if (A.denv && !(bounce == 0 && !L.env_background)) {
            const float w = (!spec && L.env_sampling) ? mis(bsdf_pdf, env_pdf(L, rd)) : 1.f;
            const float k = clamp_scale(thr * env, bounce, uclamp) * w * L.env_intensity;
            add_env_grad(A, L, equirect_uv(env_to_local(L, rd)), dl, thr * k);
          }
        }
        if (!done) {
          galb = make_float4(tint.x, tint.y, tint.z, galb.w);
          gnrm = make_float4(-rd.x, -rd.y, -rd.z, gnrm.w);
          done = true;
        }
        break;
      }
      if (bounce == 0) {
        gnrm.w = closest;
        galb.w = 1.f;
      }
      // Hit record.
      const float3 pos = ro + rd * closest;
      if (bounce == 0) P.gpos[p] = make_float4(pos.x, pos.y, pos.z, 1.f);
      float3 normal, gn;
      bool front;
      int material, light = -1;
      if (ground) {
        front = rd.y < 0.f;
        normal = f3(0.f, front ? 1.f : -1.f, 0.f);
        gn = normal;
        material = S.ground_material;
      } else if (best_sphere >= 0) {
        const float4 sp = __ldg(&S.spheres[best_sphere]);
        const float3 nn = (pos - f3(sp)) / sp.w;
        front = dot3(rd, nn) < 0.f;
        normal = front ? nn : -nn;
        gn = normal;
        material = __ldg(&S.sphere_materials[best_sphere]);
        light = __ldg(&S.sphere_lights[best_sphere]);
      } else {  // scene.glsl:407-440
        const float4 g0 = __ldg(&S.geo[3 * (size_t)slot]), g1 = __ldg(&S.geo[3 * (size_t)slot + 1]),
                     g2 = __ldg(&S.geo[3 * (size_t)slot + 2]);
        const float4 a0 = __ldg(&S.attr[4 * (size_t)slot]), a1 = __ldg(&S.attr[4 * (size_t)slot + 1]),
                     a2 = __ldg(&S.attr[4 * (size_t)slot + 2]);
        const float bu = hv.y, bv = hv.z, w = 1.f - bu - bv;
        const float3 e1 = f3(g1) - f3(g0), e2 = f3(g2) - f3(g0);
        float3 ng = norm3(cross3(e1, e2));
        float3 ns = norm3(f3(a0) * w + f3(a1) * bu + f3(a2) * bv);
        front = dot3(rd, ng) < 0.f;
        if (!front) {
          ng = -ng;
          ns = -ns;
        }
        if (dot3(ns, ng) < 0.05f) ns = ng;
        normal = ns;
        gn = ng;
        material = (int)g0.w;
        light = (int)g1.w;
      }
      // surfaceAt (trace.frag:72-124).
      const float4* M = S.materials + (size_t)material * 10;
      const float4 m0 = __ldg(M), m1 = __ldg(M + 1), m2 = __ldg(M + 2), m3 = __ldg(M + 3), m5 = __ldg(M + 5),
                   m6 = __ldg(M + 6), m7 = __ldg(M + 7), m8 = __ldg(M + 8);
      Surface s;
      s.albedo = f3(m0);
      if (m1.w > 0.f) {
        const float qx = floorf(pos.x * m1.w + 0.5f), qy = floorf(pos.y * m1.w + 0.5f), qz = floorf(pos.z * m1.w + 0.5f);
        const float sum = qx + qy + qz;
        if (sum - 2.f * floorf(sum / 2.f) >= 0.5f) s.albedo = f3(m3);
      }
      s.metallic = m0.w;
      s.roughness = m1.x;
      float3 emission = f3(m2);
      s.nc = normal;
      s.n = normal;
      const float4 m4 = __ldg(M + 4);
      if (S.tex_size > 0 && fmaxf(fmaxf(m4.x, m4.y), fmaxf(m4.z, m4.w)) >= 0.f) {
        if constexpr (!TEX) {  // nothing of this path has been written yet
          deferred = true;
          break;
        } else {
          const MapSample ms =
              sample_maps(S, M, m4, ground ? -1 : (tri ? slot : -2), hv, pos, rd, normal, gn, front);
          s.albedo = s.albedo * ms.albedo;
          s.roughness *= ms.roughness;
          s.metallic *= ms.metallic;
          emission = emission * ms.emission;
          if (ms.mapped) s.n = ms.n;
        }
      }
      s.ior = m1.y;
      s.transmission = m1.z * (1.f - s.metallic);
      s.clearcoat = m5.y;
      s.clearcoat_roughness = m5.z;
      s.sheen_color = f3(m6);
      s.sheen_roughness = m6.w;
      s.thin = m8.w > 0.5f;
      if (m7.w > 0.f) {
        s.absorption = f3(-logf(fmaxf(m7.x, 1e-4f)), -logf(fmaxf(m7.y, 1e-4f)), -logf(fmaxf(m7.z, 1e-4f))) / m7.w;
      } else {
        s.absorption = f3(0.f, 0.f, 0.f);
      }
      const float3 wo = -rd;
      if (!front && !s.thin && s.transmission > 0.f)  // trace.frag:168
        thr = thr * f3(expf(-s.absorption.x * closest), expf(-s.absorption.y * closest), expf(-s.absorption.z * closest));
      if (emission.x > 0.f || emission.y > 0.f || emission.z > 0.f) {  // :170-184
        float w = 1.f;
        if (!spec && light >= 0) w = mis(bsdf_pdf, light_pdf(S, light, ro, rd, closest) / (float)S.light_count);
        rad = rad + clamp_c(thr * emission * w, bounce, uclamp);
        if (adj) lrem = lrem - clamp_c(thr * emission * w, bounce, uclamp);
        if (!done) {
          galb = make_float4(tint.x, tint.y, tint.z, galb.w);
          gnrm = make_float4(s.n.x, s.n.y, s.n.z, gnrm.w);
          done = true;
        }
        if (light >= 0) break;
      }
      const bool glass = s.transmission > 0.f && rnd(st) < s.transmission;
      if (bounce == 0) {  // trace.frag:187-193: reflections and refractions do not move with the surface
        const float sharp = 1.f - smooth(0.1f, 0.7f, s.roughness);
        float glossy = fmaxf(sharp * mixf(0.5f, 1.f, s.metallic), s.transmission);
        glossy = fmaxf(glossy, s.clearcoat * 0.5f * (1.f - smooth(0.08f, 0.5f, s.clearcoat_roughness)));
        P.gpos[p].w = 1.f - glossy;
      }
      const bool mirror = !glass && s.metallic > 0.9f && s.roughness < 0.1f;
      if (!done && !((glass || mirror) && bounce < 3)) {
        galb = make_float4(tint.x * s.albedo.x, tint.y * s.albedo.y, tint.z * s.albedo.z, galb.w);
        gnrm = make_float4(s.n.x, s.n.y, s.n.z, gnrm.w);
        done = true;
      }
      auto U = [&]() { return rnd(st); };
      if (glass) {
        float3 wi, weight;
        bool refl;
        if (!sample_dielectric(s, front, gn, wo, wi, weight, refl, U)) break;
        thr = thr * weight;
        if (adj) {
          if (!refl) {  // transmission weight = base colour: d/d albedo_c of what follows = lrem_c / albedo_c
            const float g[6] = {s.albedo.x > 0.f ? dl.x * lrem.x / s.albedo.x : 0.f,
                                s.albedo.y > 0.f ? dl.y * lrem.y / s.albedo.y : 0.f,
                                s.albedo.z > 0.f ? dl.z * lrem.z / s.albedo.z : 0.f, 0.f, 0.f, 0.f};
            add_material_grad(A.dmat, material, g);
          }
        }
        if (!done) tint = tint * weight;
        ro = offset_ray(pos, refl ? gn : -gn);
        rd = wi;
        spec = true;
      } else {
        if (!done) tint = tint * s.albedo;
        const float3 so = offset_ray(pos, gn);
        const float3 n = s.n;
        // Next-event estimation (:216-252): sun, environment, then one light,
        // each with the reference's sampling and MIS. One loop body evaluates
        // the BSDF for all three, so the kernel holds one copy of the layered
        // BSDF evaluation instead of three (instruction-cache pressure).
#pragma unroll 1
        for (int j = 0; j < 3; j++) {
          float3 wi, le;
          float pdf, tmax;
          bool ok;
          float2 env_uv = make_float2(0.f, 0.f);
          if (j == 0) {  // sun (:216-225)
            if (!L.sun_enabled) continue;
            const float u0 = rnd(st), u1 = rnd(st);
            float3 t, b;
            basis(L.sun_dir, t, b);
            wi = to_world(uniform_cone(u0, u1, L.sun_cos), t, b, L.sun_dir);
            le = L.sun_radiance;
            pdf = L.sun_pdf;
            tmax = INF;
            ok = true;
          } else if (j == 1) {  // environment (:228-237)
            if (!L.env_sampling) continue;
            const LightSample ls = sample_environment(L, st);
            wi = ls.dir;
            le = ls.radiance;
            pdf = ls.pdf;
            tmax = INF;
            ok = ls.pdf > 0.f;
            env_uv = ls.uv;
          } else {  // one light, chosen uniformly (:240-252)
            if (S.light_count <= 0) continue;
            const int li = min((int)(rnd(st) * (float)S.light_count), S.light_count - 1);
            const float u0 = rnd(st), u1 = rnd(st);
            const LightSample ls = sample_light(S, li, pos, u0, u1);
            wi = ls.dir;
            le = ls.radiance;
            pdf = ls.pdf / (float)S.light_count;
            tmax = ls.dist * (1.f - 1e-4f);
            ok = ls.pdf > 0.f;
          }
          const float NdotL = dot3(n, wi);
          if (!(ok && NdotL > 0.f && dot3(gn, wi) > 0.f && !analytic_occluded(S, so, wi, tmax))) continue;
          float pb;
          const float3 f = eval_opaque(L, s, wo, wi, pb);
          const float w = mis(pdf, pb);
          const float3 cu = thr * f * NdotL * le * (w / pdf);
          const float3 c = clamp_c(cu, bounce, uclamp);
          emit_shadow(P, p, j, so, wi, tmax, st, c);
          emitted |= 1u << j;
          if (adj) {
            nee_grad(A, L, s, wo, wi, dl, c, material, 3 * p + j);
            if (j == 1) {
              const float3 sv = thr * f * (clamp_scale(cu, bounce, uclamp) * NdotL * (w / pdf) * L.env_intensity);
              A.genv[2 * (size_t)p] = make_float4(env_uv.x, env_uv.y, sv.x, sv.y);
              A.genv[2 * (size_t)p + 1] = make_float4(sv.z, 0.f, 0.f, 0.f);
            }
          }
        }
        const BsdfSample bs = sample_opaque(L, s, wo, U);  // :255-261
        if (bs.pdf <= 0.f || dot3(bs.dir, gn) <= 0.f) break;
        if (adj) {
          float3 df[6];
          const float3 fg = eval_opaque_grad(L, s, wo, bs.dir, df);
          const float w[3] = {fg.x != 0.f ? dl.x / fg.x : 0.f, fg.y != 0.f ? dl.y / fg.y : 0.f,
                              fg.z != 0.f ? dl.z / fg.z : 0.f};
          float gc[18];
#pragma unroll
          for (int k = 0; k < 6; k++) gc[3 * k] = w[0] * df[k].x, gc[3 * k + 1] = w[1] * df[k].y, gc[3 * k + 2] = w[2] * df[k].z;
          float4* o = A.gcont + 5 * (size_t)p;
          o[0] = make_float4(gc[0], gc[1], gc[2], gc[3]);
          o[1] = make_float4(gc[4], gc[5], gc[6], gc[7]);
          o[2] = make_float4(gc[8], gc[9], gc[10], gc[11]);
          o[3] = make_float4(gc[12], gc[13], gc[14], gc[15]);
          o[4].x = gc[16];
          o[4].y = gc[17];
          cont_mat = material;
        }
        thr = thr * bs.weight;
        bsdf_pdf = bs.pdf;
        spec = false;
        ro = so;
        rd = bs.dir;
      }
      if (bounce >= 2) {  // Russian roulette (:265-269)
        const float pr = fminf(0.95f, max3(thr));
        if (rnd(st) >= pr) {
          cont_mat = -1;
          break;
        }
        thr = thr / pr;
      }
      alive = bounce < max_bounces;
      if (!alive) cont_mat = -1;
    } while (false);
    if (deferred) {
      P.qtex[atomicAdd(&P.ctr[kCtrTex], 1u)] = kq;
      continue;
    }
    if (adj) {
      A.lrem[p].x = lrem.x, A.lrem[p].y = lrem.y, A.lrem[p].z = lrem.z;
      A.gcont[5 * (size_t)p + 4].z = __int_as_float(cont_mat);
    }

    P.rad[p] = make_float4(rad.x, rad.y, rad.z, 0.f);
    // Flags always (the slots this bounce left pending, for resolve), the rest if the path goes on.
    P.tint[p] = make_float4(tint.x, tint.y, tint.z,
                            __uint_as_float((spec ? kSpecular : 0u) | (done ? kGuideDone : 0u) | emitted << kPendShift));
    P.galb[p] = galb;
    P.gnrm[p] = gnrm;
    if (alive) {
      P.ro[p] = make_float4(ro.x, ro.y, ro.z, __uint_as_float(st));
      P.rd[p] = make_float4(rd.x, rd.y, rd.z, 0.f);
      P.thr[p] = make_float4(thr.x, thr.y, thr.z, bsdf_pdf);
      const uint32_t pos = atomicAdd(&P.ctr[kCtrQ0 + (cur ^ 1)], 1u);
      qn[pos] = p;
      P.nray[2 * (size_t)pos] = make_float4(ro.x, ro.y, ro.z, __uint_as_float(p));
      P.nray[2 * (size_t)pos + 1] = make_float4(rd.x, rd.y, rd.z, __int_as_float(src.index(p)));
    }
  }
}

// Resolve for the adjoint replay: the unoccluded next-event contributions
// leave the path's remaining radiance and add their material (and
// environment) gradients; what remains is the radiance that followed the
// BSDF-sampled direction, whose gradient is lrem (.) dl (.) df/f.
__global__ void k_resolve_adjoint(Paths P, const __grid_constant__ AdjointDev A, const SceneRec* __restrict__ rec,
                                  int cur) {
  const LightingDev& L = rec->light;
  const uint32_t n = P.ctr[kCtrQ0 + cur];
  const uint32_t* q = P.q[cur];
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const uint32_t p = q[k];
    float4 r = P.rad[p];
    const float4 l4 = A.lrem[p];
    float3 lrem = f3(l4);
    const float3 dl = l4.w == 0.f ? f3(A.dl[p % A.WH]) : f3(0.f, 0.f, 0.f);
    float g[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    int mat = -1;
    const unsigned pending = __float_as_uint(P.tint[p].w) >> kPendShift & 7u;
    for (int j = 0; j < 3; j++) {
      const uint32_t s = 3 * p + j;
      if (!(pending >> j & 1u)) continue;
      const float4 c = P.sh_c[s];
      if (c.w != 0.f) {  // unoccluded
        r.x += c.x;
        r.y += c.y;
        r.z += c.z;
        lrem = lrem - f3(c);
        const float4 a = A.gslot[2 * (size_t)s], b = A.gslot[2 * (size_t)s + 1];
        g[0] += a.x, g[1] += a.y, g[2] += a.z, g[3] += a.w, g[4] += b.x, g[5] += b.y;
        mat = __float_as_int(b.z);
        if (j == 1 && A.denv) {
          const float4 e0 = A.genv[2 * (size_t)p], e1 = A.genv[2 * (size_t)p + 1];
          add_env_grad(A, L, make_float2(e0.x, e0.y), dl, f3(e0.z, e0.w, e1.x));
        }
      }
    }
    const float4* gc = A.gcont + 5 * (size_t)p;
    const int cm = __float_as_int(gc[4].z);
    if (cm >= 0) {
      mat = cm;
      const float4 a = gc[0], b = gc[1], c = gc[2], d = gc[3], e = gc[4];
      const float v[18] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x, c.y, c.z, c.w, d.x, d.y, d.z, d.w, e.x, e.y};
#pragma unroll
      for (int t = 0; t < 6; t++) g[t] += lrem.x * v[3 * t] + lrem.y * v[3 * t + 1] + lrem.z * v[3 * t + 2];
    }
    P.rad[p] = r;
    A.lrem[p] = make_float4(lrem.x, lrem.y, lrem.z, l4.w);
    add_material_grad(A.dmat, mat, g);
  }
}

// Primal radiance of each replayed sample -> the adjoint replay's remaining
// radiance (a dropped NaN/inf sample is flagged in w and contributes nothing).
// The primal replay's last shaded bounce is resolved here, as the forward
// render's accumulation resolves it.
__global__ void k_seed_lrem(Paths P, AdjointDev A, uint32_t total) {
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < total; p += gridDim.x * blockDim.x) {
    float4 c = P.rad[p];
    const unsigned pending = __float_as_uint(P.tint[p].w) >> kPendShift & 7u;
    for (int j = 0; j < 3; j++) {
      if (!(pending >> j & 1u)) continue;
      const float4 e = P.sh_c[3 * (size_t)p + j];
      if (e.w == 0.f) continue;  // occluded
      c = make_float4(c.x + e.x, c.y + e.y, c.z + e.z, c.w);
    }
    const bool bad = isnan(c.x) || isnan(c.y) || isnan(c.z) || isinf(c.x) || isinf(c.y) || isinf(c.z);
    A.lrem[p] = bad ? make_float4(0.f, 0.f, 0.f, 1.f) : make_float4(c.x, c.y, c.z, 0.f);
  }
}

__device__ __forceinline__ float4 h4f(half4 v) {
  return make_float4(__half2float(v.x), __half2float(v.y), __half2float(v.z), __half2float(v.w));
}

// reprojectHistory (trace.frag:274-322): the previous view's averages at the
// place this sample's primary surface (or sky direction) occupied there,
// bilinear over the taps that saw the same surface. False: disoccluded.
__device__ bool reproject_history(const SceneRec& R, float4 gp, float4 ga, float4 gn, float4& col, float4& alb,
                                  float4& nrm, float& n) {
  col = alb = nrm = make_float4(0.f, 0.f, 0.f, 0.f);
  n = 0.f;
  const bool surface = ga.w > 0.5f;
  const CameraDev& C = R.prev_cam;
  const float3 d = surface ? f3(gp) - C.pos : -f3(gn);  // a sky guide normal is -rd
  const float z = dot3(d, C.forward);
  if (z <= 1e-6f) return false;
  const float pw = (float)R.prev_w, ph = (float)R.prev_h;
  const float aspect = pw / ph;
  const float px = (dot3(d, C.right) / (z * C.tan_half_fov * aspect) * 0.5f + 0.5f) * pw;
  const float py = (dot3(d, C.up) / (z * C.tan_half_fov) * 0.5f + 0.5f) * ph;
  if (!(px >= 0.f && py >= 0.f && px < pw && py < ph)) return false;
  const float expected = len3(d);
  const float fx = px - 0.5f, fy = py - 0.5f;
  const int bx = (int)floorf(fx), by = (int)floorf(fy);
  const float tx = fx - floorf(fx), ty = fy - floorf(fy);
  const float3 g = f3(gn);
  float wsum = 0.f;
  for (int i = 0; i < 4; i++) {
    const int ox = i & 1, oy = i >> 1;
    const int qx = bx + ox, qy = by + oy;
    if (qx < 0 || qy < 0 || qx >= R.prev_w || qy >= R.prev_h) continue;
    const size_t q = (size_t)qy * R.prev_w + qx;
    const float4 a = h4f(R.prev.albedo[q]), nq = h4f(R.prev.normal[q]);
    const bool same = surface ? a.w > 0.5f && fabsf(nq.w - expected) < 0.02f * expected &&
                                    dot3(norm3(f3(nq) + f3(1e-6f, 1e-6f, 1e-6f)), g) > 0.85f
                              : a.w < 0.5f;
    if (!same) continue;
    const float w = (ox == 1 ? tx : 1.f - tx) * (oy == 1 ? ty : 1.f - ty);
    const float4 c = R.prev.color[q];
    col = make_float4(col.x + c.x * w, col.y + c.y * w, col.z + c.z * w, col.w + c.w * w);
    alb = make_float4(alb.x + a.x * w, alb.y + a.y * w, alb.z + a.z * w, alb.w + a.w * w);
    nrm = make_float4(nrm.x + nq.x * w, nrm.y + nq.y * w, nrm.z + nq.z * w, nrm.w + nq.w * w);
    n += R.prev.history[q] * w;
    wsum += w;
  }
  if (wsum < 1e-3f) return false;
  col = make_float4(col.x / wsum, col.y / wsum, col.z / wsum, col.w / wsum);
  alb = make_float4(alb.x / wsum, alb.y / wsum, alb.z / wsum, alb.w / wsum);
  nrm = make_float4(nrm.x / wsum, nrm.y / wsum, nrm.z / wsum, nrm.w / wsum);
  n = fminf(n / wsum, kHistoryCap * gp.w);
  return true;
}

// Running means (trace.frag:335-354) of one pixel over the batch's samples,
// in order; sample s of the pixel is path path_base + s * W * H + px. With
// R.reproject the first sample starts from the reprojected history.
__device__ __forceinline__ void accumulate_pixel(const Paths& P, const SceneRec& R, uint32_t WH, int S, uint32_t px,
                                                 uint32_t path_base) {
  const AccumDev& A = R.accum;
  float4 col, alb, nrm;
  float n;
  if (R.reproject) {
    const uint32_t p0 = path_base + px;
    if (!reproject_history(R, P.gpos[p0], P.galb[p0], P.gnrm[p0], col, alb, nrm, n)) n = 0.f;  // disoccluded
  } else {
    col = A.color[px];
    alb = h4f(A.albedo[px]);
    nrm = h4f(A.normal[px]);
    n = A.history[px];
  }
  for (int s = 0; s < S; s++) {
    const uint32_t p = path_base + (uint32_t)s * WH + px;
    float4 c = P.rad[p];
    // The contributions of the path's last shaded bounce, resolved here (the
    // forward render folds resolve into the next shade and this pass).
    const unsigned pending = __float_as_uint(P.tint[p].w) >> kPendShift & 7u;
    for (int j = 0; j < 3; j++) {
      if (!(pending >> j & 1u)) continue;
      const float4 e = P.sh_c[3 * (size_t)p + j];
      if (e.w == 0.f) continue;  // occluded
      c = make_float4(c.x + e.x, c.y + e.y, c.z + e.z, c.w);
    }
    if (isnan(c.x) || isnan(c.y) || isnan(c.z) || isinf(c.x) || isinf(c.y) || isinf(c.z)) c = make_float4(0.f, 0.f, 0.f, 0.f);
    const float l = lum(f3(c));
    const float k = 1.f / (n + 1.f);
    const float4 ga = P.galb[p], gn = P.gnrm[p];
    col = make_float4(mixf(col.x, c.x, k), mixf(col.y, c.y, k), mixf(col.z, c.z, k), mixf(col.w, l * l, k));
    // RGBA16F targets (renderer.ts:490): every store rounds to half.
    alb = make_float4(__half2float(__float2half_rn(mixf(alb.x, ga.x, k))), __half2float(__float2half_rn(mixf(alb.y, ga.y, k))),
                      __half2float(__float2half_rn(mixf(alb.z, ga.z, k))), __half2float(__float2half_rn(mixf(alb.w, ga.w, k))));
    nrm = make_float4(__half2float(__float2half_rn(mixf(nrm.x, gn.x, k))), __half2float(__float2half_rn(mixf(nrm.y, gn.y, k))),
                      __half2float(__float2half_rn(mixf(nrm.z, gn.z, k))), __half2float(__float2half_rn(mixf(nrm.w, gn.w, k))));
    n = n + 1.f;
  }
  A.color[px] = col;
  A.albedo[px] = make_half4(alb);
  A.normal[px] = make_half4(nrm);
  A.history[px] = n;
}

// Scene i owns batch pixels [pix_base[i], pix_base[i + 1]).
__global__ void k_accumulate_multi(Paths P, const SceneRec* __restrict__ recs, const uint32_t* __restrict__ pix_base,
                                   const uint32_t* __restrict__ path_base, int n, int S) {
  const uint32_t total = __ldg(pix_base + n);
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
    const int sc = find_scene(pix_base, n, g);
    const SceneRec& R = recs[sc];
    accumulate_pixel(P, R, (uint32_t)R.W * R.H, S, g - __ldg(pix_base + sc), __ldg(path_base + sc));
  }
}

// Advances every scene's sample seed by the wave's S samples (on the device,
// so a captured wave can be replayed unchanged).
__global__ void k_advance_seeds(SceneRec* recs, int n, int S) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    recs[i].seed0 += (uint32_t)S;
    recs[i].reproject = 0;  // only a view's first sample reprojects
  }
}

__global__ void k_zero_counters(uint32_t* ctr, int nxt) {
  if (threadIdx.x == 0) {
    ctr[kCtrQ0 + nxt] = 0;
    ctr[kCtrShadow] = 0;
    ctr[kCtrWork] = 0;
    ctr[kCtrSlow] = 0;
    ctr[kCtrWork2] = 0;
    ctr[kCtrSlow2] = 0;
    ctr[kCtrTex] = 0;
  }
}

// k_zero_counters in two halves, for a bounce whose predecessor's shadow rays
// run on the side stream: the closest-hit counters before the closest hit,
// the rest after the join.
__global__ void k_zero_closest_counters(uint32_t* ctr) {
  if (threadIdx.x == 0) {
    ctr[kCtrWork] = 0;
    ctr[kCtrSlow] = 0;
  }
}
__global__ void k_zero_shade_counters(uint32_t* ctr, int nxt) {
  if (threadIdx.x == 0) {
    ctr[kCtrQ0 + nxt] = 0;
    ctr[kCtrShadow] = 0;
    ctr[kCtrWork2] = 0;
    ctr[kCtrSlow2] = 0;
    ctr[kCtrTex] = 0;
  }
}
__global__ void k_count_rays(uint32_t* ctr, int cur) {  // statistics: rays traced this bounce
  if (threadIdx.x == 0) {
    atomicAdd((unsigned long long*)(ctr + kCtrStatClosest), (unsigned long long)ctr[kCtrQ0 + cur]);
    atomicAdd((unsigned long long*)(ctr + kCtrStatShadow), (unsigned long long)ctr[kCtrShadow]);
  }
}

// ------------------------------------------------------------ ray capture
// Closest-hit rays of a bounce in queue order with their hits and alpha keys:
// (origin, path id), (direction, scene), (t, u, v, slot), (key, 0, 0, 0).
// The hit is the triangle the traversal found with the values the shade
// kernel computes for it (hit_values).
__global__ void k_capture_closest(const uint32_t* __restrict__ cnt, const float4* __restrict__ rays,
                                  const float4* __restrict__ hits, PathField ro,
                                  const SceneRec* __restrict__ recs, float4* __restrict__ out,
                                  uint32_t* __restrict__ count, uint32_t cap) {
  const uint32_t n = *cnt, m = n < cap ? n : cap;
  if (blockIdx.x == 0 && threadIdx.x == 0) *count = n;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
    const float4 a = rays[2 * (size_t)k], b = rays[2 * (size_t)k + 1];
    float4 h = hits[k];
    if (__float_as_int(h.w) >= 0)
      h = hit_values(recs[__float_as_int(b.w)].scene.geo, make_float3(a.x, a.y, a.z), make_float3(b.x, b.y, b.z),
                     __float_as_int(h.w));
    out[4 * (size_t)k] = a;
    out[4 * (size_t)k + 1] = b;
    out[4 * (size_t)k + 2] = h;
    out[4 * (size_t)k + 3] = make_float4(ro[__float_as_uint(a.w)].w, 0.f, 0.f, 0.f);
  }
}

// Shadow rays of a bounce in shadow-queue order with their answers:
// (origin, t_max), (direction, alpha key), (occluded, shadow slot, 0, 0), 0.
__global__ void k_capture_shadow(const uint32_t* __restrict__ cnt, const uint32_t* __restrict__ queue,
                                 const float4* __restrict__ so, const float4* __restrict__ sd,
                                 const float4* __restrict__ sh_c, float4* __restrict__ out,
                                 uint32_t* __restrict__ count, uint32_t cap) {
  const uint32_t n = *cnt, m = n < cap ? n : cap;
  if (blockIdx.x == 0 && threadIdx.x == 0) *count = n;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
    const uint32_t slot = queue[k];
    out[4 * (size_t)k] = so[k];
    out[4 * (size_t)k + 1] = sd[k];
    out[4 * (size_t)k + 2] = make_float4(sh_c[slot].w == 0.f ? 1.f : 0.f, __uint_as_float(slot), 0.f, 0.f);
    out[4 * (size_t)k + 3] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

// ------------------------------------------------------------ ray reordering
// Between bounces the queue of surviving paths is counting-sorted by a
// 15-bit key of (BVH class, direction: cube-map face and a 4 x 4 cell on it,
// origin: Morton code of an 8^3 grid over its scene's bounds), so that a
// warp's rays start in similar places and head the same way: fewer divergent
// traversal steps and more cache reuse. Paths are independent, so the order
// changes no result.
__device__ __forceinline__ uint32_t spread3(uint32_t x) {  // 4 bits -> every third bit
  x &= 15u;
  x = (x | (x << 4)) & 0x0C3u;
  x = (x | (x << 2)) & 0x249u;
  return x;
}

__global__ void k_sort_keys(Paths P, const SceneRec* __restrict__ recs, int n_classes, int nxt) {
  const uint32_t n = P.ctr[kCtrQ0 + nxt];
  int sbits = 0;
  while ((1 << sbits) < n_classes) sbits++;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const float4 o = P.nray[2 * (size_t)k], d = P.nray[2 * (size_t)k + 1];  // the queue's rays, in order
    const int sc = __float_as_int(d.w);
    const Node* nodes = recs[sc].scene.nodes;
    const float4 lo = __ldg(reinterpret_cast<const float4*>(nodes)), hi = __ldg(reinterpret_cast<const float4*>(nodes) + 1);
    auto cell = [](float v, float a, float b) {
      const float t = (v - a) / fmaxf(b - a, 1e-20f);
      return (uint32_t)fminf(fmaxf(t * 16.f, 0.f), 15.f);
    };
    // origin: Morton code of an 8^3 grid over the scene box (9 bits)
    const uint32_t m = spread3(cell(o.x, lo.x, hi.x) >> 1) | (spread3(cell(o.y, lo.y, hi.y) >> 1) << 1) |
                       (spread3(cell(o.z, lo.z, hi.z) >> 1) << 2);
    // direction: cube-map face (major axis and sign) and a 4 x 4 cell on it (7 bits)
    const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    uint32_t face;
    float fu, fv, fm;
    if (ax >= ay && ax >= az) { face = d.x < 0.f ? 1u : 0u; fu = d.y; fv = d.z; fm = ax; }
    else if (ay >= az) { face = d.y < 0.f ? 3u : 2u; fu = d.x; fv = d.z; fm = ay; }
    else { face = d.z < 0.f ? 5u : 4u; fu = d.x; fv = d.y; fm = az; }
    const uint32_t cu = (uint32_t)fminf(fmaxf((fu / fm + 1.f) * 2.f, 0.f), 3.f);
    const uint32_t cv = (uint32_t)fminf(fmaxf((fv / fm + 1.f) * 2.f, 0.f), 3.f);
    const uint32_t local = (((face << 4) | (cu << 2) | cv) << 9 | m) >> 1;  // 15 bits (the finest origin bit dropped)
    const uint32_t cls = (uint32_t)min(max(recs[sc].sort_class, 0), n_classes - 1);  // keys stay below kSortBins
    const uint32_t key = (cls << (kSortBits - sbits)) | (local >> sbits);
    P.sort_keys[k] = key;
    const unsigned peers = __match_any_sync(__activemask(), key);  // one atomic per distinct key per warp
    if ((threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(P.sort_hist + key, (uint32_t)__popc(peers));
  }
}

// Exclusive scan of the kSortBins counters, one block of 32 warps: warp w
// owns bins [w * 1024, (w + 1) * 1024), read 32 at a time (coalesced) and
// scanned with shuffles; then the warp totals are scanned.
__global__ void __launch_bounds__(1024) k_sort_scan(uint32_t* __restrict__ hist) {
  constexpr int kPerWarp = kSortBins / 32, kSteps = kPerWarp / 32;
  __shared__ uint32_t warp_total[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t* seg = hist + w * kPerWarp;
  uint32_t v[kSteps], carry = 0;
#pragma unroll
  for (int j = 0; j < kSteps; j++) {
    const uint32_t x = seg[j * 32 + lane];
    uint32_t incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    v[j] = carry + incl - x;
    carry += __shfl_sync(0xffffffffu, incl, 31);
  }
  if (lane == 0) warp_total[w] = carry;
  __syncthreads();
  if (w == 0) {
    const uint32_t x = warp_total[lane];
    uint32_t incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    warp_total[lane] = incl - x;
  }
  __syncthreads();
  const uint32_t base = warp_total[w];
#pragma unroll
  for (int j = 0; j < kSteps; j++) seg[j * 32 + lane] = base + v[j];
}

// Copies each queued ray (read in queue order from the unsorted stream) to
// its sorted position in the sorted stream, and the path to the sorted queue.
__global__ void k_sort_scatter(Paths P, int nxt) {
  const uint32_t n = P.ctr[kCtrQ0 + nxt];
  const uint32_t* q = P.q[nxt];
  const unsigned lane = threadIdx.x & 31;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const uint32_t key = P.sort_keys[k];
    const unsigned peers = __match_any_sync(__activemask(), key);
    const int leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if ((int)lane == leader) base = atomicAdd(P.sort_hist + key, (uint32_t)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    const uint32_t pos = base + __popc(peers & ((1u << lane) - 1u));
    P.sray[2 * (size_t)pos] = P.nray[2 * (size_t)k];  // origin + path id
    P.sray[2 * (size_t)pos + 1] = P.nray[2 * (size_t)k + 1];  // direction + scene
    P.sort_tmp[pos] = q[k];
  }
}

// Sorts the rays of queue `nxt` into the ray stream and the queue into the
// free queue buffer `dst`, which becomes queue `nxt`; returns the buffer of
// the pre-sort queue. P is the caller's copy of the path state: every wave
// starts from the launch's own pointers, so a captured wave replays the same
// sequence of buffer rotations.
static uint32_t* sort_rays_into(const MultiLaunch& M, Paths& P, int nxt, int blocks, cudaStream_t s, uint32_t* dst) {
  Paths Ps = P;
  Ps.sort_tmp = dst;
  cudaMemsetAsync(P.sort_hist, 0, (size_t)kSortBins * 4, s);
  k_sort_keys<<<blocks, 256, 0, s>>>(Ps, M.recs, M.sort_classes > 0 ? M.sort_classes : M.n, nxt);
  k_sort_scan<<<1, 1024, 0, s>>>(P.sort_hist);
  k_sort_scatter<<<blocks, 256, 0, s>>>(Ps, nxt);
  uint32_t* pre = P.q[nxt];
  P.q[nxt] = dst;
  return pre;
}
// The sorted queue into sort_tmp, the pre-sort queue kept there in its place.
static void sort_rays(const MultiLaunch& M, Paths& P, int nxt, int blocks, cudaStream_t s) {
  P.sort_tmp = sort_rays_into(M, P, nxt, blocks, s, P.sort_tmp);
}

// ------------------------------------------------------------ one wave
// Grid of the any-hit (twice this many blocks of 256), resolve and sort
// kernels: five 128-thread blocks per SM (measured; smaller grids slowed the
// any-hit and resolve kernels).
static int aux_blocks() {
  static int n = 0;
  if (!n) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    n = 5 * (sms > 0 ? sms : 152);
  }
  return n;
}

// Closest hit of a bounce: over the scenes' four-wide BVH views, or the
// binary nodes with the top levels staged in shared memory. Hits are the same.
static void launch_closest_multi(int wide, int blocks, int top, const TravArgs& A, const PathClosestMulti& pc,
                                 cudaStream_t s) {
  if (wide)
    k_closest_wide_t<PathClosestMulti><<<blocks, PathClosestMulti::kThreads, 0, s>>>(A, pc);
  else
    k_closest_fast_t<PathClosestMulti><<<blocks, PathClosestMulti::kThreads, top_smem_bytes(top), s>>>(A, pc);
}

static void launch_shadow_multi(int wide, int blocks, int top, const TravArgs& A, const PathShadowMulti& ps,
                                cudaStream_t s) {
  if (wide)
    k_anyhit_wide_t<PathShadowMulti><<<blocks, 256, 0, s>>>(A, ps);
  else
    k_anyhit_fast_t<PathShadowMulti><<<blocks, 256, top_smem_bytes(top), s>>>(A, ps);
}

int render_wave_multi(const MultiLaunch& M, cudaStream_t s, PhaseEvents* pe, bool accumulate) {
  int nl = 0;  // kernels launched
  Paths P = M.paths;  // queue buffers swap with the sort buffer below
  PhaseEvents none{nullptr, nullptr, 0, 0};
  PhaseEvents& E = pe ? *pe : none;
  E.mark(-1, s);
  k_camera_multi<<<grid_for(M.total_paths, 256), 256, 0, s>>>(P, M.recs, M.path_base, M.n, M.sid, M.S);
  nl++;
  E.mark(kPhCamera, s);
  static int max_closest = 0, max_wide = 0, max_shade = 0;
  if (!max_closest) {
    max_closest = persistent_blocks((const void*)k_closest_fast_t<PathClosestMulti>, PathClosestMulti::kThreads);
    max_wide = persistent_blocks((const void*)k_closest_wide_t<PathClosestMulti>, PathClosestMulti::kThreads);
    max_shade = persistent_blocks((const void*)k_shade_t<SceneTable>, 128);
  }
  const int closest_blocks = M.trace_blocks > 0 ? M.trace_blocks : M.wide ? max_wide : max_closest;
  const int shade_blocks = M.shade_blocks > 0 ? M.shade_blocks : max_shade;
  const int aux = M.shade_blocks > 0 ? M.shade_blocks : aux_blocks();
  const int top = M.top_levels ? (M.n < kTopMaxScenes ? M.n : kTopMaxScenes) : 0;
  bool sorted = false;  // the rays of this bounce are in the sorted stream
  bool forked = false;  // the previous bounce's shadow rays and resolve run on M.side
  for (int b = 0; b <= M.max_bounces; b++) {
    const int cur = b & 1;
    if (forked)  // the side stream still reads the other counters
      k_zero_closest_counters<<<1, 32, 0, s>>>(P.ctr);
    else
      k_zero_counters<<<1, 32, 0, s>>>(P.ctr, cur ^ 1);
    nl++;
    E.mark(kPhResolve, s);
    PathClosestMulti pc{P.ctr + kCtrQ0 + cur, sorted ? P.sray : P.nray, P.ro, P.hit, M.recs, M.any_alpha};
    TravArgs A{nullptr, 0, nullptr, 1e-6, 1e30, P.slow, P.ctr + kCtrSlow, P.ctr + kCtrWork, P.ctr + kCtrErr,
               M.trav_stats, top};
    launch_closest_multi(M.wide, closest_blocks, top, A, pc, s);
    k_closest_exact_t<PathClosestMulti><<<64, 128, 0, s>>>(A, pc);
    nl += 2;
    const bool capture = M.cap && (M.cap_mask >> b & 1u);
    const uint32_t region = capture ? 2u * (uint32_t)__builtin_popcount(M.cap_mask & ((1u << b) - 1u)) : 0u;
    if (capture)
      k_capture_closest<<<aux, 256, 0, s>>>(P.ctr + kCtrQ0 + cur, pc.rays, P.hit, P.ro, M.recs,
                                            M.cap + (size_t)region * M.cap_stride * 4, M.cap_count + region,
                                            M.cap_stride);
    nl += capture;
    E.mark(kPhClosest, s);
    if (forked) {  // join: the previous bounce's radiance is resolved before this bounce shades
      cudaStreamWaitEvent(s, M.ev_join, 0);
      k_zero_shade_counters<<<1, 32, 0, s>>>(P.ctr, cur ^ 1);
      nl++;
    }
    k_shade_t<SceneTable><<<shade_blocks, 128, 0, s>>>(P, SceneTable{M.recs, M.sid}, cur, b);
    if (M.any_tex) k_shade_t<SceneTable, false, true><<<shade_blocks, 128, 0, s>>>(P, SceneTable{M.recs, M.sid}, cur, b);
    nl += 1 + (M.any_tex != 0);
    E.mark(kPhShade, s);
    // This bounce's shadow rays do not depend on the next bounce's ray sort
    // and closest hit, nor they on them: they run side by side on two streams,
    // so the short launches of the deep bounces overlap; the next shade, which
    // resolves them, waits for both. Profiling keeps one stream (phase times).
    const bool fork = M.side && !pe && b < M.max_bounces;
    cudaStream_t t = s;
    if (fork) {
      cudaEventRecord(M.ev_fork, s);
      cudaStreamWaitEvent(M.side, M.ev_fork, 0);
      t = M.side;
    }
    PathShadowMulti ps{P.ctr + kCtrShadow, P.qs, P.sh_o, P.sh_d, P.sh_c, M.recs, M.sid, M.any_alpha};
    TravArgs B{nullptr, 0, nullptr, 1e-6, 1e30, P.slow2, P.ctr + kCtrSlow2, P.ctr + kCtrWork2, P.ctr + kCtrErr,
               nullptr, top};
    launch_shadow_multi(M.wide, aux * 2, top, B, ps, t);
    k_anyhit_exact_t<PathShadowMulti><<<64, 128, 0, t>>>(B, ps);
    nl += 2;
    if (capture)
      k_capture_shadow<<<aux, 256, 0, t>>>(P.ctr + kCtrShadow, P.qs, P.sh_o, P.sh_d, P.sh_c,
                                           M.cap + (size_t)(region + 1) * M.cap_stride * 4, M.cap_count + region + 1,
                                           M.cap_stride);
    nl += capture;
    E.mark(kPhShadow, s);
    // No resolve launch: the next shade (or the accumulation, for paths
    // that end here) adds this bounce's unoccluded contributions.
    k_count_rays<<<1, 32, 0, t>>>(P.ctr, cur);
    nl++;
    if (fork) cudaEventRecord(M.ev_join, t);
    forked = fork;
    const bool was_sorted = sorted;
    // The two largest queues; the third too in waves of 2^21 paths or more
    // (measured: it pays for its sort there, not in smaller waves).
    sorted = M.sort_rays && b < M.max_bounces && (b < 2 || (b == 2 && M.total_paths >= (1u << 21)));
    nl += sorted ? 3 : 0;  // keys, scan, scatter
    if (sorted && was_sorted) {
      // This bounce's pre-sort queue in sort_tmp stays as it is (the backward
      // replays' resolve, perhaps still running on the side stream, walks it);
      // its sorted queue buffer is free once shaded, so the next queue is
      // sorted into that one instead, and sort_tmp becomes the next-but-one
      // queue after the join.
      uint32_t* busy = P.sort_tmp;
      P.sort_tmp = sort_rays_into(M, P, cur ^ 1, aux, s, P.q[cur]);
      P.q[cur] = busy;
    } else if (sorted) {
      sort_rays(M, P, cur ^ 1, aux, s);
    }
  }
  E.mark(kPhResolve, s);
  if (accumulate) nl += accumulate_wave(M, s);
  E.mark(kPhAccumulate, s);
  return nl;
}

int accumulate_wave(const MultiLaunch& M, cudaStream_t s) {
  k_accumulate_multi<<<grid_for(M.total_pixels, 256), 256, 0, s>>>(M.paths, M.recs, M.pix_base, M.path_base, M.n,
                                                                     M.S);
  k_advance_seeds<<<1, 64, 0, s>>>(M.recs, M.n, M.S);
  return 2;
}

// ------------------------------------------------------------ path replay backpropagation
// Replays the wave's samples twice with the adjoint instantiation of the
// shade kernel (one instantiation, so both replays make identical choices):
// first with the adjoint work off to recover each sample's primal radiance,
// then propagating dl through every vertex.
void render_backward(const MultiLaunch& M, const AdjointDevHost& H, cudaStream_t s) {
  const SceneRec* rec = M.recs;
  static int binary_blocks = 0, wide_blocks = 0, shade_blocks = 0;
  if (!binary_blocks) {
    binary_blocks = persistent_blocks((const void*)k_closest_fast_t<PathClosestMulti>, PathClosestMulti::kThreads);
    wide_blocks = persistent_blocks((const void*)k_closest_wide_t<PathClosestMulti>, PathClosestMulti::kThreads);
    shade_blocks = persistent_blocks((const void*)k_shade_t<SceneTable, true>, 128);
  }
  const int closest_blocks = M.wide ? wide_blocks : binary_blocks;
  const int aux = aux_blocks();
  const int top = M.top_levels ? (M.n < kTopMaxScenes ? M.n : kTopMaxScenes) : 0;
  for (int pass = 0; pass < 2; pass++) {
    const AdjointDev A{H.dl, H.lrem, H.gcont, H.gslot, H.genv, H.dmat, H.denv, M.total_pixels, pass == 0 ? 1 : 0};
    Paths P = M.paths;     // queue buffers swap with the sort buffer below
    bool sorted = false;  // as in render_wave_multi: the rays of bounces 1 and 2 are sorted
    bool forked = false;  // as in render_wave_multi: shadow rays and resolve on M.side
    k_camera_multi<<<grid_for(M.total_paths, 256), 256, 0, s>>>(P, M.recs, M.path_base, M.n, M.sid, M.S);
    for (int b = 0; b <= M.max_bounces; b++) {
      const int cur = b & 1;
      if (forked)
        k_zero_closest_counters<<<1, 32, 0, s>>>(P.ctr);
      else
        k_zero_counters<<<1, 32, 0, s>>>(P.ctr, cur ^ 1);
      PathClosestMulti pc{P.ctr + kCtrQ0 + cur, sorted ? P.sray : P.nray, P.ro, P.hit, M.recs, M.any_alpha};
      TravArgs TA{nullptr, 0, nullptr, 1e-6, 1e30, P.slow, P.ctr + kCtrSlow, P.ctr + kCtrWork, P.ctr + kCtrErr,
                  nullptr, top};
      launch_closest_multi(M.wide, closest_blocks, top, TA, pc, s);
      k_closest_exact_t<PathClosestMulti><<<64, 128, 0, s>>>(TA, pc);
      if (forked) {  // the previous bounce's resolve (lrem, radiance) precedes this shade
        cudaStreamWaitEvent(s, M.ev_join, 0);
        k_zero_shade_counters<<<1, 32, 0, s>>>(P.ctr, cur ^ 1);
      }
      k_shade_t<SceneTable, true><<<shade_blocks, 128, 0, s>>>(P, SceneTable{M.recs, M.sid}, cur, b, A);
      const bool fork = M.side && b < M.max_bounces;
      cudaStream_t t = s;
      if (fork) {
        cudaEventRecord(M.ev_fork, s);
        cudaStreamWaitEvent(M.side, M.ev_fork, 0);
        t = M.side;
      }
      PathShadowMulti ps{P.ctr + kCtrShadow, P.qs, P.sh_o, P.sh_d, P.sh_c, M.recs, M.sid, M.any_alpha};
      TravArgs TB{nullptr, 0, nullptr, 1e-6, 1e30, P.slow2, P.ctr + kCtrSlow2, P.ctr + kCtrWork2, P.ctr + kCtrErr,
                  nullptr, top};
      launch_shadow_multi(M.wide, aux * 2, top, TB, ps, t);
      k_anyhit_exact_t<PathShadowMulti><<<64, 128, 0, t>>>(TB, ps);
      Paths Pr = P;  // resolve walks the pre-sort queue, in path order
      if (sorted) Pr.q[cur] = P.sort_tmp;
      if (pass == 1)  // the primal replay resolves in its next shade and in k_seed_lrem
        k_resolve_adjoint<<<aux, 128, 0, t>>>(Pr, A, rec, cur);
      if (fork) cudaEventRecord(M.ev_join, t);
      forked = fork;
      const bool was_sorted = sorted;
      sorted = M.sort_rays && b < M.max_bounces && (b < 2 || (b == 2 && M.total_paths >= (1u << 21)));
      if (sorted && was_sorted) {  // as in render_wave_multi
        uint32_t* busy = P.sort_tmp;
        P.sort_tmp = sort_rays_into(M, P, cur ^ 1, aux, s, P.q[cur]);
        P.q[cur] = busy;
      } else if (sorted) {
        sort_rays(M, P, cur ^ 1, aux, s);
      }
    }
    if (pass == 0) k_seed_lrem<<<grid_for(M.total_paths, 256), 256, 0, s>>>(P, A, M.total_paths);
  }
}

}  // namespace lucent
