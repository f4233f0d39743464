// Renderer C ABI: scene / lighting / camera upload, accumulation targets,
// trace, readback. Mirrors the Renderer class of src/renderer.ts.
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/lucent.h"
#include "api_util.h"
#include "internal.h"
#include "render_internal.h"

using namespace lucent;

namespace lucent {

// Packs the scene's triangles into BVH leaf order (scene.ts:215-235):
// geo = (v0, material), (v1, light), (v2, alpha flag);
// attr = (n0, u0), (n1, u1), (n2, u2), (v0, v1, v2, 0).
__global__ void k_pack_scene(const float* __restrict__ pos, const float* __restrict__ nrm,
                             const float* __restrict__ uvs, const int32_t* __restrict__ mat,
                             const int32_t* __restrict__ light, const uint8_t* __restrict__ alpha,
                             const uint32_t* __restrict__ tri_indices, uint32_t n, float4* __restrict__ geo,
                             float4* __restrict__ attr) {
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    const uint32_t src = tri_indices[s];
    const float* p = pos + (size_t)src * 9;
    const float* q = nrm + (size_t)src * 9;
    const float* u = uvs ? uvs + (size_t)src * 6 : nullptr;
    geo[3 * (size_t)s] = make_float4(p[0], p[1], p[2], (float)mat[src]);
    geo[3 * (size_t)s + 1] = make_float4(p[3], p[4], p[5], light ? (float)light[src] : -1.f);
    geo[3 * (size_t)s + 2] = make_float4(p[6], p[7], p[8], alpha ? (float)alpha[src] : 0.f);
    for (int v = 0; v < 3; v++)
      attr[4 * (size_t)s + v] = make_float4(q[v * 3], q[v * 3 + 1], q[v * 3 + 2], u ? u[v * 2] : 0.f);
    attr[4 * (size_t)s + 3] = make_float4(u ? u[1] : 0.f, u ? u[3] : 0.f, u ? u[5] : 0.f, 0.f);
  }
}

__global__ void k_clear_accum(AccumDev A, uint32_t n) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    A.color[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    A.albedo[i] = make_half4(make_float4(0.f, 0.f, 0.f, 0.f));
    A.normal[i] = make_half4(make_float4(0.f, 0.f, 0.f, 0.f));
    A.history[i] = 0.f;
  }
}

__global__ void k_unpack_accum(AccumDev A, uint32_t n, float* alb, float* nrm) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const half4 a = A.albedo[i], b = A.normal[i];
    if (alb) {
      alb[4 * i] = __half2float(a.x), alb[4 * i + 1] = __half2float(a.y);
      alb[4 * i + 2] = __half2float(a.z), alb[4 * i + 3] = __half2float(a.w);
    }
    if (nrm) {
      nrm[4 * i] = __half2float(b.x), nrm[4 * i + 1] = __half2float(b.y);
      nrm[4 * i + 2] = __half2float(b.z), nrm[4 * i + 3] = __half2float(b.w);
    }
  }
}

// ------------------------------------------------------------ host precompute
// buildAliasTable (src/math/alias.ts:17-65), Vose's method.
static bool alias_table(const std::vector<double>& w, std::vector<float>& prob, std::vector<uint32_t>& alias,
                        std::vector<double>& pmf, double& total) {
  const size_t n = w.size();
  if (n == 0) return false;
  total = 0;
  for (double x : w) {
    if (!(x >= 0) || !std::isfinite(x)) return false;
    total += x;
  }
  pmf.resize(n);
  for (size_t i = 0; i < n; i++) pmf[i] = total > 0 ? w[i] / total : 1.0 / (double)n;
  std::vector<double> scaled(n);
  std::vector<uint32_t> small, large;
  small.reserve(n);
  large.reserve(n);
  for (size_t i = 0; i < n; i++) {
    scaled[i] = pmf[i] * (double)n;
    (scaled[i] < 1 ? small : large).push_back((uint32_t)i);
  }
  prob.assign(n, 0.f);
  alias.assign(n, 0u);
  while (!small.empty() && !large.empty()) {
    const uint32_t s = small.back(), l = large.back();
    small.pop_back();
    large.pop_back();
    prob[s] = (float)scaled[s];
    alias[s] = l;
    scaled[l] = scaled[l] + scaled[s] - 1;
    (scaled[l] < 1 ? small : large).push_back(l);
  }
  while (!large.empty()) {
    prob[large.back()] = 1;
    alias[large.back()] = large.back();
    large.pop_back();
  }
  while (!small.empty()) {
    prob[small.back()] = 1;
    alias[small.back()] = small.back();
    small.pop_back();
  }
  return true;
}

// buildEnvSampler (src/scene/environment.ts:52-85): cells of a grid at most
// max_w wide, weight = mean luminance x sin(theta), then the alias table; 4
// floats per cell (keep probability, alias cell, pdfUV, alias pdfUV).
static bool env_sampler(const float* rgb, uint32_t w, uint32_t h, uint32_t max_w, uint32_t& gw, uint32_t& gh,
                        std::vector<float>& table, double& total) {
  gw = std::max(1u, std::min(w, max_w));
  gh = std::max(1u, std::min(h, (uint32_t)std::floor((double)h * gw / w + 0.5)));
  std::vector<double> weights((size_t)gw * gh);
  for (uint32_t cy = 0; cy < gh; cy++) {
    const uint64_t y0 = (uint64_t)std::floor((double)cy * h / gh);
    const uint64_t y1 = std::max(y0 + 1, (uint64_t)std::floor((double)(cy + 1) * h / gh));
    const double st = std::sin(M_PI * (cy + 0.5) / gh);
    for (uint32_t cx = 0; cx < gw; cx++) {
      const uint64_t x0 = (uint64_t)std::floor((double)cx * w / gw);
      const uint64_t x1 = std::max(x0 + 1, (uint64_t)std::floor((double)(cx + 1) * w / gw));
      double sum = 0;
      for (uint64_t y = y0; y < y1; y++)
        for (uint64_t x = x0; x < x1; x++) {
          const float* p = rgb + (y * w + x) * 3;
          sum += 0.2126 * (double)p[0] + 0.7152 * (double)p[1] + 0.0722 * (double)p[2];
        }
      weights[(size_t)cy * gw + cx] = (sum / (double)((y1 - y0) * (x1 - x0))) * st;
    }
  }
  std::vector<float> prob;
  std::vector<uint32_t> alias;
  std::vector<double> pmf;
  if (!alias_table(weights, prob, alias, pmf, total)) return false;
  const size_t n = weights.size();
  table.resize(n * 4);
  for (size_t i = 0; i < n; i++) {
    table[i * 4] = prob[i];
    table[i * 4 + 1] = (float)alias[i];
    table[i * 4 + 2] = (float)(pmf[i] * (double)n);
    table[i * 4 + 3] = (float)(pmf[alias[i]] * (double)n);
  }
  return true;
}

// sheenAlbedoLUT (src/scene/sheen.ts:13-60): 16 x 16, 96 quadrature steps,
// then rounded to half precision like the reference's R16F upload.
void sheen_lut_half(float* out) {
  const int size = 16, steps = 96;
  for (int y = 0; y < size; y++)
    for (int x = 0; x < size; x++) {
      const double cosV = std::max(1e-3, (double)x / (size - 1));
      const double r = std::max(0.07, (double)y / (size - 1));
      const double alpha = r * r, inv = 1 / alpha;
      const double v0 = std::sqrt(std::max(0.0, 1 - cosV * cosV)), v2 = cosV;
      const int phi_steps = steps / 2;
      const double dth = M_PI / 2 / steps, dph = M_PI / phi_steps;
      double e = 0;
      for (int i = 0; i < steps; i++) {
        const double th = (i + 0.5) * dth, ch = std::cos(th), shh = std::sin(th);
        const double d = ((2 + inv) * std::pow(std::max(0.0, 1 - ch * ch), inv * 0.5)) / (2 * M_PI);
        for (int j = 0; j < phi_steps; j++) {
          const double ph = (j + 0.5) * dph;
          const double vh = v0 * (shh * std::cos(ph)) + v2 * ch;
          if (vh <= 0) continue;
          const double cosL = 2 * vh * ch - v2;
          if (cosL <= 0) continue;
          e += d * (1 / (4 * (cosL + cosV - cosL * cosV))) * cosL * 4 * vh * shh * dth * dph;
        }
      }
      out[y * size + x] = __half2float(__float2half_rn((float)std::min(1.0, 2 * e)));
    }
}

}  // namespace lucent

// One full wave captured as a CUDA graph on a private stream (the legacy
// stream cannot be captured) and replayed while the launch parameters it
// bakes in (`key`: sizes, options, buffer addresses) are unchanged. Saves the
// launch gaps between the wave's ~80 dependent kernels.
struct WaveGraph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  uint64_t key[4] = {0, 0, 0, 0};
  cudaStream_t cap = nullptr;
  int launches = 0;  // kernels in the captured wave
  void drop() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
  }
  void destroy() {
    drop();
    if (cap) cudaStreamDestroy(cap);
    cap = nullptr;
  }
  lucent_status run(const MultiLaunch& M, const uint64_t k[4], cudaStream_t s, bool accumulate = true) {
    cudaError_t e;
    if (!exec || std::memcmp(k, key, sizeof key) != 0) {
      drop();
      if (!cap && (e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking)) != cudaSuccess)
        return cuda_fail(e, "capture stream");
      if ((e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
        return cuda_fail(e, "begin capture");
      launches = render_wave_multi(M, cap, nullptr, accumulate);
      e = cudaStreamEndCapture(cap, &graph);
      if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
      if (e != cudaSuccess) {
        drop();
        return cuda_fail(e, "capture wave");
      }
      std::memcpy(key, k, sizeof key);
    }
    e = cudaGraphLaunch(exec, s);
    return e == cudaSuccess ? LUCENT_OK : cuda_fail(e, "launch wave graph");
  }
};

// The second stream of a wave (MultiLaunch::side) with its fork / join events.
struct SideStream {
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  lucent_status ensure() {
    if (stream) return LUCENT_OK;
    cudaError_t e = cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&join, cudaEventDisableTiming);
    if (e != cudaSuccess) {
      destroy();
      return cuda_fail(e, "side stream");
    }
    return LUCENT_OK;
  }
  void set(MultiLaunch& M) const {
    M.side = stream;
    M.ev_fork = fork;
    M.ev_join = join;
  }
  void destroy() {
    if (join) cudaEventDestroy(join);
    if (fork) cudaEventDestroy(fork);
    if (stream) cudaStreamDestroy(stream);
    stream = nullptr;
    fork = join = nullptr;
  }
};

// The path state of one wave and what launches it. A renderer keeps two:
// successive waves alternate between them, each traced on its set's own
// stream, so one wave's deep bounces (short, latency-bound launches that
// leave most SMs idle) run beside the next wave's first bounces. Only the
// accumulation into the targets runs on the caller's stream, after the wave
// and in call order.
struct WaveSet {
  DeviceBuffer paths, ctr;
  DeviceBuffer rec, base;  // the wave's scene records and path / pixel bases
  DeviceBuffer sid;        // scene index per path (written by the camera kernel)
  uint32_t path_cap = 0, sid_cap = 0;
  Paths P{};
  WaveGraph graph;  // full waves replay a captured graph (not while profiling)
  SideStream side;  // second stream of the wave
  cudaStream_t stream = nullptr;
  cudaEvent_t traced = nullptr;  // on `stream`: the wave's last bounce is done
  cudaEvent_t done = nullptr;    // on the caller's stream: the wave is accumulated
  bool used = false;             // `done` has been recorded
  lucent_status ensure() {
    if (stream) return LUCENT_OK;
    cudaError_t e = cudaEventCreateWithFlags(&traced, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {  // nothing half made: the next call tries again
      if (done) cudaEventDestroy(done);
      if (traced) cudaEventDestroy(traced);
      traced = done = nullptr;
      stream = nullptr;
      return cuda_fail(e, "wave stream");
    }
    return LUCENT_OK;
  }
  void release_paths() {
    paths.release();
    path_cap = 0;
    P = Paths{};
    P.ctr = (uint32_t*)ctr.ptr;
  }
  // Path buffers and scene indices for `cap` paths.
  lucent_status reserve(uint32_t cap);
  void destroy() {
    for (DeviceBuffer* b : {&paths, &ctr, &rec, &base, &sid}) b->release();
    sid_cap = 0;
    graph.destroy();
    side.destroy();
    if (done) cudaEventDestroy(done);
    if (traced) cudaEventDestroy(traced);
    if (stream) cudaStreamDestroy(stream);
    stream = nullptr;
    traced = done = nullptr;
  }
};

// Everything a captured wave bakes in besides the buffer contents.
static void wave_key(const MultiLaunch& M, uint64_t key[4]) {
  key[0] = (uint64_t)(uint32_t)M.S | ((uint64_t)(uint32_t)M.n << 32);
  key[1] = (uint64_t)M.total_pixels | ((uint64_t)(uint32_t)M.trace_blocks << 32) ^ ((uint64_t)M.sort_classes << 48);
  key[2] = ((uint64_t)(uintptr_t)M.paths.rec) ^ ((uint64_t)M.max_bounces << 48) ^ ((uint64_t)M.shade_blocks << 56);
  key[3] = ((uint64_t)(uintptr_t)M.recs) ^ ((uint64_t)(uintptr_t)M.path_base << 20) ^ ((uint64_t)M.any_alpha << 59) ^
           ((uint64_t)(M.side != nullptr) << 57) ^ ((uint64_t)M.wide << 58) ^ ((uint64_t)M.any_tex << 60) ^ ((uint64_t)M.sort_rays << 61) ^
           ((uint64_t)M.top_levels << 62) ^
           ((uint64_t)(M.trav_stats != nullptr) << 63);
}

struct lucent_renderer {
  uint32_t W = 1, H = 1;
  // scene
  DeviceBuffer nodes, geo, attr, mats, spheres, sph_mat, sph_light, lights;
  DeviceBuffer wide;  // four-wide view of `nodes` (traverse_wide.cuh)
  // A view (lucent_renderer_create_view) renders `src`'s scene: the scene
  // fields below are read from src; n_views counts the views of this one.
  lucent_renderer* src = nullptr;
  int n_views = 0;
  // texture arrays (sRGB colour layers, linear data layers), decode tables, layer size (0: none)
  DeviceBuffer color_maps, data_maps, texel_lut;
  int tex_size = 0;
  uint32_t color_layers = 0, data_layers = 0;
  uint32_t node_count = 0, tri_count = 0, material_count = 0, sphere_count = 0, light_count = 0;
  int32_t ground_material = -1, ground_enabled = 0, any_alpha = 0;
  float ground_height = 0;
  bool has_scene = false;
  // lighting
  DeviceBuffer env_rgb, env_alias, sheen;
  sh::LightingDev light{};
  bool has_lighting = false;
  // camera and settings (renderer.ts DEFAULT_SETTINGS: maxBounces 6, fireflyClamp 8)
  sh::CameraDev cam{};
  uint32_t max_bounces = 6;
  float clamp = 8.f;
  // targets and path state
  DeviceBuffer color, albedo, normal, history;
  WaveSet set[2];   // set 0 also serves every wave that is not pipelined
  int next_set = 0;  // set of the next pipelined wave
  int pipeline = 1;  // alternate the waves between the sets (lucent_renderer_set_pipelining)
  uint32_t frame = 0, seed = 0;
  double last_ms = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;  // around the last trace (recorded once it traced)
  bool timed = false;
  // optional per-phase timing (lucent_renderer_set_profiling)
  bool profiling = false;
  bool trav_counters = false;  // closest-hit traversal counters (profiling mode 2)
  std::vector<cudaEvent_t> pev;
  std::vector<int> ptag;
  int pn = 0;
  double phase_ms[kPhases] = {0, 0, 0, 0, 0, 0};
  // denoiser ping-pong targets, guide buffers, display staging
  DeviceBuffer den_a, den_b, guide0, guide1, disp;
  // path-replay backward pass
  DeviceBuffer adj_dl, adj_path, adj_grad;
  uint32_t waves = 0;
  uint64_t kernel_launches = 0;  // by reset and trace (lucent_render_stats)
  int sort_rays = 1;   // sort the rays of bounces 1 and 2 (lucent_renderer_set_ray_sort)
  int top_levels = 1;  // top BVH levels in shared memory (lucent_renderer_set_top_levels)
  int wide_bvh = 1;    // four-wide closest-hit traversal (lucent_renderer_set_wide_bvh)
  // temporal reprojection (renderer.ts:441-451, 717-731): the view the accumulation was traced with
  int temporal = 1;
  bool has_history = false, reproject_pending = false;
  sh::CameraDev hist_cam{};
  uint32_t hist_w = 0, hist_h = 0;
  DeviceBuffer prev;  // the targets as the previous view left them (36 B per pixel)
  const float4* denoised = nullptr;  // result of the last lucent_renderer_denoise, or null
  // ray capture (lucent_renderer_capture_rays): bounces, rays per region, records and queue lengths
  uint32_t cap_mask = 0, cap_rays = 0;
  DeviceBuffer cap, cap_count;
};

static AccumDev accum_of(lucent_renderer* r) {
  return {(float4*)r->color.ptr, (half4*)r->albedo.ptr, (half4*)r->normal.ptr, (float*)r->history.ptr};
}

static lucent_status alloc_targets(lucent_renderer* r, uint32_t w, uint32_t h) {
  const size_t n = (size_t)w * h;
  lucent_status st;
  if ((st = r->color.reserve(n * 16)) || (st = r->albedo.reserve(n * 8)) || (st = r->normal.reserve(n * 8)) ||
      (st = r->history.reserve(n * 4)))
    return st;
  r->W = w;
  r->H = h;
  k_clear_accum<<<grid_for((uint32_t)n, 256), 256>>>(accum_of(r), (uint32_t)n);
  r->frame = 0;
  r->denoised = nullptr;
  r->has_history = r->reproject_pending = false;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LUCENT_OK : cuda_fail(e, "clear targets");
}

// Path buffers for `cap` paths (bytes per path: the 128-byte path record, the
// hit, 3 shadow slots of 3 float4 (ray origin + tMax, direction + key,
// contribution + unoccluded flag), queues, slow-path queues, the sort key,
// the ray streams, the sorted and textured-hit queues).
// cudaMemset runs on the legacy default stream, which does not order itself
// with non-blocking streams (a batch's parts, the side streams): wait for it
// before any stream's kernels may touch the memory.
static cudaError_t clear_now(void* p, size_t bytes) {
  cudaError_t e = cudaMemset(p, 0, bytes);
  return e == cudaSuccess ? cudaStreamSynchronize(0) : e;
}

static lucent_status alloc_path_buffers(DeviceBuffer& paths, DeviceBuffer& ctr, uint32_t& path_cap, Paths& P,
                                        uint32_t cap) {
  if (cap <= path_cap) return LUCENT_OK;
  // Per-path arrays in allocation order (bytes per path); each starts on a 256-byte boundary.
  static const size_t kPer[] = {16 * kPathRecord, 16, 48, 48, 48, 4, 4, 12, 4, 12, 4, 32, 32, 4, 4};
  size_t total = 0;
  for (size_t b : kPer) total += ((size_t)cap * b + 255) & ~(size_t)255;
  total += (size_t)kSortBins * 4;
  lucent_status st = paths.reserve(total);
  if (st) return st;
  if ((st = ctr.reserve(kCtrWords * 4))) return st;
  char* b = (char*)paths.ptr;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char* p = b + off;
    off += (bytes + 255) & ~(size_t)255;
    return (void*)p;
  };
  P.rec = (float4*)take((size_t)cap * 16 * kPathRecord);
  P.ro = {P.rec};
  P.rd = {P.rec + 1};
  P.thr = {P.rec + 2};
  P.tint = {P.rec + 3};
  P.galb = {P.rec + 4};
  P.gnrm = {P.rec + 5};
  P.gpos = {P.rec + 6};
  P.rad = {P.rec + 7};
  P.hit = (float4*)take((size_t)cap * 16);
  P.sh_o = (float4*)take((size_t)cap * 48);
  P.sh_d = (float4*)take((size_t)cap * 48);
  P.sh_c = (float4*)take((size_t)cap * 48);
  P.q[0] = (uint32_t*)take((size_t)cap * 4);
  P.q[1] = (uint32_t*)take((size_t)cap * 4);
  P.qs = (uint32_t*)take((size_t)cap * 12);
  P.slow = (uint32_t*)take((size_t)cap * 4);
  P.slow2 = (uint32_t*)take((size_t)cap * 12);
  P.sort_keys = (uint32_t*)take((size_t)cap * 4);
  P.nray = (float4*)take((size_t)cap * 32);
  P.sray = (float4*)take((size_t)cap * 32);
  P.sort_tmp = (uint32_t*)take((size_t)cap * 4);
  P.qtex = (uint32_t*)take((size_t)cap * 4);
  P.sort_hist = (uint32_t*)take((size_t)kSortBins * 4);
  if (off > paths.cap) return fail(LUCENT_ERR_DEVICE, "path buffer layout overflow");
  P.ctr = (uint32_t*)ctr.ptr;
  cudaError_t e = clear_now(P.sh_c, (size_t)cap * 48);
  if (e == cudaSuccess) e = clear_now(P.ctr, kCtrWords * 4);
  if (e != cudaSuccess) return cuda_fail(e, "clear path buffers");
  path_cap = cap;
  return LUCENT_OK;
}

lucent_status WaveSet::reserve(uint32_t cap) {
  lucent_status st = alloc_path_buffers(paths, ctr, path_cap, P, cap);
  if (st || cap <= sid_cap) return st;
  if ((st = sid.reserve((size_t)cap * 2))) return st;
  if (clear_now(sid.ptr, (size_t)cap * 2) != cudaSuccess) return cuda_fail(cudaGetLastError(), "clear sid");
  sid_cap = cap;
  return LUCENT_OK;
}

// Orders stream s after every wave of r in flight: the accumulations stay in
// call order, and a set's buffers are reused only after its wave is done.
static void after_waves(lucent_renderer* r, cudaStream_t s) {
  for (WaveSet& w : r->set)
    if (w.used) cudaStreamWaitEvent(s, w.done, 0);
}

// Calls that change what a wave reads (geometry, materials, lighting) wait for
// the waves in flight, which run on streams of their own, and return only
// once the change is on the device, so a later wave needs no wait for it.
static lucent_status settle(const char* what) {
  cudaError_t e = cudaDeviceSynchronize();
  return e == cudaSuccess ? LUCENT_OK : cuda_fail(e, what);
}

// buildTextureArrays (renderer.ts:314-333): every referenced image resampled
// into its layer of the sRGB or linear array, at one shared size.
static lucent_status load_textures(lucent_renderer* r, const lucent_scene_desc* d, cudaStream_t s) {
  r->tex_size = 0;
  r->color_layers = r->data_layers = 0;
  const uint32_t nc = d->color_layer_count, nd = d->data_layer_count;
  if (nc + nd == 0) return LUCENT_OK;
  std::vector<int32_t> used(d->color_layers, d->color_layers + nc);
  used.insert(used.end(), d->data_layers, d->data_layers + nd);
  const int size = texture_array_size(d->texture_width, d->texture_height, used.data(), (uint32_t)used.size());
  float lut[512], mid[255];
  texel_tables(lut, mid);
  std::vector<float> tables(lut, lut + 512);
  tables.insert(tables.end(), mid, mid + 255);
  const size_t layer_bytes = (size_t)size * size * 4;
  lucent_status st;
  if ((st = r->texel_lut.reserve(tables.size() * 4)) || (st = r->color_maps.reserve((nc ? nc : 1) * layer_bytes)) ||
      (st = r->data_maps.reserve((nd ? nd : 1) * layer_bytes)))
    return st;
  cudaError_t e = cudaMemcpy(r->texel_lut.ptr, tables.data(), tables.size() * 4, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "texel tables");
  const float* lut_d = (const float*)r->texel_lut.ptr;
  if ((st = build_texture_layers(d->texture_rgba8, d->texture_width, d->texture_height, d->color_layers, nc, size, true,
                                 lut_d, lut_d + 512, (uint8_t*)r->color_maps.ptr, s)) ||
      (st = build_texture_layers(d->texture_rgba8, d->texture_width, d->texture_height, d->data_layers, nd, size, false,
                                 lut_d, lut_d + 512, (uint8_t*)r->data_maps.ptr, s)))
    return st;
  r->tex_size = size;
  r->color_layers = nc;
  r->data_layers = nd;
  return LUCENT_OK;
}

// The renderer holding r's scene: r itself, or the source of a view.
static lucent_renderer* scene_owner(lucent_renderer* r) { return r->src ? r->src : r; }
static const lucent_renderer* scene_owner(const lucent_renderer* r) { return r->src ? r->src : r; }

static SceneRec scene_rec(const lucent_renderer* r) {
  SceneRec R{};
  const lucent_renderer* o = scene_owner(r);
  R.scene = {(const Node*)o->nodes.ptr, o->node_count, (const float4*)o->geo.ptr, (const float4*)o->attr.ptr,
             (const float4*)o->mats.ptr, (const float4*)o->spheres.ptr, (const int*)o->sph_mat.ptr,
             (const int*)o->sph_light.ptr, (int)o->sphere_count, (const float4*)o->lights.ptr, (int)o->light_count,
             r->ground_enabled ? o->ground_material : -1, r->ground_height, o->any_alpha,
             (const uchar4*)o->color_maps.ptr, (const uchar4*)o->data_maps.ptr, (const float*)o->texel_lut.ptr,
             o->tex_size, (const Node*)o->wide.ptr};
  R.light = r->light;
  R.cam = r->cam;
  R.accum = {(float4*)r->color.ptr, (half4*)r->albedo.ptr, (half4*)r->normal.ptr, (float*)r->history.ptr};
  R.W = (int)r->W;
  R.H = (int)r->H;
  R.max_bounces = (int)r->max_bounces;
  R.clamp = r->clamp;
  R.seed0 = r->seed;
  R.reproject = r->reproject_pending ? 1 : 0;
  if (R.reproject) {
    const size_t n = (size_t)r->hist_w * r->hist_h;
    char* b = (char*)r->prev.ptr;
    R.prev = {(float4*)b, (half4*)(b + n * 16), (half4*)(b + n * 24), (float*)(b + n * 32)};
    R.prev_cam = r->hist_cam;
    R.prev_w = (int)r->hist_w;
    R.prev_h = (int)r->hist_h;
  }
  return R;
}

// Before a trace that reprojects: copies the targets (the previous view's
// averages) aside, since the first sample reads them around each pixel while
// it writes the new averages in place.
static lucent_status prepare_reprojection(lucent_renderer* r, cudaStream_t s) {
  if (!r->reproject_pending) return LUCENT_OK;
  const size_t n = (size_t)r->W * r->H;
  if (r->hist_w != r->W || r->hist_h != r->H) {  // the targets were reallocated: nothing to reproject
    r->reproject_pending = false;
    return LUCENT_OK;
  }
  lucent_status st = r->prev.reserve(n * 36);
  if (st) return st;
  char* b = (char*)r->prev.ptr;
  cudaError_t e = cudaMemcpyAsync(b, r->color.ptr, n * 16, cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(b + n * 16, r->albedo.ptr, n * 8, cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(b + n * 24, r->normal.ptr, n * 8, cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(b + n * 32, r->history.ptr, n * 4, cudaMemcpyDeviceToDevice, s);
  return e == cudaSuccess ? LUCENT_OK : cuda_fail(e, "copy history");
}

// After a trace: the targets now hold this view's averages.
static void record_history(lucent_renderer* r) {
  r->has_history = true;
  r->reproject_pending = false;
  r->hist_cam = r->cam;
  r->hist_w = r->W;
  r->hist_h = r->H;
}

// The renderer as a launch of one scene on path set w: uploads its SceneRec
// (sample seed `seed0`; a pending reprojection only with `first`) and the
// path/pixel bases of a full wave of S samples and of a last wave of `tail`
// samples; fills M for the full wave.
static lucent_status single_launch(lucent_renderer* r, WaveSet& w, uint32_t S, uint32_t tail, uint32_t seed0,
                                   bool first, cudaStream_t s, MultiLaunch& M) {
  const uint32_t WH = r->W * r->H;
  lucent_status st = w.reserve(S * WH);
  if (st) return st;
  if ((st = w.rec.reserve(sizeof(SceneRec))) || (st = w.base.reserve(32))) return st;
  SceneRec rec = scene_rec(r);
  rec.seed0 = seed0;
  if (!first) rec.reproject = 0;
  const uint32_t bases[8] = {0, WH * S, 0, WH, 0, WH * tail, 0, WH};
  // pageable host-to-device copies are staged before the call returns, so the locals may go
  cudaError_t e = cudaMemcpyAsync(w.rec.ptr, &rec, sizeof rec, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(w.base.ptr, bases, sizeof bases, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "upload scene record");
  M = MultiLaunch{};
  M.paths = w.P;
  M.recs = (SceneRec*)w.rec.ptr;
  M.path_base = (const uint32_t*)w.base.ptr;
  M.pix_base = M.path_base + 2;
  M.sid = (uint16_t*)w.sid.ptr;
  M.n = 1;
  M.S = (int)S;
  M.max_bounces = (int)r->max_bounces;
  M.total_paths = WH * S;
  M.total_pixels = WH;
  M.any_alpha = scene_owner(r)->any_alpha;
  M.sort_rays = r->sort_rays;
  M.top_levels = r->top_levels;
  M.wide = r->wide_bvh;
  M.sort_classes = 1;
  M.any_tex = scene_owner(r)->tex_size > 0;
  if (r->cap_mask) {
    M.cap_mask = r->cap_mask;
    M.cap = (float4*)r->cap.ptr;
    M.cap_count = (uint32_t*)r->cap_count.ptr;
    M.cap_stride = r->cap_rays;
  }
  if (lucent_status st = w.side.ensure()) return st;
  w.side.set(M);
  return LUCENT_OK;
}

// Switches M to the last wave of `tail` samples.
static void single_tail(lucent_renderer* r, const WaveSet& w, uint32_t tail, MultiLaunch& M) {
  M.S = (int)tail;
  M.total_paths = r->W * r->H * tail;
  M.path_base = (const uint32_t*)w.base.ptr + 4;
  M.pix_base = M.path_base + 2;
}

extern "C" {

lucent_status lucent_renderer_create(uint32_t width, uint32_t height, lucent_renderer** out) {
  clear_error();
  if (!out) return fail(LUCENT_ERR_INVALID, "null argument");
  *out = nullptr;
  if (width == 0 || height == 0 || (uint64_t)width * height > (1u << 26))
    return fail(LUCENT_ERR_INVALID, "bad size %ux%u", width, height);
  lucent_renderer* r = new lucent_renderer();
  lucent_status st = alloc_targets(r, width, height);
  if (!st) st = r->sheen.reserve(256 * 4);
  if (!st) {
    float lut[256];
    sheen_lut_half(lut);
    cudaError_t e = cudaMemcpy(r->sheen.ptr, lut, sizeof lut, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaEventCreate(&r->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&r->ev1);
    if (e != cudaSuccess) st = cuda_fail(e, "renderer setup");
  }
  if (st) {
    lucent_renderer_destroy(r);
    return st;
  }
  r->light.sheen_lut = (const float*)r->sheen.ptr;
  *out = r;
  return LUCENT_OK;
}

lucent_status lucent_renderer_create_view(lucent_renderer* src, uint32_t width, uint32_t height, lucent_renderer** out) {
  clear_error();
  if (!src || !out) return fail(LUCENT_ERR_INVALID, "null argument");
  *out = nullptr;
  src = scene_owner(src);  // a view of a view renders the same scene
  if (!src->has_scene) return fail(LUCENT_ERR_INVALID, "create_view before the source's load_scene");
  lucent_renderer* r = nullptr;
  lucent_status st = lucent_renderer_create(width, height, &r);
  if (st) return st;
  r->src = src;
  src->n_views++;
  *out = r;
  return LUCENT_OK;
}

void lucent_renderer_destroy(lucent_renderer* r) {
  if (!r) return;
  cudaDeviceSynchronize();  // waves in flight on the renderer's own streams read its buffers
  if (r->src) r->src->n_views--;
  for (DeviceBuffer* b : {&r->nodes, &r->wide, &r->geo, &r->attr, &r->mats, &r->spheres, &r->sph_mat, &r->sph_light,
                          &r->lights, &r->env_rgb, &r->env_alias, &r->sheen, &r->color, &r->albedo, &r->normal,
                          &r->history, &r->den_a, &r->den_b, &r->guide0, &r->guide1, &r->disp, &r->adj_dl, &r->adj_path, &r->adj_grad, &r->prev,
                          &r->color_maps, &r->data_maps, &r->texel_lut})
    b->release();
  for (WaveSet& w : r->set) w.destroy();
  if (r->ev0) cudaEventDestroy(r->ev0);
  if (r->ev1) cudaEventDestroy(r->ev1);
  for (cudaEvent_t e : r->pev) cudaEventDestroy(e);
  delete r;
}

static lucent_status upload(DeviceBuffer& b, const void* src, size_t bytes) {
  lucent_status st = b.reserve(bytes ? bytes : 16);
  if (st) return st;
  if (!bytes) return LUCENT_OK;
  cudaError_t e = cudaMemcpy(b.ptr, src, bytes, cudaMemcpyHostToDevice);
  return e == cudaSuccess ? LUCENT_OK : cuda_fail(e, "upload");
}

lucent_status lucent_renderer_load_scene(lucent_renderer* r, const lucent_scene_desc* d) {
  clear_error();
  if (!r || !d) return fail(LUCENT_ERR_INVALID, "null argument");
  if (r->n_views > 0) return fail(LUCENT_ERR_INVALID, "renderer has %d views of its scene", r->n_views);
  if (r->src) {  // a view loading a scene of its own stops being a view
    r->src->n_views--;
    r->src = nullptr;
  }
  const uint32_t n = d->tri_count;
  if (n && (!d->positions || !d->normals || !d->tri_material))
    return fail(LUCENT_ERR_INVALID, "triangles need positions, normals and material ids");
  if (n > (1u << 23)) return fail(LUCENT_ERR_UNSUPPORTED, "%u triangles; the limit is 2^23", n);
  if (d->sphere_count > 64) return fail(LUCENT_ERR_INVALID, "scene has %u spheres; max is 64", d->sphere_count);
  if (d->light_count > 8) return fail(LUCENT_ERR_INVALID, "scene has %u lights; max is 8", d->light_count);
  if (lucent_status st = settle("load scene")) return st;
  if (d->material_count == 0 || !d->materials) return fail(LUCENT_ERR_INVALID, "scene has no materials");
  const uint32_t M = d->material_count;
  // Map fields hold layer indices: base colour and emissive into the colour
  // array, metal-rough and normal into the data array (scene.ts:271-283).
  for (uint32_t m = 0; m < M; m++)
    for (int k = 16; k < 20; k++) {
      const float v = d->materials[m * 40 + k];
      const uint32_t layers = (k == 16 || k == 19) ? d->color_layer_count : d->data_layer_count;
      if (v >= 0 && !(v < (float)layers && v == std::floor(v)))
        return fail(LUCENT_ERR_INVALID, "material %u map %d is layer %g of %u", m, k - 16, v, layers);
    }
  if (d->color_layer_count + d->data_layer_count > 0) {
    if (!d->texture_rgba8 || !d->texture_width || !d->texture_height)
      return fail(LUCENT_ERR_INVALID, "texture layers without textures");
    for (int a = 0; a < 2; a++) {
      const int32_t* L = a ? d->data_layers : d->color_layers;
      const uint32_t n_l = a ? d->data_layer_count : d->color_layer_count;
      if (n_l && !L) return fail(LUCENT_ERR_INVALID, "null layer list");
      for (uint32_t i = 0; i < n_l; i++) {
        const int32_t t = L[i];
        if (t < 0 || (uint32_t)t >= d->texture_count)  // scene.ts:281-283
          return fail(LUCENT_ERR_INVALID, "material references texture %d, scene has %u", t, d->texture_count);
        if (!d->texture_rgba8[t] || d->texture_width[t] == 0 || d->texture_height[t] == 0 ||
            (uint64_t)d->texture_width[t] * d->texture_height[t] > (1ull << 28))
          return fail(LUCENT_ERR_INVALID, "texture %d is empty or too large", t);
      }
    }
  }
  for (uint32_t i = 0; i < n; i++) {
    if (d->tri_material[i] < 0 || (uint32_t)d->tri_material[i] >= M)
      return fail(LUCENT_ERR_INVALID, "triangle %u has material %d", i, d->tri_material[i]);
    if (d->tri_light && (d->tri_light[i] < -1 || d->tri_light[i] >= (int32_t)d->light_count))
      return fail(LUCENT_ERR_INVALID, "triangle %u has light %d", i, d->tri_light[i]);
  }
  for (uint32_t i = 0; i < d->sphere_count; i++) {
    if (d->sphere_materials[i] < 0 || (uint32_t)d->sphere_materials[i] >= M)
      return fail(LUCENT_ERR_INVALID, "sphere %u has material %d", i, d->sphere_materials[i]);
    if (d->sphere_lights && (d->sphere_lights[i] < -1 || d->sphere_lights[i] >= (int32_t)d->light_count))
      return fail(LUCENT_ERR_INVALID, "sphere %u has light %d", i, d->sphere_lights[i]);
  }
  if (d->ground_material >= (int32_t)M) return fail(LUCENT_ERR_INVALID, "ground material %d", d->ground_material);
  for (uint64_t i = 0; i < (uint64_t)n * 9; i++)
    if (!std::isfinite(d->positions[i])) return fail(LUCENT_ERR_UNSUPPORTED, "positions[%llu] is not finite", (unsigned long long)i);
  if (d->bvh_nodes) {
    if (!d->bvh_tri_indices) return fail(LUCENT_ERR_INVALID, "prebuilt BVH without triIndices");
    lucent_status st = validate_bvh(d->bvh_nodes, d->bvh_node_count, d->bvh_tri_indices, n);
    if (st) return st;
  }
  cudaStream_t s = 0;
  DeviceBuffer pos, nrm, uvs, mat, lgt, alp, idx;
  auto cleanup = [&](lucent_status st) {
    for (DeviceBuffer* b : {&pos, &nrm, &uvs, &mat, &lgt, &alp, &idx}) b->release();
    return st;
  };
  lucent_status st;
  if ((st = upload(pos, d->positions, (size_t)n * 36)) || (st = upload(nrm, d->normals, (size_t)n * 36)) ||
      (st = upload(mat, d->tri_material, (size_t)n * 4)))
    return cleanup(st);
  if (d->uvs && (st = upload(uvs, d->uvs, (size_t)n * 24))) return cleanup(st);
  if (d->tri_light && (st = upload(lgt, d->tri_light, (size_t)n * 4))) return cleanup(st);
  if (d->tri_alpha && (st = upload(alp, d->tri_alpha, (size_t)n))) return cleanup(st);
  std::vector<float> ref;
  std::vector<uint32_t> tri;
  double bounds[6];
  if (d->bvh_nodes) {
    ref.assign(d->bvh_nodes, d->bvh_nodes + (size_t)d->bvh_node_count * 8);
    tri.assign(d->bvh_tri_indices, d->bvh_tri_indices + n);
    DeviceBuffer rb;
    if ((st = upload(rb, ref.data(), ref.size() * 4)) || (st = r->nodes.reserve((size_t)d->bvh_node_count * 32))) {
      rb.release();
      return cleanup(st);
    }
    launch_pack_nodes((const float*)rb.ptr, d->bvh_node_count, (Node*)r->nodes.ptr, s);
    cudaStreamSynchronize(s);
    rb.release();
  } else {
    if ((st = gpu_build_bvh((const float*)pos.ptr, n, 4, 12, s, ref, tri, bounds, &r->nodes, nullptr)))
      return cleanup(st);
  }
  const uint32_t nc = (uint32_t)(ref.size() / 8);
  if (tree_depth(ref.data(), nc, n) + 2 > kTsStack)
    return cleanup(fail(LUCENT_ERR_UNSUPPORTED, "BVH deeper than the reference's 64-entry traversal stack"));
  if ((st = r->wide.reserve((size_t)nc * 4 * sizeof(Node)))) return cleanup(st);
  launch_wide_view((const Node*)r->nodes.ptr, nc, (Node*)r->wide.ptr, s);
  if ((st = upload(idx, tri.data(), (size_t)n * 4)) || (st = r->geo.reserve((size_t)(n ? n : 1) * 48)) ||
      (st = r->attr.reserve((size_t)(n ? n : 1) * 64)))
    return cleanup(st);
  if (n)
    k_pack_scene<<<grid_for(n, 256), 256, 0, s>>>((const float*)pos.ptr, (const float*)nrm.ptr,
                                                   d->uvs ? (const float*)uvs.ptr : nullptr, (const int32_t*)mat.ptr,
                                                   d->tri_light ? (const int32_t*)lgt.ptr : nullptr,
                                                   d->tri_alpha ? (const uint8_t*)alp.ptr : nullptr,
                                                   (const uint32_t*)idx.ptr, n, (float4*)r->geo.ptr,
                                                   (float4*)r->attr.ptr);
  if ((st = upload(r->mats, d->materials, (size_t)M * 160))) return cleanup(st);
  std::vector<float> sph(256 * 4, 0.f);
  std::vector<int32_t> sm(64, 0), sl(64, -1);
  for (uint32_t i = 0; i < d->sphere_count; i++) {
    for (int k = 0; k < 4; k++) sph[i * 4 + k] = d->spheres[i * 4 + k];
    sm[i] = d->sphere_materials[i];
    sl[i] = d->sphere_lights ? d->sphere_lights[i] : -1;
  }
  std::vector<float> lts(8 * 16, 0.f);
  if (d->light_count) std::memcpy(lts.data(), d->lights, (size_t)d->light_count * 64);
  if ((st = upload(r->spheres, sph.data(), sph.size() * 4)) || (st = upload(r->sph_mat, sm.data(), 256)) ||
      (st = upload(r->sph_light, sl.data(), 256)) || (st = upload(r->lights, lts.data(), lts.size() * 4)))
    return cleanup(st);
  int any_alpha = 0;
  if (d->tri_alpha)
    for (uint32_t i = 0; i < n && !any_alpha; i++) any_alpha = d->tri_alpha[i] != 0;
  cudaError_t e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return cleanup(cuda_fail(e, "scene upload"));
  if ((st = load_textures(r, d, s))) return cleanup(st);
  r->node_count = nc;
  r->tri_count = n;
  r->material_count = M;
  r->sphere_count = d->sphere_count;
  r->light_count = d->light_count;
  r->ground_material = d->ground_material;
  r->any_alpha = any_alpha;
  r->has_scene = true;
  cleanup(LUCENT_OK);
  if ((st = settle("load scene"))) return st;
  return lucent_renderer_reset(r);
}

lucent_status lucent_renderer_upload_lighting(lucent_renderer* r, const lucent_lighting* l) {
  clear_error();
  if (!r || !l) return fail(LUCENT_ERR_INVALID, "null argument");
  if (!l->env_rgb || l->env_width == 0 || l->env_height == 0) return fail(LUCENT_ERR_INVALID, "lighting needs an environment map");
  const size_t texels = (size_t)l->env_width * l->env_height;
  for (size_t i = 0; i < texels * 3; i++)
    if (!(l->env_rgb[i] >= 0) || !std::isfinite(l->env_rgb[i]))
      return fail(LUCENT_ERR_INVALID, "environment texel %zu is negative or not finite", i / 3);
  uint32_t gw, gh;
  std::vector<float> table;
  double total;
  if (!env_sampler(l->env_rgb, l->env_width, l->env_height, 1024, gw, gh, table, total))
    return fail(LUCENT_ERR_INVALID, "environment sampler failed");
  lucent_status st;
  if ((st = settle("upload lighting")) || (st = upload(r->env_rgb, l->env_rgb, texels * 12)) ||
      (st = upload(r->env_alias, table.data(), table.size() * 4)) || (st = settle("upload lighting")))
    return st;
  sh::LightingDev& L = r->light;
  L.sun_enabled = l->sun_enabled;
  L.sun_dir = make_float3(l->sun_dir[0], l->sun_dir[1], l->sun_dir[2]);
  L.sun_radiance = make_float3(l->sun_radiance[0], l->sun_radiance[1], l->sun_radiance[2]);
  L.sun_cos = l->sun_cos_angle;
  L.sun_pdf = l->sun_pdf;
  L.env_rgb = (const float*)r->env_rgb.ptr;
  L.env_w = (int)l->env_width;
  L.env_h = (int)l->env_height;
  L.env_alias = (const float4*)r->env_alias.ptr;
  L.grid_w = (int)gw;
  L.grid_h = (int)gh;
  L.env_cos = l->env_rotation_cos;
  L.env_sin = l->env_rotation_sin;
  L.env_intensity = l->env_intensity;
  L.env_sampling = total > 0 ? 1 : 0;  // renderer.ts:412
  L.env_background = l->env_background;
  L.backdrop = make_float3(l->backdrop[0], l->backdrop[1], l->backdrop[2]);
  L.sheen_lut = (const float*)r->sheen.ptr;
  r->has_lighting = true;
  return lucent_renderer_reset(r);
}

// The environment map from host or device memory, its sampler built on the GPU.
static lucent_status set_env_gpu(lucent_renderer* r, const float* rgb, bool on_device, uint32_t width,
                                 uint32_t height, cudaStream_t s) {
  if (!r || !rgb || width == 0 || height == 0) return fail(LUCENT_ERR_INVALID, "null argument or empty map");
  if (!r->has_lighting) return fail(LUCENT_ERR_INVALID, "set_env before upload_lighting");
  const size_t texels = (size_t)width * height;
  uint32_t gw, gh;
  env_grid(width, height, 1024, gw, gh);
  lucent_status st = settle("set environment");
  if (!st) st = r->env_rgb.reserve(texels * 12);
  if (!st) st = r->env_alias.reserve((size_t)gw * gh * 16);
  if (st) return st;
  cudaError_t e = cudaMemcpyAsync(r->env_rgb.ptr, rgb, texels * 12,
                                  on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "copy environment map");
  double total = 0;
  if ((st = gpu_env_sampler((const float*)r->env_rgb.ptr, width, height, 1024, gw, gh, (float4*)r->env_alias.ptr,
                            total, s)))
    return st;
  sh::LightingDev& L = r->light;
  L.env_rgb = (const float*)r->env_rgb.ptr;
  L.env_w = (int)width;
  L.env_h = (int)height;
  L.env_alias = (const float4*)r->env_alias.ptr;
  L.grid_w = (int)gw;
  L.grid_h = (int)gh;
  L.env_sampling = total > 0 ? 1 : 0;  // renderer.ts:412
  if ((st = settle("set environment"))) return st;
  return lucent_renderer_reset(r);
}

lucent_status lucent_renderer_set_env_device(lucent_renderer* r, const float* rgb_d, uint32_t width, uint32_t height,
                                            void* stream) {
  clear_error();
  return set_env_gpu(r, rgb_d, true, width, height, (cudaStream_t)stream);
}

lucent_status lucent_renderer_set_env(lucent_renderer* r, const float* rgb, uint32_t width, uint32_t height,
                                     void* stream) {
  clear_error();
  return set_env_gpu(r, rgb, false, width, height, (cudaStream_t)stream);
}

lucent_status lucent_renderer_upload_ground(lucent_renderer* r, int32_t enabled, float height) {
  clear_error();
  if (!r) return fail(LUCENT_ERR_INVALID, "null renderer");
  r->ground_enabled = enabled;
  r->ground_height = height;
  return lucent_renderer_reset(r);
}

lucent_status lucent_renderer_upload_camera(lucent_renderer* r, const lucent_camera* c) {
  clear_error();
  if (!r || !c) return fail(LUCENT_ERR_INVALID, "null argument");
  r->cam.pos = make_float3(c->position[0], c->position[1], c->position[2]);
  r->cam.right = make_float3(c->right[0], c->right[1], c->right[2]);
  r->cam.up = make_float3(c->up[0], c->up[1], c->up[2]);
  r->cam.forward = make_float3(c->forward[0], c->forward[1], c->forward[2]);
  r->cam.tan_half_fov = c->tan_half_fov;
  r->cam.aperture = c->aperture;
  r->cam.focus = c->focus_distance;
  // invalidateView (renderer.ts:441-451): keep the history for reprojection if allowed, else start over
  if (r->temporal && r->has_history && r->frame > 0) {
    r->reproject_pending = true;
    r->frame = std::min(r->frame, (uint32_t)kHistoryCap);
    r->denoised = nullptr;
    return LUCENT_OK;
  }
  return lucent_renderer_reset(r);
}

lucent_status lucent_renderer_apply_settings(lucent_renderer* r, const lucent_settings* s) {
  clear_error();
  if (!r || !s) return fail(LUCENT_ERR_INVALID, "null argument");
  if (s->max_bounces > 64) return fail(LUCENT_ERR_INVALID, "max_bounces %u", s->max_bounces);
  r->max_bounces = s->max_bounces;
  r->clamp = s->firefly_clamp;
  r->temporal = s->temporal ? 1 : 0;
  return LUCENT_OK;
}

lucent_status lucent_renderer_resize(lucent_renderer* r, uint32_t w, uint32_t h) {
  clear_error();
  if (!r || w == 0 || h == 0 || (uint64_t)w * h > (1u << 26)) return fail(LUCENT_ERR_INVALID, "bad size");
  return alloc_targets(r, w, h);
}

lucent_status lucent_renderer_reset(lucent_renderer* r) {
  clear_error();
  if (!r) return fail(LUCENT_ERR_INVALID, "null renderer");
  const uint32_t n = r->W * r->H;
  k_clear_accum<<<grid_for(n, 256), 256>>>(accum_of(r), n);
  r->kernel_launches++;
  r->frame = 0;
  r->denoised = nullptr;
  r->has_history = r->reproject_pending = false;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LUCENT_OK : cuda_fail(e, "reset");
}

lucent_status lucent_renderer_set_seed(lucent_renderer* r, uint32_t seed) {
  clear_error();
  if (!r) return fail(LUCENT_ERR_INVALID, "null renderer");
  r->seed = seed;
  return LUCENT_OK;
}

lucent_status lucent_renderer_trace(lucent_renderer* r, uint32_t samples, void* stream) {
  clear_error();
  if (!r) return fail(LUCENT_ERR_INVALID, "null renderer");
  if (!scene_owner(r)->has_scene || !r->has_lighting)
    return fail(LUCENT_ERR_INVALID, "trace before load_scene / upload_lighting");
  if (samples == 0) return LUCENT_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const uint32_t WH = r->W * r->H;
  const uint32_t max_paths = 1u << 23;
  const uint32_t batch = std::max(1u, std::min(samples, max_paths / std::max(1u, WH)));
  const uint32_t full = samples / batch, tail = samples % batch;
  MultiLaunch M{};
  after_waves(r, s);  // the previous traces' accumulations first (the reprojection copies their result)
  lucent_status st = prepare_reprojection(r, s);
  if (st) return st;
  // Profiling (phase events on one stream, traversal counters) and ray
  // capture keep every wave on the caller's stream, in path set 0.
  const bool pipelined = r->pipeline && !r->profiling && !r->cap_mask && !r->trav_counters;
  if (pipelined) {
    for (uint32_t w = 0; w < full + (tail ? 1 : 0); w++) {
      WaveSet& X = r->set[r->next_set];
      r->next_set ^= 1;
      if ((st = X.ensure())) return st;
      // The set's previous wave is accumulated (its buffers and record are free).
      if (X.used) cudaStreamWaitEvent(X.stream, X.done, 0);
      const uint32_t S = w < full ? batch : tail;
      if ((st = single_launch(r, X, S, 0, r->seed + w * batch, w == 0, X.stream, M))) return st;
      if (w == 0) cudaEventRecord(r->ev0, X.stream);
      // The first wave ever runs uncaptured (one-time setup).
      if (w < full && r->waves > 0) {
        uint64_t key[4];
        wave_key(M, key);
        key[0] |= 1ull << 63;  // captured without the accumulation
        if ((st = X.graph.run(M, key, X.stream, false))) return st;
        r->kernel_launches += X.graph.launches;
      } else {
        r->kernel_launches += render_wave_multi(M, X.stream, nullptr, false);
      }
      cudaEventRecord(X.traced, X.stream);
      cudaStreamWaitEvent(s, X.traced, 0);
      r->kernel_launches += accumulate_wave(M, s);
      cudaEventRecord(X.done, s);
      X.used = true;
      r->waves++;
    }
  } else {
    WaveSet& X = r->set[0];
    if ((st = X.ensure()) || (st = single_launch(r, X, batch, tail, r->seed, true, s, M))) return st;
    M.trav_stats = r->trav_counters ? (unsigned long long*)((uint32_t*)X.ctr.ptr + kCtrTrav) : nullptr;
    cudaEventRecord(r->ev0, s);
    PhaseEvents pe{r->pev.data(), r->ptag.data(), (int)r->pev.size(), 0};
    uint64_t key[4];
    wave_key(M, key);
    for (uint32_t w = 0; w < full + (tail ? 1 : 0); w++) {
      if (w == full) single_tail(r, X, tail, M);
      // The first wave ever runs uncaptured (one-time setup); profiling and ray
      // capture launch directly.
      if (w < full && !r->profiling && !r->cap_mask && r->waves > 0) {
        if ((st = X.graph.run(M, key, s))) return st;
        r->kernel_launches += X.graph.launches;
      } else {
        r->kernel_launches += render_wave_multi(M, s, r->profiling ? &pe : nullptr);  // seeds advance on the device
      }
      r->waves++;
    }
    cudaEventRecord(X.done, s);
    X.used = true;
    r->pn = pe.n;
  }
  r->seed += samples;
  r->frame += samples;
  record_history(r);
  cudaEventRecord(r->ev1, s);
  r->timed = true;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LUCENT_OK : cuda_fail(e, "trace launch");
}

lucent_status lucent_renderer_set_materials(lucent_renderer* r, const float* materials, uint32_t count) {
  clear_error();
  if (!r || !materials) return fail(LUCENT_ERR_INVALID, "null argument");
  lucent_renderer* o = scene_owner(r);  // a view's materials are its source's (shared)
  if (!o->has_scene) return fail(LUCENT_ERR_INVALID, "set_materials before load_scene");
  if (count != o->material_count)
    return fail(LUCENT_ERR_INVALID, "scene has %u materials, got %u", o->material_count, count);
  for (size_t i = 0; i < (size_t)count * 40; i++)
    if (!std::isfinite(materials[i])) return fail(LUCENT_ERR_INVALID, "material value %zu is not finite", i);
  if (lucent_status st = settle("upload materials")) return st;
  cudaError_t e = cudaMemcpy(o->mats.ptr, materials, (size_t)count * 160, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "upload materials");
  if (lucent_status st = settle("upload materials")) return st;
  return lucent_renderer_reset(r);
}

lucent_status lucent_renderer_backward(lucent_renderer* r, uint32_t samples, uint32_t seed, const float* dl_dimage,
                                       float* d_materials, float* d_env, void* stream) {
  clear_error();
  if (!r || !dl_dimage || !d_materials) return fail(LUCENT_ERR_INVALID, "null argument");
  if (!scene_owner(r)->has_scene || !r->has_lighting)
    return fail(LUCENT_ERR_INVALID, "backward before load_scene / upload_lighting");
  // The parameters are the material factors; with maps the BSDF sees factor x texel.
  if (scene_owner(r)->tex_size > 0) return fail(LUCENT_ERR_UNSUPPORTED, "backward through texture-mapped materials");
  if (samples == 0) return LUCENT_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const uint32_t WH = r->W * r->H;
  const uint32_t max_paths = 1u << 23;
  const uint32_t batch = std::max(1u, std::min(samples, max_paths / std::max(1u, WH)));
  WaveSet& X = r->set[0];
  lucent_status st = X.reserve(batch * WH);
  if (st) return st;
  const size_t cap = X.path_cap;
  const size_t nmat = (size_t)scene_owner(r)->material_count * 6;
  const size_t texels = d_env ? (size_t)r->light.env_w * r->light.env_h : 0;
  const size_t env_off = (nmat + 3) & ~(size_t)3;  // the env gradients: float4 per texel, 16-byte aligned
  const size_t nenv = texels * 4;
  // per path: lrem 1 + gcont 5 + genv 2 float4; per shadow slot: gslot 2 float4 (3 slots per path)
  if ((st = r->adj_dl.reserve((size_t)WH * 16)) || (st = r->adj_path.reserve(cap * 16 * (1 + 5 + 2 + 6))) ||
      (st = r->adj_grad.reserve((env_off + nenv) * 4 + 16)))
    return st;
  std::vector<float> dl((size_t)WH * 4);
  const float inv = 1.f / (float)samples;
  for (size_t i = 0; i < dl.size(); i++) {
    if (!std::isfinite(dl_dimage[i])) return fail(LUCENT_ERR_INVALID, "dl_dimage value %zu is not finite", i);
    dl[i] = dl_dimage[i] * inv;
  }
  after_waves(r, s);
  cudaError_t e = cudaMemcpyAsync(r->adj_dl.ptr, dl.data(), dl.size() * 4, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(r->adj_grad.ptr, 0, (env_off + nenv) * 4, s);
  if (e != cudaSuccess) return cuda_fail(e, "backward setup");
  float4* base = (float4*)r->adj_path.ptr;
  AdjointDevHost H{(const float4*)r->adj_dl.ptr, base, base + cap, base + 6 * cap, base + 12 * cap,
                   (float*)r->adj_grad.ptr, nenv ? (float*)r->adj_grad.ptr + env_off : nullptr};
  for (uint32_t done = 0; done < samples; done += batch) {
    const uint32_t S = std::min(batch, samples - done);
    MultiLaunch M{};
    if ((st = single_launch(r, X, S, 0, seed + done, true, s, M))) return st;
    render_backward(M, H, s);
  }
  std::vector<float> g(env_off + nenv);
  e = cudaMemcpyAsync(g.data(), r->adj_grad.ptr, g.size() * 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "backward");
  uint32_t word = 0;
  cudaMemcpy(&word, (uint32_t*)X.ctr.ptr + kCtrErr, 4, cudaMemcpyDeviceToHost);
  if (word) {
    clear_now((uint32_t*)X.ctr.ptr + kCtrErr, 4);
    return fail(LUCENT_ERR_DEVICE, "backward raised device error word 0x%x", word);
  }
  for (size_t i = 0; i < nmat; i++) d_materials[i] += g[i];
  for (size_t i = 0; i < texels; i++)
    for (int c = 0; c < 3; c++) d_env[3 * i + c] += g[env_off + 4 * i + c];
  return LUCENT_OK;
}

lucent_status lucent_renderer_set_ray_sort(lucent_renderer* r, int32_t enabled) {
  clear_error();
  if (!r) return fail(LUCENT_ERR_INVALID, "null renderer");
  r->sort_rays = enabled ? 1 : 0;
  return LUCENT_OK;
}

lucent_status lucent_renderer_read_textures(lucent_renderer* r, uint32_t* size, uint8_t* color_out, uint8_t* data_out) {
  clear_error();
  if (!r || !size) return fail(LUCENT_ERR_INVALID, "null argument");
  r = scene_owner(r);
  *size = (uint32_t)r->tex_size;
  const size_t layer = (size_t)r->tex_size * r->tex_size * 4;
  cudaError_t e = cudaSuccess;
  if (color_out && r->color_layers) e = cudaMemcpy(color_out, r->color_maps.ptr, r->color_layers * layer, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && data_out && r->data_layers)
    e = cudaMemcpy(data_out, r->data_maps.ptr, r->data_layers * layer, cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? LUCENT_OK : cuda_fail(e, "read textures");
}

lucent_status lucent_renderer_set_top_levels(lucent_renderer* r, int32_t enabled) {
  clear_error();
  if (!r) return fail(LUCENT_ERR_INVALID, "null renderer");
  r->top_levels = enabled ? 1 : 0;
  return LUCENT_OK;
}

lucent_status lucent_renderer_set_wide_bvh(lucent_renderer* r, int32_t enabled) {
  clear_error();
  if (!r) return fail(LUCENT_ERR_INVALID, "null renderer");
  r->wide_bvh = enabled ? 1 : 0;
  return LUCENT_OK;
}

lucent_status lucent_renderer_set_pipelining(lucent_renderer* r, int32_t enabled) {
  clear_error();
  if (!r) return fail(LUCENT_ERR_INVALID, "null renderer");
  r->pipeline = enabled ? 1 : 0;
  return LUCENT_OK;
}

lucent_status lucent_renderer_trim(lucent_renderer* r) {
  clear_error();
  if (!r) return fail(LUCENT_ERR_INVALID, "null renderer");
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return cuda_fail(e, "synchronize");
  for (WaveSet& w : r->set) w.release_paths();
  return LUCENT_OK;
}

lucent_status lucent_env_sampler(const float* rgb, uint32_t width, uint32_t height, uint32_t max_width, uint32_t* gw,
                                 uint32_t* gh, float* table, double* total) {
  clear_error();
  if (!rgb || !gw || !gh || width == 0 || height == 0 || max_width == 0)
    return fail(LUCENT_ERR_INVALID, "null argument or empty image");
  uint32_t a = 0, b = 0;
  double t = 0;
  std::vector<float> tab;
  if (!env_sampler(rgb, width, height, max_width, a, b, tab, t))
    return fail(LUCENT_ERR_INVALID, "environment weights must be finite and >= 0");
  *gw = a;
  *gh = b;
  if (total) *total = t;
  if (table) std::memcpy(table, tab.data(), tab.size() * sizeof(float));
  return LUCENT_OK;
}

lucent_status lucent_renderer_capture_rays(lucent_renderer* r, uint32_t bounce_mask, uint32_t max_rays) {
  clear_error();
  if (!r) return fail(LUCENT_ERR_INVALID, "null renderer");
  if (bounce_mask == 0 || max_rays == 0) {
    r->cap.release();
    r->cap_count.release();
    r->cap_mask = r->cap_rays = 0;
    return LUCENT_OK;
  }
  const uint32_t regions = 2u * (uint32_t)__builtin_popcount(bounce_mask);
  lucent_status st = r->cap.reserve((size_t)regions * max_rays * 64);
  if (!st) st = r->cap_count.reserve(64 * 4);
  if (st) return st;
  if (clear_now(r->cap_count.ptr, 64 * 4) != cudaSuccess) return cuda_fail(cudaGetLastError(), "clear capture");
  r->cap_mask = bounce_mask;
  r->cap_rays = max_rays;
  return LUCENT_OK;
}

lucent_status lucent_renderer_read_rays(lucent_renderer* r, uint32_t bounce, int32_t shadow, float* out16,
                                        uint32_t cap, uint32_t* count) {
  lucent_status st = lucent_renderer_check(r, nullptr);
  if (st) return st;
  if (!count) return fail(LUCENT_ERR_INVALID, "null argument");
  if (bounce >= 32 || !(r->cap_mask >> bounce & 1u)) return fail(LUCENT_ERR_INVALID, "bounce %u is not captured", bounce);
  const uint32_t region = 2u * (uint32_t)__builtin_popcount(r->cap_mask & ((1u << bounce) - 1u)) + (shadow ? 1u : 0u);
  uint32_t n = 0;
  cudaError_t e = cudaMemcpy(&n, (uint32_t*)r->cap_count.ptr + region, 4, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "read capture count");
  *count = n;
  const uint32_t m = std::min(std::min(n, cap), r->cap_rays);
  if (out16 && m) {
    e = cudaMemcpy(out16, (const char*)r->cap.ptr + (size_t)region * r->cap_rays * 64, (size_t)m * 64,
                   cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "read captured rays");
  }
  return LUCENT_OK;
}

lucent_status lucent_renderer_set_profiling(lucent_renderer* r, int32_t enabled) {
  clear_error();
  if (!r) return fail(LUCENT_ERR_INVALID, "null renderer");
  r->profiling = enabled != 0;
  r->trav_counters = enabled == 2;
  if (r->profiling && r->pev.empty()) {
    r->pev.resize(1024);
    r->ptag.resize(1024);
    for (cudaEvent_t& e : r->pev) {
      cudaError_t err = cudaEventCreate(&e);
      if (err != cudaSuccess) return cuda_fail(err, "profiling events");
    }
  }
  return LUCENT_OK;
}

lucent_status lucent_renderer_check(lucent_renderer* r, void* stream) {
  clear_error();
  if (!r) return fail(LUCENT_ERR_INVALID, "null renderer");
  after_waves(r, (cudaStream_t)stream);  // and so the waves themselves
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "synchronize");
  uint32_t word = 0;
  WaveSet* bad = nullptr;
  for (WaveSet& w : r->set) {
    if (!w.ctr.ptr || word) continue;
    e = cudaMemcpy(&word, (uint32_t*)w.ctr.ptr + kCtrErr, 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "read error word");
    if (word) bad = &w;
  }
  float ms = 0;
  if (r->timed && cudaEventElapsedTime(&ms, r->ev0, r->ev1) == cudaSuccess) r->last_ms = ms;
  if (r->profiling && r->pn > 1) {
    for (double& v : r->phase_ms) v = 0;
    for (int i = 1; i < r->pn; i++) {
      if (r->ptag[i] < 0) continue;
      float d = 0;
      if (cudaEventElapsedTime(&d, r->pev[i - 1], r->pev[i]) == cudaSuccess) r->phase_ms[r->ptag[i]] += d;
    }
    r->pn = 0;
  }
  if (word) {
    clear_now((uint32_t*)bad->ctr.ptr + kCtrErr, 4);
    return fail(LUCENT_ERR_DEVICE, "render raised device error word 0x%x", word);
  }
  return LUCENT_OK;
}

lucent_status lucent_renderer_read(lucent_renderer* r, float* color4, float* albedo4, float* normal4, float* history) {
  lucent_status st = lucent_renderer_check(r, nullptr);
  if (st) return st;
  const uint32_t n = r->W * r->H;
  cudaError_t e = cudaSuccess;
  if (color4) e = cudaMemcpy(color4, r->color.ptr, (size_t)n * 16, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && history) e = cudaMemcpy(history, r->history.ptr, (size_t)n * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && (albedo4 || normal4)) {
    DeviceBuffer tmp;
    if ((st = tmp.reserve((size_t)n * 32))) return st;
    float* a = (float*)tmp.ptr;
    float* b = a + (size_t)n * 4;
    k_unpack_accum<<<grid_for(n, 256), 256>>>(accum_of(r), n, albedo4 ? a : nullptr, normal4 ? b : nullptr);
    if (albedo4) e = cudaMemcpy(albedo4, a, (size_t)n * 16, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && normal4) e = cudaMemcpy(normal4, b, (size_t)n * 16, cudaMemcpyDeviceToHost);
    tmp.release();
  }
  return e == cudaSuccess ? LUCENT_OK : cuda_fail(e, "read targets");
}

lucent_status lucent_renderer_read_color_async(lucent_renderer* r, float* color4, void* stream) {
  clear_error();
  if (!r || !color4) return fail(LUCENT_ERR_INVALID, "null argument");
  after_waves(r, (cudaStream_t)stream);
  cudaError_t e = cudaMemcpyAsync(color4, r->color.ptr, (size_t)r->W * r->H * 16, cudaMemcpyDeviceToHost,
                                  (cudaStream_t)stream);
  return e == cudaSuccess ? LUCENT_OK : cuda_fail(e, "read colour target");
}

lucent_status lucent_renderer_denoise(lucent_renderer* r, uint32_t levels, float sigma_l, float sigma_n,
                                      float sigma_p, void* stream) {
  clear_error();
  if (!r) return fail(LUCENT_ERR_INVALID, "null renderer");
  if (levels > 5) return fail(LUCENT_ERR_INVALID, "at most 5 a-trous levels (steps 1, 2, 4, 8, 16)");
  const size_t n = (size_t)r->W * r->H;
  lucent_status st;
  if ((st = r->den_a.reserve(n * 16)) || (st = r->den_b.reserve(n * 16)) || (st = r->guide0.reserve(n * 16)) ||
      (st = r->guide1.reserve(n * 16)))
    return st;
  after_waves(r, (cudaStream_t)stream);  // the traces' accumulations, wherever they were queued
  r->denoised = denoise_run(accum_of(r), r->cam, (int)r->W, (int)r->H, (int)levels, sigma_l, sigma_n, sigma_p,
                            (float4*)r->den_a.ptr, (float4*)r->den_b.ptr, (float4*)r->guide0.ptr,
                            (float4*)r->guide1.ptr, (cudaStream_t)stream);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LUCENT_OK : cuda_fail(e, "denoise launch");
}

lucent_status lucent_renderer_read_denoised(lucent_renderer* r, float* out4) {
  lucent_status st = lucent_renderer_check(r, nullptr);
  if (st) return st;
  if (!out4) return fail(LUCENT_ERR_INVALID, "null output");
  if (!r->denoised) return fail(LUCENT_ERR_INVALID, "no denoised image since the last reset");
  cudaError_t e = cudaMemcpy(out4, r->denoised, (size_t)r->W * r->H * 16, cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? LUCENT_OK : cuda_fail(e, "read denoised");
}

lucent_status lucent_renderer_display(lucent_renderer* r, float denoise_weight, int32_t tonemap, float exposure,
                                      uint8_t* rgba8_out, float* rgb_out, void* stream) {
  clear_error();
  if (!r) return fail(LUCENT_ERR_INVALID, "null renderer");
  return lucent_renderer_display_view(r, r->W, r->H, denoise_weight, tonemap, exposure, rgba8_out, rgb_out, stream);
}

lucent_status lucent_renderer_display_view(lucent_renderer* r, uint32_t view_w, uint32_t view_h, float denoise_weight,
                                           int32_t tonemap, float exposure, uint8_t* rgba8_out, float* rgb_out,
                                           void* stream) {
  clear_error();
  if (!r) return fail(LUCENT_ERR_INVALID, "null renderer");
  if (view_w == 0 || view_h == 0 || (uint64_t)view_w * view_h > (1u << 26)) return fail(LUCENT_ERR_INVALID, "bad view size");
  if (tonemap < 0 || tonemap > 2) return fail(LUCENT_ERR_INVALID, "tonemap must be 0 (ACES), 1 (Reinhard) or 2 (none)");
  if (!(denoise_weight >= 0.f && denoise_weight <= 1.f)) return fail(LUCENT_ERR_INVALID, "denoise weight outside [0, 1]");
  if (denoise_weight > 0.f && !r->denoised)
    return fail(LUCENT_ERR_INVALID, "denoise weight > 0 with no denoised image since the last reset");
  const size_t n = (size_t)view_w * view_h;
  lucent_status st = r->disp.reserve(n * 16);
  if (st) return st;
  uchar4* d8 = (uchar4*)r->disp.ptr;
  float* drgb = (float*)((char*)r->disp.ptr + n * 4);
  cudaStream_t s = (cudaStream_t)stream;
  after_waves(r, s);
  display_run(accum_of(r), denoise_weight > 0.f ? r->denoised : nullptr, (int)r->W, (int)r->H, (int)view_w,
              (int)view_h, denoise_weight, exposure, tonemap, rgba8_out ? d8 : nullptr, rgb_out ? drgb : nullptr, s);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && rgba8_out) e = cudaMemcpyAsync(rgba8_out, d8, n * 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && rgb_out) e = cudaMemcpyAsync(rgb_out, drgb, n * 12, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? LUCENT_OK : cuda_fail(e, "display");
}

lucent_status lucent_renderer_stats(lucent_renderer* r, lucent_render_stats* out) {
  clear_error();
  if (!r || !out) return fail(LUCENT_ERR_INVALID, "null argument");
  std::memset(out, 0, sizeof *out);
  out->samples = r->frame;
  out->seed = r->seed;
  out->width = r->W;
  out->height = r->H;
  out->triangles = scene_owner(r)->tri_count;
  out->bvh_nodes = scene_owner(r)->node_count;
  for (WaveSet& w : r->set) {
    if (!w.ctr.ptr) continue;
    uint64_t c[2] = {0, 0};
    cudaError_t e = cudaMemcpy(c, (uint32_t*)w.ctr.ptr + kCtrStatClosest, 16, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "read stats");
    out->closest_rays += c[0];
    out->shadow_rays += c[1];
  }
  out->last_trace_ms = r->last_ms;
  out->kernel_launches = r->kernel_launches;
  for (int k = 0; k < kPhases; k++) out->phase_ms[k] = r->phase_ms[k];
  if (r->set[0].ctr.ptr) {  // profiling mode 2 traces in set 0
    cudaError_t e = cudaMemcpy(out->traversal, (uint32_t*)r->set[0].ctr.ptr + kCtrTrav, 40, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "read traversal counters");
  }
  return LUCENT_OK;
}

// ---------------------------------------------------------------------------
// Multi-scene batches: one wavefront over the paths of several renderers.
// ---------------------------------------------------------------------------
}  // extern "C"

struct lucent_batch {
  std::vector<lucent_renderer*> rs;
  lucent_batch_options opt{0, 1u << 25, 1, 0, 0, 1, 1, 1, 0, 1};
  // Pipelined as a renderer's waves: successive waves alternate between the
  // two sets, each traced on its set's stream, accumulated on the caller's.
  WaveSet set[2];
  int next_set = 0;
  std::vector<WaveGraph> graphs[2];  // per set: a captured full wave per group of scenes
  // opt.streams > 1: consecutive parts of the renderers traced as batches of
  // their own, side by side on their own streams
  std::vector<lucent_batch*> parts;
  std::vector<SideStream> part_streams;  // stream + done event per part (fork: part_streams[0].fork)
  uint32_t waves = 0, graph_waves = 0;
  uint64_t kernel_launches = 0;  // by its traces (lucent_batch_stats)
  void drop_graphs() {
    for (std::vector<WaveGraph>& gs : graphs)
      for (WaveGraph& g : gs) g.drop();
  }
  void destroy_graphs() {
    for (std::vector<WaveGraph>& gs : graphs) {
      for (WaveGraph& g : gs) g.destroy();
      gs.clear();
    }
  }
};


extern "C" {

lucent_status lucent_batch_create(lucent_renderer* const* renderers, uint32_t n, lucent_batch** out) {
  clear_error();
  if (!out || (!renderers && n)) return fail(LUCENT_ERR_INVALID, "null argument");
  *out = nullptr;
  if (n == 0 || n > 65535) return fail(LUCENT_ERR_INVALID, "a batch holds 1 to 65535 renderers, got %u", n);
  for (uint32_t i = 0; i < n; i++) {
    if (!renderers[i]) return fail(LUCENT_ERR_INVALID, "renderer %u is null", i);
    for (uint32_t j = 0; j < i; j++)
      if (renderers[j] == renderers[i]) return fail(LUCENT_ERR_INVALID, "renderer %u appears twice", i);
  }
  lucent_batch* b = new lucent_batch();
  b->rs.assign(renderers, renderers + n);
  *out = b;
  return LUCENT_OK;
}

static void drop_parts(lucent_batch* b) {
  for (lucent_batch* q : b->parts) lucent_batch_destroy(q);
  for (SideStream& s : b->part_streams) s.destroy();
  b->parts.clear();
  b->part_streams.clear();
}

void lucent_batch_destroy(lucent_batch* b) {
  if (!b) return;
  cudaDeviceSynchronize();  // waves in flight on the batch's own streams read its buffers
  drop_parts(b);
  b->destroy_graphs();
  for (WaveSet& w : b->set) w.destroy();
  delete b;
}

lucent_status lucent_batch_set_options(lucent_batch* b, const lucent_batch_options* o) {
  clear_error();
  if (!b || !o) return fail(LUCENT_ERR_INVALID, "null argument");
  if (o->max_wave_paths == 0) return fail(LUCENT_ERR_INVALID, "max_wave_paths must be positive");
  if (o->streams == 0 || o->streams > 16) return fail(LUCENT_ERR_INVALID, "streams must be 1 to 16, got %u", o->streams);
  b->opt = *o;
  b->drop_graphs();
  drop_parts(b);
  return LUCENT_OK;
}

// opt.streams > 1: the renderers in that many consecutive parts, each a
// batch of its own (same options, one stream) on a stream of its own, forked
// from and joined back into the caller's stream.
static lucent_status trace_parts(lucent_batch* b, uint32_t samples, cudaStream_t s) {
  const uint32_t n = (uint32_t)b->rs.size(), k = std::min<uint32_t>(b->opt.streams, n);
  lucent_status st;
  if (b->parts.size() != k) {
    drop_parts(b);
    lucent_batch_options o = b->opt;
    o.streams = 1;
    for (uint32_t i = 0; i < k; i++) {
      const uint32_t i0 = n * i / k, i1 = n * (i + 1) / k;
      lucent_batch* q = nullptr;
      if ((st = lucent_batch_create(b->rs.data() + i0, i1 - i0, &q))) return st;
      b->parts.push_back(q);
      if ((st = lucent_batch_set_options(q, &o))) return st;
      b->part_streams.emplace_back();
      if ((st = b->part_streams.back().ensure())) return st;
    }
  }
  cudaEventRecord(b->part_streams[0].fork, s);
  for (uint32_t i = 0; i < k; i++) {
    SideStream& ps = b->part_streams[i];
    cudaStreamWaitEvent(ps.stream, b->part_streams[0].fork, 0);
    if ((st = lucent_batch_trace(b->parts[i], samples, ps.stream))) return st;
    cudaEventRecord(ps.join, ps.stream);
    cudaStreamWaitEvent(s, ps.join, 0);
  }
  return LUCENT_OK;
}

lucent_status lucent_batch_trace(lucent_batch* b, uint32_t samples, void* stream) {
  clear_error();
  if (!b) return fail(LUCENT_ERR_INVALID, "null batch");
  if (samples == 0) return LUCENT_OK;
  if (b->opt.streams > 1 && b->rs.size() > 1) {
    for (size_t i = 0; i < b->rs.size(); i++)
      if (!scene_owner(b->rs[i])->has_scene || !b->rs[i]->has_lighting)
        return fail(LUCENT_ERR_INVALID, "renderer %zu: trace before load_scene / upload_lighting", i);
    return trace_parts(b, samples, (cudaStream_t)stream);
  }
  const int n = (int)b->rs.size();
  std::vector<SceneRec> recs(n);
  uint64_t pixels = 0;
  int max_bounces = 0, any_alpha = 0;
  cudaStream_t s = (cudaStream_t)stream;
  for (int i = 0; i < n; i++) {
    lucent_renderer* r = b->rs[i];
    if (!scene_owner(r)->has_scene || !r->has_lighting)
      return fail(LUCENT_ERR_INVALID, "renderer %d: trace before load_scene / upload_lighting", i);
    after_waves(r, s);  // the renderer's own traces accumulate first
    lucent_status st = prepare_reprojection(r, s);
    if (st) return st;
    recs[i] = scene_rec(r);
    pixels += (uint64_t)r->W * r->H;
    max_bounces = std::max(max_bounces, (int)r->max_bounces);
    any_alpha |= scene_owner(r)->any_alpha;
  }
  // Waves hold consecutive groups of scenes_per_wave scenes (0: all of them),
  // each group traced for all `samples` before the next; samples per wave, per
  // group: samples_per_wave, or as many as fit in max_wave_paths (at least one).
  const int k = b->opt.scenes_per_wave ? (int)std::min<uint32_t>(b->opt.scenes_per_wave, (uint32_t)n) : n;
  struct Group {
    int i0, i1, max_bounces, any_alpha, any_tex, classes;
    uint64_t pixels;
    uint32_t S, full, tail;
    size_t base;  // offset of the group's bases (full waves, then the tail wave) in b->bases, in words
  };
  std::vector<Group> gs;
  std::vector<uint32_t> hb;
  uint64_t cap64 = 0;
  auto make_bases = [&](const Group& G, uint32_t s_wave) {
    const int ng = G.i1 - G.i0;
    const size_t o = hb.size();
    hb.resize(o + 2 * (ng + 1), 0);
    for (int i = 0; i < ng; i++) {
      const uint32_t wh = (uint32_t)recs[G.i0 + i].W * recs[G.i0 + i].H;
      hb[o + i + 1] = hb[o + i] + wh * s_wave;                   // path_base
      hb[o + ng + 1 + i + 1] = hb[o + ng + 1 + i] + wh;          // pix_base
    }
  };
  for (int i0 = 0; i0 < n; i0 += k) {
    Group G{i0, std::min(n, i0 + k), 0, 0, 0, 0, 0, 0, 0, 0, hb.size()};
    std::vector<const Node*> bvhs;  // ray-sort classes: scenes sharing a BVH (views) sort together
    for (int i = G.i0; i < G.i1; i++) {
      const Node* nodes = recs[i].scene.nodes;
      int c = 0;
      while (c < (int)bvhs.size() && bvhs[c] != nodes) c++;
      if (c == (int)bvhs.size()) bvhs.push_back(nodes);
      recs[i].sort_class = c;
      G.pixels += (uint64_t)recs[i].W * recs[i].H;
      G.max_bounces = std::max(G.max_bounces, (int)b->rs[i]->max_bounces);
      G.any_alpha |= scene_owner(b->rs[i])->any_alpha;
      G.any_tex |= scene_owner(b->rs[i])->tex_size > 0;
    }
    G.classes = (int)bvhs.size();
    uint64_t S = b->opt.samples_per_wave ? b->opt.samples_per_wave
                                         : std::max<uint64_t>(1, b->opt.max_wave_paths / G.pixels);
    S = std::min<uint64_t>(S, samples);
    if (G.pixels * S * 3 >= (1ull << 32))
      return fail(LUCENT_ERR_UNSUPPORTED, "wave of %llu paths exceeds the 32-bit path index",
                  (unsigned long long)(G.pixels * S));
    G.S = (uint32_t)S;
    G.full = samples / G.S;
    G.tail = samples % G.S;
    cap64 = std::max(cap64, G.pixels * S);
    make_bases(G, G.S);
    make_bases(G, G.tail ? G.tail : G.S);
    gs.push_back(G);
  }
  (void)pixels;
  (void)max_bounces;
  (void)any_alpha;
  const uint32_t cap = (uint32_t)cap64;
  lucent_status st;
  for (WaveSet& X : b->set) {
    if ((st = X.ensure()) || (st = X.side.ensure())) return st;
    if (X.used) cudaStreamWaitEvent(X.stream, X.done, 0);  // the set's last wave is accumulated
    const uint32_t had = X.path_cap;
    if ((st = X.reserve(cap))) return st;
    if (X.path_cap != had) b->drop_graphs();  // new buffer addresses
    if ((st = X.rec.reserve(sizeof(SceneRec) * n)) || (st = X.base.reserve(4 * hb.size()))) return st;
    cudaError_t e = cudaMemcpyAsync(X.base.ptr, hb.data(), 4 * hb.size(), cudaMemcpyHostToDevice, X.stream);
    if (e != cudaSuccess) return cuda_fail(e, "upload batch tables");
  }
  for (std::vector<WaveGraph>& g : b->graphs)
    if (g.size() != gs.size()) {
      b->destroy_graphs();
      b->graphs[0].resize(gs.size());
      b->graphs[1].resize(gs.size());
      break;
    }
  MultiLaunch M{};
  M.trace_blocks = (int)b->opt.trace_blocks;
  M.shade_blocks = (int)b->opt.shade_blocks;
  M.sort_rays = b->opt.sort_rays;
  M.top_levels = b->opt.top_levels;
  M.wide = b->opt.wide_bvh;
  for (size_t g = 0; g < gs.size(); g++) {
    const Group& G = gs[g];
    const int ng = G.i1 - G.i0;
    M.n = ng;
    M.max_bounces = G.max_bounces;
    M.any_alpha = G.any_alpha;
    M.any_tex = G.any_tex;
    M.total_pixels = (uint32_t)G.pixels;
    M.sort_classes = G.classes;
    for (uint32_t w = 0; w < G.full + (G.tail ? 1u : 0u); w++) {
      const int x = b->next_set;
      WaveSet& X = b->set[x];
      b->next_set ^= 1;
      if (X.used) cudaStreamWaitEvent(X.stream, X.done, 0);
      // the group's scene records with this wave's sample seeds (a pending
      // reprojection in the group's first wave only)
      std::vector<SceneRec> wr(recs.begin() + G.i0, recs.begin() + G.i1);
      for (int i = 0; i < ng; i++) {
        wr[i].seed0 = b->rs[G.i0 + i]->seed + w * G.S;
        if (w > 0) wr[i].reproject = 0;
      }
      cudaError_t e = cudaMemcpyAsync((SceneRec*)X.rec.ptr + G.i0, wr.data(), sizeof(SceneRec) * ng,
                                      cudaMemcpyHostToDevice, X.stream);
      if (e != cudaSuccess) return cuda_fail(e, "upload scene records");
      M.paths = X.P;
      M.sid = (uint16_t*)X.sid.ptr;
      X.side.set(M);
      M.recs = (SceneRec*)X.rec.ptr + G.i0;
      const bool full = w < G.full;
      M.S = (int)(full ? G.S : G.tail);
      M.total_paths = (uint32_t)(G.pixels * (uint32_t)M.S);
      M.path_base = (const uint32_t*)X.base.ptr + G.base + (full ? 0 : 2 * (ng + 1));
      M.pix_base = M.path_base + (ng + 1);
      if (full && b->opt.use_graph && b->waves > 0) {  // first wave ever runs uncaptured (one-time setup inside)
        uint64_t key[4];
        wave_key(M, key);
        key[0] |= 1ull << 63;  // captured without the accumulation
        if ((st = b->graphs[x][g].run(M, key, X.stream, false))) return st;
        b->graph_waves++;
        b->kernel_launches += b->graphs[x][g].launches;
      } else {
        b->kernel_launches += render_wave_multi(M, X.stream, nullptr, false);
      }
      cudaEventRecord(X.traced, X.stream);
      cudaStreamWaitEvent(s, X.traced, 0);
      b->kernel_launches += accumulate_wave(M, s);
      cudaEventRecord(X.done, s);
      X.used = true;
      b->waves++;
    }
  }
  for (lucent_renderer* r : b->rs) {
    r->seed += samples;
    r->frame += samples;
    record_history(r);
  }
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LUCENT_OK : cuda_fail(e, "batch trace launch");
}

lucent_status lucent_batch_check(lucent_batch* b, void* stream, lucent_batch_stats* out) {
  clear_error();
  if (!b) return fail(LUCENT_ERR_INVALID, "null batch");
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "synchronize");
  lucent_batch_stats acc;
  std::memset(&acc, 0, sizeof acc);
  for (lucent_batch* q : b->parts) {  // parts traced on their own streams (the caller's joined them)
    lucent_batch_stats ps;
    if (lucent_status st = lucent_batch_check(q, stream, &ps)) return st;
    acc.closest_rays += ps.closest_rays;
    acc.shadow_rays += ps.shadow_rays;
    acc.waves += ps.waves;
    acc.graph_waves += ps.graph_waves;
    acc.wave_paths += ps.wave_paths;
    acc.kernel_launches += ps.kernel_launches;
  }
  if (out) {
    *out = acc;
    out->waves += b->waves;
    out->graph_waves += b->graph_waves;
    out->wave_paths += std::max(b->set[0].path_cap, b->set[1].path_cap);
    out->kernel_launches += b->kernel_launches;
  }
  for (WaveSet& X : b->set) {
    if (!X.ctr.ptr) continue;
    uint32_t words[kCtrWords];
    e = cudaMemcpy(words, X.ctr.ptr, sizeof words, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "read batch counters");
    if (out) {
      uint64_t c = 0, sh = 0;
      std::memcpy(&c, words + kCtrStatClosest, 8);
      std::memcpy(&sh, words + kCtrStatShadow, 8);
      out->closest_rays += c;
      out->shadow_rays += sh;
    }
    if (words[kCtrErr]) {
      clear_now((uint32_t*)X.ctr.ptr + kCtrErr, 4);
      return fail(LUCENT_ERR_DEVICE, "batch raised device error word 0x%x", words[kCtrErr]);
    }
  }
  return LUCENT_OK;
}

}  // extern "C"
