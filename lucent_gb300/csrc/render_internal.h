// Device-side state of the wavefront renderer, shared by its kernels and the C ABI.
#pragma once
#include <cuda_fp16.h>

#include "shade.cuh"

namespace lucent {

// Counter words (uint32) in Paths::ctr.
enum : int {
  kCtrQ0 = 0,           // active-queue lengths [0], [1]
  kCtrShadow = 2,       // shadow-queue length
  kCtrWork = 3,         // closest-hit persistent ray counter
  kCtrSlow = 4,         // closest-hit slow-path queue length
  kCtrWork2 = 5,        // any-hit work counter (unused by the grid-stride kernel)
  kCtrSlow2 = 6,        // any-hit slow-path queue length
  kCtrErr = 7,          // device error word
  kCtrTex = 12,         // textured-hit queue length (paths left to the TEX shade instantiation)
  kCtrStatClosest = 8,  // u64: closest-hit rays traced (words 8-9)
  kCtrStatShadow = 10,  // u64: shadow rays traced (words 10-11)
  kCtrTrav = 16,        // 5 x u64 closest-hit traversal counters (words 16-25), profiling only
  kCtrWords = 32,
};

struct __align__(8) half4 {
  __half x, y, z, w;
};
__device__ __forceinline__ half4 make_half4(float4 v) {
  half4 h;
  h.x = __float2half_rn(v.x);
  h.y = __float2half_rn(v.y);
  h.z = __float2half_rn(v.z);
  h.w = __float2half_rn(v.w);
  return h;
}

// Structure-of-arrays path state; shadow slots are 3 per path (sun, env, light).
// Path state lives in one 128-byte record per path (8 float4: origin + RNG
// state bits, direction, throughput + bsdf pdf, guide tint + flags, guide
// albedo, guide normal + depth, guide position + reuse, radiance); field f of
// path p is float4 number f of record p. A kernel that walks paths in sorted
// (not path) order then touches one DRAM line per path instead of one per
// field.
constexpr int kPathRecord = 8;
struct PathField {
  float4* base;  // the field in record 0
  __host__ __device__ float4& operator[](size_t p) const { return base[p * kPathRecord]; }
};

struct Paths {
  float4* rec;  // path records
  PathField ro, rd, thr, tint, galb, gnrm;
  PathField gpos;  // guide: primary hit position (xyz) and how much history it may reuse (w)
  PathField rad;   // radiance per path
  float4* hit;     // closest hit per position of the bounce's queue
  float4 *sh_o, *sh_d, *sh_c;
  uint32_t* q[2];
  uint32_t* qs;
  uint32_t* slow;
  uint32_t* slow2;
  uint32_t* sort_keys;  // per queued path: ray-sort key (BVH class, direction cell, origin cell)
  float4* nray;         // the bounce's rays in queue order: 2 float4 each (origin + path id, direction + scene)
  float4* sray;         // the same sorted (after a ray sort)
  uint32_t* sort_tmp;   // the sorted queue, swapped with the queue it sorts
  uint32_t* qtex;       // queue positions of hits on texture-mapped materials (shaded by the TEX instantiation)
  uint32_t* sort_hist;  // kSortBins counters
  uint32_t* ctr;
};

constexpr int kSortBits = 15, kSortBins = 1 << kSortBits;

// Accumulation targets (renderer.ts:490): RGBA32F colour + lum^2, RGBA16F
// albedo + coverage, RGBA16F normal + depth, R32F history.
struct AccumDev {
  float4* color;
  half4* albedo;
  half4* normal;
  float* history;
};

// One scene of a multi-scene wave (device table, one entry per scene).
struct SceneRec {
  sh::SceneDev scene;
  sh::LightingDev light;
  sh::CameraDev cam;
  AccumDev accum;
  int W, H, max_bounces;
  float clamp;
  uint32_t seed0;  // sample seed (uSeed) of the wave's first sample; advanced on the device
  // temporal reprojection of the wave's first sample (trace.frag:275-322); cleared on the device after it
  int reproject;
  AccumDev prev;       // copy of the targets as the previous view left them
  sh::CameraDev prev_cam;
  int prev_w, prev_h;
  // Ray-sort class: scenes of a wave that traverse the same BVH (views of
  // one scene) share a class, 0 .. MultiLaunch::sort_classes - 1, so their
  // rays sort together by direction and origin.
  int sort_class;
};

constexpr float kHistoryCap = 8.f;  // HISTORY_CAP (renderer.ts:139)

struct MultiLaunch {
  Paths paths;
  SceneRec* recs;              // device, n entries
  const uint32_t* path_base;   // device, n + 1 entries: scene i owns paths [path_base[i], path_base[i+1])
  const uint32_t* pix_base;    // device, n + 1 entries: the same for pixels
  uint16_t* sid;               // device, scene index per path
  int n, S, max_bounces;       // max_bounces = the largest over the scenes
  uint32_t total_paths, total_pixels;
  int any_alpha;
  int trace_blocks, shade_blocks;  // 0 = all resident blocks
  unsigned long long* trav_stats;  // closest-hit traversal counters (profiling) or nullptr
  int sort_rays;                   // after bounces 0 and 1, sort the rays by BVH class, direction and origin cell
  int top_levels;                  // stage the top BVH levels of (up to 8) scenes in shared memory
  int any_tex;                     // some scene has texture maps: launch the TEX shade instantiation
  int wide;                        // closest hit over the scenes' four-wide BVH views
  int sort_classes;                // distinct SceneRec::sort_class values (>= 1)
  // Ray capture (lucent_renderer_capture_rays; parity tests): for every
  // bounce b in cap_mask, the bounce's closest-hit rays with their hits and
  // its shadow rays with their answers are copied, 4 float4 per ray, into
  // regions 2r and 2r + 1 of cap (r = rank of b in cap_mask, cap_stride rays
  // each); cap_count[2r], cap_count[2r + 1] receive the queue lengths.
  unsigned cap_mask;
  float4* cap;
  uint32_t* cap_count;
  uint32_t cap_stride;
  // Second stream and fork / join events (nullptr: one stream): the deep
  // bounces' shadow rays run beside the next bounce's closest hit.
  cudaStream_t side;
  cudaEvent_t ev_fork, ev_join;
};

// Optional per-phase timing: events recorded between launches, each tagged
// with the phase of the interval that ends at it.
enum Phase : int { kPhCamera = 0, kPhClosest, kPhShade, kPhShadow, kPhResolve, kPhAccumulate, kPhases };
struct PhaseEvents {
  cudaEvent_t* ev;  // pool
  int* tag;         // phase of the interval ending at ev[i]
  int cap, n;
  void mark(int phase, cudaStream_t s) {
    if (ev && n < cap) {
      cudaEventRecord(ev[n], s);
      tag[n++] = phase;
    }
  }
};


// One wave of S samples for every scene of a launch (a single renderer is a
// launch of one scene: the same kernels, so a batch reproduces it bit for
// bit). Graph-safe: no host synchronisation, every count stays on the device.
// Returns the number of kernels it launched. Without `accumulate` it stops
// after the last bounce: accumulate_wave then adds the wave's samples to the
// targets (and advances the seeds), on any stream ordered after it.
int render_wave_multi(const MultiLaunch& M, cudaStream_t s, PhaseEvents* pe = nullptr, bool accumulate = true);
int accumulate_wave(const MultiLaunch& M, cudaStream_t s);

// Device buffers of a path-replay backward pass (per path: lrem 1, gcont 5,
// genv 2 float4; per shadow slot: gslot 2 float4; dl per pixel).
struct AdjointDevHost {
  const float4* dl;
  float4 *lrem, *gcont, *gslot, *genv;
  float* dmat;
  float* denv;  // environment texel gradients, 4 floats (RGB, pad) per texel, 16-byte aligned
};
// Gradient of sum_px dl[px] . (mean of the wave's samples) with respect to
// material parameters (6 per material) and environment texels, for a launch
// of one scene (recs[0].seed0 = the wave's first sample seed).
void render_backward(const MultiLaunch& M, const AdjointDevHost& H, cudaStream_t s);

// sheenAlbedoLUT (16 x 16) rounded to half precision, as the reference uploads it.
void sheen_lut_half(float* out);

// Denoiser (variance + `levels` a-trous steps of spacing 1, 2, 4, ...): fa,
// fb are W*H float4 ping-pong targets, g0, g1 W*H float4 guide buffers.
// Returns fa or fb, whichever holds the result.
float4* denoise_run(AccumDev A, const sh::CameraDev& cam, int W, int H, int levels, float sigma_l, float sigma_n,
                    float sigma_p, float4* fa, float4* fb, float4* g0, float4* g1, cudaStream_t s);
// Display pass of the W x H targets into a VW x VH view: RGBA8 and/or the
// pre-quantization RGB floats (either may be null).
void display_run(AccumDev A, const float4* den, int W, int H, int VW, int VH, float weight, float exposure,
                 int tonemap, uchar4* rgba8, float* rgb, cudaStream_t s);

}  // namespace lucent
