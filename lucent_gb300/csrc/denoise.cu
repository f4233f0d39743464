// SVGF-style denoiser and display pass: the reference's variance.frag,
// atrous.frag (driven as runDenoiser, src/renderer.ts:788-830) and
// display.frag, as CUDA kernels over the accumulation targets.
//
// The a-trous taps need, per neighbour, the unit guide normal and the world
// position reconstructed from the primary ray and depth (atrous.frag:92-126).
// Both depend only on the pixel, so k_guides computes them once per denoise
// (32 B per pixel) instead of once per tap; the values are the reference's
// formulas evaluated the same way.
#include <cuda_fp16.h>

#include "internal.h"
#include "render_internal.h"
#include "shade.cuh"

namespace lucent {

using namespace sh;

__device__ __forceinline__ float lum3(float r, float g, float b) { return r * 0.2126f + g * 0.7152f + b * 0.0722f; }

__device__ __forceinline__ float3 unit_normal(float x, float y, float z) {  // denoise.glsl:21-24
  const float l = sqrtf(x * x + y * y + z * z);
  return l > 1e-6f ? make_float3(x / l, y / l, z / l) : make_float3(0.f, 0.f, 1.f);
}

__device__ __forceinline__ float4 h4(half4 v) {
  return make_float4(__half2float(v.x), __half2float(v.y), __half2float(v.z), __half2float(v.w));
}

// variance.frag:15-55 -> (demodulated illumination, variance).
__global__ void k_variance(AccumDev A, int W, int H, float4* __restrict__ out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= W || y >= H) return;
  const size_t p = (size_t)y * W + x;
  const float4 c = A.color[p];
  const float4 a = h4(A.albedo[p]);
  if (a.w < 0.5f) {
    out[p] = make_float4(c.x, c.y, c.z, 0.f);
    return;
  }
  const float3 illum = make_float3(c.x / fmaxf(a.x, 1e-3f), c.y / fmaxf(a.y, 1e-3f), c.z / fmaxf(a.z, 1e-3f));
  const float samples = fmaxf(A.history[p], 1.f);
  const float la = fmaxf(lum3(a.x, a.y, a.z), 1e-3f);
  float variance;
  if (samples >= 4.f) {
    const float l = lum3(c.x, c.y, c.z);
    variance = fmaxf(0.f, c.w - l * l) / (la * la) / samples;
  } else {  // 7 x 7 spatial estimate for the first samples
    const float4 np = h4(A.normal[p]);
    const float3 n = unit_normal(np.x, np.y, np.z);
    float s1 = 0.f, s2 = 0.f, ws = 0.f;
    for (int dy = -3; dy <= 3; dy++)
      for (int dx = -3; dx <= 3; dx++) {
        const int qx = x + dx, qy = y + dy;
        if (qx < 0 || qy < 0 || qx >= W || qy >= H) continue;
        const size_t q = (size_t)qy * W + qx;
        const float4 aq = h4(A.albedo[q]);
        if (aq.w < 0.5f) continue;
        const float4 nq = h4(A.normal[q]);
        const float3 un = unit_normal(nq.x, nq.y, nq.z);
        const float st = (0.1f * np.w < fabsf(np.w - nq.w)) ? 0.f : 1.f;
        const float w = powf(fmaxf(0.f, n.x * un.x + n.y * un.y + n.z * un.z), 32.f) * st;
        const float4 cq = A.color[q];
        const float l = lum3(cq.x / fmaxf(aq.x, 1e-3f), cq.y / fmaxf(aq.y, 1e-3f), cq.z / fmaxf(aq.z, 1e-3f));
        s1 += w * l;
        s2 += w * l * l;
        ws += w;
      }
    const float m1 = s1 / fmaxf(ws, 1e-6f);
    variance = fmaxf(0.f, s2 / fmaxf(ws, 1e-6f) - m1 * m1) / samples;
  }
  out[p] = make_float4(illum.x, illum.y, illum.z, variance);
}

// Per pixel: (unit normal, covered) and (world position, depth).
__global__ void k_guides(AccumDev A, CameraDev cam, int W, int H, float4* __restrict__ g0, float4* __restrict__ g1) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= W || y >= H) return;
  const size_t p = (size_t)y * W + x;
  const float4 np = h4(A.normal[p]);
  const float cov = __half2float(A.albedo[p].w);
  const float3 n = unit_normal(np.x, np.y, np.z);
  // primaryDir (atrous.frag:77-81)
  const float ux = ((float)x + 0.5f) / (float)W * 2.f - 1.f, uy = ((float)y + 0.5f) / (float)H * 2.f - 1.f;
  const float aspect = (float)W / (float)H;
  const float3 d = norm3(cam.forward + cam.right * (ux * aspect * cam.tan_half_fov) + cam.up * (uy * cam.tan_half_fov));
  const float3 P = cam.pos + d * np.w;
  g0[p] = make_float4(n.x, n.y, n.z, cov);
  g1[p] = make_float4(P.x, P.y, P.z, np.w);
}

// One a-trous iteration (atrous.frag:85-137) at hole spacing `step`.
__global__ void __launch_bounds__(256) k_atrous(const float4* __restrict__ in, const float4* __restrict__ g0,
                                                const float4* __restrict__ g1, int W, int H, int step, float tan_half,
                                                float sigma_l, float sigma_n, float sigma_p,
                                                float4* __restrict__ out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= W || y >= H) return;
  const size_t p = (size_t)y * W + x;
  const float4 cp = __ldg(in + p);
  const float4 gp = __ldg(g0 + p);
  if (gp.w < 0.5f) {
    out[p] = cp;
    return;
  }
  const float4 Pp = __ldg(g1 + p);
  const float footprint = 2.f * tan_half * Pp.w / (float)H;
  float var = 0.f, wv = 0.f;
#pragma unroll
  for (int dy = -1; dy <= 1; dy++)
#pragma unroll
    for (int dx = -1; dx <= 1; dx++) {
      const int qx = x + dx, qy = y + dy;
      if (qx < 0 || qy < 0 || qx >= W || qy >= H) continue;
      const float k = (dx == 0 ? 0.5f : 0.25f) * (dy == 0 ? 0.5f : 0.25f);
      var += __ldg(&in[(size_t)qy * W + qx].w) * k;
      wv += k;
    }
  const float denom = sigma_l * sqrtf(fmaxf(var / wv, 0.f)) + 1e-6f;
  const float lp = lum3(cp.x, cp.y, cp.z);
  const float h[3] = {0.375f, 0.25f, 0.0625f};
  float3 sum = make_float3(cp.x * (h[0] * h[0]), cp.y * (h[0] * h[0]), cp.z * (h[0] * h[0]));
  float sumVar = cp.w * (h[0] * h[0]) * (h[0] * h[0]);
  float wsum = h[0] * h[0];
#pragma unroll
  for (int dy = -2; dy <= 2; dy++)
#pragma unroll
    for (int dx = -2; dx <= 2; dx++) {
      if (dx == 0 && dy == 0) continue;
      const int qx = x + dx * step, qy = y + dy * step;
      if (qx < 0 || qy < 0 || qx >= W || qy >= H) continue;
      const size_t q = (size_t)qy * W + qx;
      const float4 gq = __ldg(g0 + q);
      if (gq.w < 0.5f) continue;
      const float4 cq = __ldg(in + q);
      const float4 Q = __ldg(g1 + q);
      const float k = h[dx < 0 ? -dx : dx] * h[dy < 0 ? -dy : dy];
      const float wn = powf(fmaxf(0.f, gp.x * gq.x + gp.y * gq.y + gp.z * gq.z), sigma_n);
      const float reach = sigma_p * footprint * (float)step * sqrtf((float)(dx * dx + dy * dy));
      const float pd = gp.x * (Q.x - Pp.x) + gp.y * (Q.y - Pp.y) + gp.z * (Q.z - Pp.z);
      const float wp = expf(-fabsf(pd) / (reach + 1e-6f));
      const float wl = expf(-fabsf(lp - lum3(cq.x, cq.y, cq.z)) / denom);
      const float w = k * wn * wp * wl;
      sum = sum + make_float3(cq.x, cq.y, cq.z) * w;
      sumVar += cq.w * w * w;
      wsum += w;
    }
  out[p] = make_float4(sum.x / wsum, sum.y / wsum, sum.z / wsum, sumVar / (wsum * wsum));
}

// k_atrous for hole spacings 1, 2 and 4 with the block's 16 x 16 pixels and
// their 2 * STEP halo staged in shared memory (illumination + variance, unit
// normal + coverage, world position + depth: 48 B per pixel), so every tap
// and the 3 x 3 variance blur read shared memory. Same arithmetic in the same
// order as k_atrous (this file is compiled without FMA contraction), so the
// two give identical results.
template <int STEP>
__global__ void __launch_bounds__(256) k_atrous_tiled(const float4* __restrict__ in, const float4* __restrict__ g0,
                                                      const float4* __restrict__ g1, int W, int H, float tan_half,
                                                      float sigma_l, float sigma_n, float sigma_p,
                                                      float4* __restrict__ out) {
  constexpr int T = 16 + 4 * STEP;
  extern __shared__ float4 sm[];
  float4* s_in = sm;
  float4* s_g0 = sm + T * T;
  float4* s_g1 = sm + 2 * T * T;
  const int ox = (int)blockIdx.x * 16 - 2 * STEP, oy = (int)blockIdx.y * 16 - 2 * STEP;
  for (int i = threadIdx.y * 16 + threadIdx.x; i < T * T; i += 256) {
    const int gx = ox + i % T, gy = oy + i / T;
    if (gx >= 0 && gy >= 0 && gx < W && gy < H) {
      const size_t q = (size_t)gy * W + gx;
      s_in[i] = __ldg(in + q);
      s_g0[i] = __ldg(g0 + q);
      s_g1[i] = __ldg(g1 + q);
    }
  }
  __syncthreads();
  const int x = (int)blockIdx.x * 16 + threadIdx.x, y = (int)blockIdx.y * 16 + threadIdx.y;
  if (x >= W || y >= H) return;
  const int lx = threadIdx.x + 2 * STEP, ly = threadIdx.y + 2 * STEP;
  const size_t p = (size_t)y * W + x;
  const float4 cp = s_in[ly * T + lx];
  const float4 gp = s_g0[ly * T + lx];
  if (gp.w < 0.5f) {
    out[p] = cp;
    return;
  }
  const float4 Pp = s_g1[ly * T + lx];
  const float footprint = 2.f * tan_half * Pp.w / (float)H;
  float var = 0.f, wv = 0.f;
#pragma unroll
  for (int dy = -1; dy <= 1; dy++)
#pragma unroll
    for (int dx = -1; dx <= 1; dx++) {
      const int qx = x + dx, qy = y + dy;
      if (qx < 0 || qy < 0 || qx >= W || qy >= H) continue;
      const float k = (dx == 0 ? 0.5f : 0.25f) * (dy == 0 ? 0.5f : 0.25f);
      var += s_in[(ly + dy) * T + lx + dx].w * k;
      wv += k;
    }
  const float denom = sigma_l * sqrtf(fmaxf(var / wv, 0.f)) + 1e-6f;
  const float lp = lum3(cp.x, cp.y, cp.z);
  const float h[3] = {0.375f, 0.25f, 0.0625f};
  float3 sum = make_float3(cp.x * (h[0] * h[0]), cp.y * (h[0] * h[0]), cp.z * (h[0] * h[0]));
  float sumVar = cp.w * (h[0] * h[0]) * (h[0] * h[0]);
  float wsum = h[0] * h[0];
#pragma unroll
  for (int dy = -2; dy <= 2; dy++)
#pragma unroll
    for (int dx = -2; dx <= 2; dx++) {
      if (dx == 0 && dy == 0) continue;
      const int qx = x + dx * STEP, qy = y + dy * STEP;
      if (qx < 0 || qy < 0 || qx >= W || qy >= H) continue;
      const int t = (ly + dy * STEP) * T + lx + dx * STEP;
      const float4 gq = s_g0[t];
      if (gq.w < 0.5f) continue;
      const float4 cq = s_in[t];
      const float4 Q = s_g1[t];
      const float k = h[dx < 0 ? -dx : dx] * h[dy < 0 ? -dy : dy];
      const float wn = powf(fmaxf(0.f, gp.x * gq.x + gp.y * gq.y + gp.z * gq.z), sigma_n);
      const float reach = sigma_p * footprint * (float)STEP * sqrtf((float)(dx * dx + dy * dy));
      const float pd = gp.x * (Q.x - Pp.x) + gp.y * (Q.y - Pp.y) + gp.z * (Q.z - Pp.z);
      const float wp = expf(-fabsf(pd) / (reach + 1e-6f));
      const float wl = expf(-fabsf(lp - lum3(cq.x, cq.y, cq.z)) / denom);
      const float w = k * wn * wp * wl;
      sum = sum + make_float3(cq.x, cq.y, cq.z) * w;
      sumVar += cq.w * w * w;
      wsum += w;
    }
  out[p] = make_float4(sum.x / wsum, sum.y / wsum, sum.z / wsum, sumVar / (wsum * wsum));
}

// display.frag:33-40: a texel of the traced region (clamped to it) with the
// remodulated denoised image blended in.
__device__ __forceinline__ float3 display_radiance(const AccumDev& A, const float4* __restrict__ den, int RW, int RH,
                                                   int x, int y, float weight) {
  x = min(max(x, 0), RW - 1);
  y = min(max(y, 0), RH - 1);
  const size_t p = (size_t)y * RW + x;
  const float4 raw = A.color[p];
  float3 c = make_float3(raw.x, raw.y, raw.z);
  if (weight > 0.f && den) {
    const float4 a = h4(A.albedo[p]);
    if (a.w >= 0.5f) {
      const float4 d = den[p];
      c = make_float3(c.x * (1.f - weight) + d.x * fmaxf(a.x, 1e-3f) * weight,
                      c.y * (1.f - weight) + d.y * fmaxf(a.y, 1e-3f) * weight,
                      c.z * (1.f - weight) + d.z * fmaxf(a.z, 1e-3f) * weight);
    }
  }
  return c;
}

// display.frag:42-67: the traced region (RW x RH, the targets) shown in a
// VW x VH view; Catmull-Rom upsampling (:47-60) when the sizes differ (the
// reference's reduced-resolution preview while the camera moves). Then
// exposure, tone map, sRGB, IGN dither, RGBA8.
__global__ void k_display(AccumDev A, const float4* __restrict__ den, int RW, int RH, int VW, int VH, float weight,
                          float exposure, int tonemap, uchar4* __restrict__ rgba8, float* __restrict__ rgb) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= VW || y >= VH) return;
  const float fx = (float)x + 0.5f, fy = (float)y + 0.5f;  // gl_FragCoord.xy
  float3 c3;
  if (RW == VW && RH == VH) {
    c3 = display_radiance(A, den, RW, RH, x, y, weight);
  } else {
    const float srx = fx * ((float)RW / (float)VW) - 0.5f, sry = fy * ((float)RH / (float)VH) - 0.5f;
    const int ix = (int)floorf(srx), iy = (int)floorf(sry);
    const float tx = srx - floorf(srx), ty = sry - floorf(sry);
    const float wx[4] = {tx * (-0.5f + tx * (1.f - 0.5f * tx)), 1.f + tx * tx * (-2.5f + 1.5f * tx),
                         tx * (0.5f + tx * (2.f - 1.5f * tx)), tx * tx * (-0.5f + 0.5f * tx)};
    const float wy[4] = {ty * (-0.5f + ty * (1.f - 0.5f * ty)), 1.f + ty * ty * (-2.5f + 1.5f * ty),
                         ty * (0.5f + ty * (2.f - 1.5f * ty)), ty * ty * (-0.5f + 0.5f * ty)};
    c3 = make_float3(0.f, 0.f, 0.f);
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int i = 0; i < 4; i++) {
        const float3 r = display_radiance(A, den, RW, RH, ix + i - 1, iy + j - 1, weight);
        const float w = wx[i] * wy[j];
        c3 = make_float3(c3.x + r.x * w, c3.y + r.y * w, c3.z + r.z * w);
      }
    c3 = make_float3(fmaxf(c3.x, 0.f), fmaxf(c3.y, 0.f), fmaxf(c3.z, 0.f));
  }
  const float c[3] = {c3.x, c3.y, c3.z};
  const float t = 0.06711056f * fx + 0.00583715f * fy;
  const float u = 52.9829189f * (t - floorf(t));
  const float ign = u - floorf(u);
  const size_t p = (size_t)y * VW + x;
  unsigned char q[3];
  for (int k = 0; k < 3; k++) {
    float v = c[k] * exposure;
    if (tonemap == 0)
      v = clampf((v * (2.51f * v + 0.03f)) / (v * (2.43f * v + 0.59f) + 0.14f), 0.f, 1.f);  // Narkowicz ACES
    else if (tonemap == 1)
      v = v / (1.f + v);
    v = clampf(v, 0.f, 1.f);
    v = v < 0.0031308f ? v * 12.92f : 1.055f * powf(v, 1.f / 2.4f) - 0.055f;
    v += (ign - 0.5f) / 255.f;
    if (rgb) rgb[3 * p + k] = v;
    q[k] = (unsigned char)__float2int_rn(clampf(v, 0.f, 1.f) * 255.f);
  }
  if (rgba8) rgba8[p] = make_uchar4(q[0], q[1], q[2], 255);
}

// runDenoiser: variance, then `levels` a-trous steps (1, 2, 4, 8, 16),
// ping-ponging; returns the buffer holding the result.
float4* denoise_run(AccumDev A, const CameraDev& cam, int W, int H, int levels, float sigma_l, float sigma_n,
                    float sigma_p, float4* fa, float4* fb, float4* g0, float4* g1, cudaStream_t s) {
  const dim3 blk(16, 16), grd((W + 15) / 16, (H + 15) / 16);
  k_variance<<<grd, blk, 0, s>>>(A, W, H, fa);
  k_guides<<<grd, blk, 0, s>>>(A, cam, W, H, g0, g1);
  float4 *rd = fa, *wr = fb;
  for (int l = 0; l < levels; l++) {
    const int step = 1 << l;
    const float th = cam.tan_half_fov;
    if (step == 1)
      k_atrous_tiled<1><<<grd, blk, 3 * 20 * 20 * 16, s>>>(rd, g0, g1, W, H, th, sigma_l, sigma_n, sigma_p, wr);
    else if (step == 2)
      k_atrous_tiled<2><<<grd, blk, 3 * 24 * 24 * 16, s>>>(rd, g0, g1, W, H, th, sigma_l, sigma_n, sigma_p, wr);
    else if (step == 4)
      k_atrous_tiled<4><<<grd, blk, 3 * 32 * 32 * 16, s>>>(rd, g0, g1, W, H, th, sigma_l, sigma_n, sigma_p, wr);
    else  // the 8 and 16 halos (4 and 8 KB rows) would not fit: taps through L1
      k_atrous<<<grd, blk, 0, s>>>(rd, g0, g1, W, H, step, th, sigma_l, sigma_n, sigma_p, wr);
    float4* t = rd;
    rd = wr;
    wr = t;
  }
  return rd;
}

void display_run(AccumDev A, const float4* den, int W, int H, int VW, int VH, float weight, float exposure,
                 int tonemap, uchar4* rgba8, float* rgb, cudaStream_t s) {
  const dim3 blk(16, 16), grd((VW + 15) / 16, (VH + 15) / 16);
  k_display<<<grd, blk, 0, s>>>(A, den, W, H, VW, VH, weight, exposure, tonemap, rgba8, rgb);
}

}  // namespace lucent
