// Runs the path tracer's own BSDF code (shade.cuh: eval_opaque,
// sample_opaque, sample_dielectric, the bsdf.glsl restatement the shade
// kernel calls) on caller-supplied tuples, so the BSDF can be checked
// against a binary64 evaluation without going through a render.
//
// Tuple (32 floats): 0-2 albedo, 3 metallic, 4 roughness, 5 ior, 6 clearcoat,
// 7 clearcoat roughness, 8-10 sheen colour, 11 sheen roughness, 12 thin
// walled, 13-15 n, 16-18 clearcoat normal, 19-21 wo, 22-24 wi, 25-30 six
// uniforms drawn in order (wrapping), 31 front face (geometric normal = n).
// Output (24 floats): 0-2 evalOpaque f, 3 its pdf; 4-6 sampleOpaque
// direction, 7-9 weight, 10 pdf; 11 sampleDielectric ok, 12-14 direction,
// 15-17 weight, 18 reflected; 19-23 zero.
#include "../../include/lucent.h"
#include "api_util.h"
#include "internal.h"
#include "render_internal.h"

namespace lucent {

using namespace sh;

__global__ void k_bsdf_tuples(const float* __restrict__ in, uint32_t n, const float* __restrict__ lut,
                              float* __restrict__ out) {
  LightingDev L{};
  L.sheen_lut = lut;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float* t = in + (size_t)i * 32;
    Surface s;
    s.albedo = f3(t[0], t[1], t[2]);
    s.metallic = t[3];
    s.roughness = t[4];
    s.ior = t[5];
    s.transmission = 0.f;
    s.clearcoat = t[6];
    s.clearcoat_roughness = t[7];
    s.sheen_color = f3(t[8], t[9], t[10]);
    s.sheen_roughness = t[11];
    s.thin = t[12] > 0.5f;
    s.n = f3(t[13], t[14], t[15]);
    s.nc = f3(t[16], t[17], t[18]);
    s.absorption = f3(0.f, 0.f, 0.f);
    const float3 wo = f3(t[19], t[20], t[21]), wi = f3(t[22], t[23], t[24]);
    float* o = out + (size_t)i * 24;
    float pdf;
    const float3 f = eval_opaque(L, s, wo, wi, pdf);
    o[0] = f.x, o[1] = f.y, o[2] = f.z, o[3] = pdf;
    int k = 0;
    auto U = [&]() { return t[25 + (k++ % 6)]; };
    const BsdfSample bs = sample_opaque(L, s, wo, U);
    o[4] = bs.dir.x, o[5] = bs.dir.y, o[6] = bs.dir.z;
    o[7] = bs.weight.x, o[8] = bs.weight.y, o[9] = bs.weight.z, o[10] = bs.pdf;
    k = 0;
    float3 dwi = f3(0.f, 0.f, 0.f), dw = f3(0.f, 0.f, 0.f);
    bool refl = false;
    const bool ok = sample_dielectric(s, t[31] > 0.5f, s.n, wo, dwi, dw, refl, U);
    o[11] = ok ? 1.f : 0.f, o[12] = dwi.x, o[13] = dwi.y, o[14] = dwi.z;
    o[15] = dw.x, o[16] = dw.y, o[17] = dw.z, o[18] = refl ? 1.f : 0.f;
    for (int q = 19; q < 24; q++) o[q] = 0.f;
  }
}

// eval_opaque_grad on the same tuples: out 24 floats = f (3), then
// df/d(albedo r, g, b, roughness, metallic, clearcoat) (6 x 3), then 3 zeros.
__global__ void k_bsdf_grad_tuples(const float* __restrict__ in, uint32_t n, const float* __restrict__ lut,
                                   float* __restrict__ out) {
  LightingDev L{};
  L.sheen_lut = lut;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float* t = in + (size_t)i * 32;
    Surface s;
    s.albedo = f3(t[0], t[1], t[2]);
    s.metallic = t[3];
    s.roughness = t[4];
    s.ior = t[5];
    s.transmission = 0.f;
    s.clearcoat = t[6];
    s.clearcoat_roughness = t[7];
    s.sheen_color = f3(t[8], t[9], t[10]);
    s.sheen_roughness = t[11];
    s.thin = t[12] > 0.5f;
    s.n = f3(t[13], t[14], t[15]);
    s.nc = f3(t[16], t[17], t[18]);
    s.absorption = f3(0.f, 0.f, 0.f);
    float3 df[6];
    const float3 f = eval_opaque_grad(L, s, f3(t[19], t[20], t[21]), f3(t[22], t[23], t[24]), df);
    float* o = out + (size_t)i * 24;
    o[0] = f.x, o[1] = f.y, o[2] = f.z;
    for (int k = 0; k < 6; k++) o[3 + 3 * k] = df[k].x, o[4 + 3 * k] = df[k].y, o[5 + 3 * k] = df[k].z;
    o[21] = o[22] = o[23] = 0.f;
  }
}

}  // namespace lucent

using namespace lucent;

static lucent_status run_tuples(const float* tuples, uint32_t n, float* out, bool grad) {
  clear_error();
  if (n == 0) return LUCENT_OK;
  if (!tuples || !out) return fail(LUCENT_ERR_INVALID, "null argument");
  if (n > (1u << 24)) return fail(LUCENT_ERR_INVALID, "at most 16,777,216 tuples per call");
  DeviceBuffer d;
  const size_t in_b = (size_t)n * 128, out_b = (size_t)n * 96;
  lucent_status st = d.reserve(in_b + out_b + 1024);
  if (st) return st;
  float* din = (float*)d.ptr;
  float* dout = (float*)((char*)d.ptr + in_b);
  float* dlut = (float*)((char*)d.ptr + in_b + out_b);
  float lut[256];
  sheen_lut_half(lut);
  cudaError_t e = cudaMemcpy(din, tuples, in_b, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dlut, lut, sizeof lut, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    if (grad)
      k_bsdf_grad_tuples<<<grid_for(n, 256), 256>>>(din, n, dlut, dout);
    else
      k_bsdf_tuples<<<grid_for(n, 256), 256>>>(din, n, dlut, dout);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(out, dout, out_b, cudaMemcpyDeviceToHost);
  d.release();
  return e == cudaSuccess ? LUCENT_OK : cuda_fail(e, "bsdf tuples");
}

extern "C" lucent_status lucent_bsdf_eval_tuples(const float* tuples, uint32_t n, float* out) {
  return run_tuples(tuples, n, out, false);
}

extern "C" lucent_status lucent_bsdf_grad_tuples(const float* tuples, uint32_t n, float* out) {
  return run_tuples(tuples, n, out, true);
}
