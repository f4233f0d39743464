// Texture arrays of the model path (renderer.ts:314-333, context.ts:224-274):
// every image a material samples is resampled into one size x size layer of
// an sRGB array (base colour, emissive) or a linear array (metal-rough,
// normal), RGBA8. The reference draws each image through resample.frag
// (texture(uSource, gl_FragCoord.xy / uSize): mipmapped, LINEAR_MIPMAP_LINEAR,
// CLAMP_TO_EDGE, sRGB decoded before filtering and encoded on write).
//
// Here: a box-filtered mip chain (2x2 texel averages, the last row or column
// repeated on odd sizes, each level stored in the array's own format), the
// level of detail log2(max(w, h) / size) computed once per layer on the host
// in binary64, bilinear taps with edge clamping, and for sRGB layers decoding
// through a table and encoding by comparison with the table of code-value
// midpoints, so the result is exactly reproducible. Compiled with -fmad=false.
#include <cmath>
#include <cstdint>
#include <vector>

#include "api_util.h"
#include "internal.h"

namespace lucent {

namespace {

// sRGB electro-optical transfer (IEC 61966-2-1) in binary64.
double srgb_to_linear(double c) { return c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4); }

struct Level {
  const uint8_t* texels;  // RGBA8, row 0 = top
  int w, h;
};

__device__ __forceinline__ float decode(uint8_t v, int ch, const float* lut, bool srgb) {
  return (srgb && ch < 3) ? lut[v] : lut[256 + v];
}

// linear [0, 1] -> 8-bit code: sRGB by the midpoint table, linear by rounding.
__device__ __forceinline__ uint8_t encode(float c, int ch, const float* mid, bool srgb) {
  if (!(c > 0.f)) return 0;
  if (srgb && ch < 3) {
    int lo = 0, hi = 255;  // number of midpoints <= c
    while (lo < hi) {
      const int m = (lo + hi + 1) >> 1;
      if (mid[m - 1] <= c) lo = m; else hi = m - 1;
    }
    return (uint8_t)lo;
  }
  const float v = c * 255.f + 0.5f;
  return v >= 255.f ? 255 : (uint8_t)v;
}

__device__ __forceinline__ float texel(const Level& L, int x, int y, int ch, const float* lut, bool srgb) {
  x = x < 0 ? 0 : (x >= L.w ? L.w - 1 : x);
  y = y < 0 ? 0 : (y >= L.h ? L.h - 1 : y);
  return decode(L.texels[((size_t)y * L.w + x) * 4 + ch], ch, lut, srgb);
}

// Bilinear with CLAMP_TO_EDGE at normalised (u, v).
__device__ float bilinear(const Level& L, float u, float v, int ch, const float* lut, bool srgb) {
  const float x = u * (float)L.w - 0.5f, y = v * (float)L.h - 0.5f;
  const float x0 = floorf(x), y0 = floorf(y);
  const float fx = x - x0, fy = y - y0;
  const int ix = (int)x0, iy = (int)y0;
  const float a = texel(L, ix, iy, ch, lut, srgb), b = texel(L, ix + 1, iy, ch, lut, srgb);
  const float c = texel(L, ix, iy + 1, ch, lut, srgb), d = texel(L, ix + 1, iy + 1, ch, lut, srgb);
  const float top = a * (1.f - fx) + b * fx, bottom = c * (1.f - fx) + d * fx;
  return top * (1.f - fy) + bottom * fy;
}

// One mip level from the one above: 2x2 averages, edges repeated.
__global__ void k_mip(Level src, uint8_t* dst, int dw, int dh, const float* lut, const float* mid, int srgb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= dw * dh) return;
  const int x = i % dw, y = i / dw;
  for (int ch = 0; ch < 4; ch++) {
    const float s = texel(src, 2 * x, 2 * y, ch, lut, srgb) + texel(src, 2 * x + 1, 2 * y, ch, lut, srgb) +
                    texel(src, 2 * x, 2 * y + 1, ch, lut, srgb) + texel(src, 2 * x + 1, 2 * y + 1, ch, lut, srgb);
    dst[(size_t)i * 4 + ch] = encode(s * 0.25f, ch, mid, srgb);
  }
}

// One layer: texel (x, y) samples the source at ((x + 0.5) / size, (y + 0.5) / size).
__global__ void k_resample(Level l0, Level l1, float blend, int size, uint8_t* out, const float* lut, const float* mid,
                           int srgb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= size * size) return;
  const float u = ((float)(i % size) + 0.5f) / (float)size, v = ((float)(i / size) + 0.5f) / (float)size;
  for (int ch = 0; ch < 4; ch++) {
    float c = bilinear(l0, u, v, ch, lut, srgb != 0);
    if (blend > 0.f) c = c * (1.f - blend) + bilinear(l1, u, v, ch, lut, srgb != 0) * blend;
    out[(size_t)i * 4 + ch] = encode(c, ch, mid, srgb != 0);
  }
}

int next_pow2(uint32_t v) {
  int p = 1;
  while ((uint32_t)p < v && p < (1 << 30)) p <<= 1;
  return p;
}

}  // namespace

void texel_tables(float lut[512], float mid[255]) {
  for (int v = 0; v < 256; v++) {
    lut[v] = (float)srgb_to_linear(v / 255.0);
    lut[256 + v] = (float)v / 255.f;
  }
  for (int k = 0; k < 255; k++) mid[k] = (float)srgb_to_linear((k + 0.5) / 255.0);
}

int texture_array_size(const uint32_t* w, const uint32_t* h, const int32_t* layers, uint32_t n_layers) {
  if (n_layers == 0) return 0;
  uint32_t largest = 1;
  for (uint32_t i = 0; i < n_layers; i++) {
    const int t = layers[i];
    largest = w[t] > largest ? w[t] : largest;
    largest = h[t] > largest ? h[t] : largest;
  }
  int size = next_pow2(largest);
  if (size > 2048) size = 2048;
  const uint64_t budget = 256ull << 20;  // TEXTURE_BUDGET_BYTES (renderer.ts:132)
  while (size > 256 && (uint64_t)n_layers * size * size * 4 > budget) size /= 2;
  return size;
}

lucent_status build_texture_layers(const uint8_t* const* images, const uint32_t* w, const uint32_t* h,
                                   const int32_t* layers, uint32_t n_layers, int size, bool srgb, const float* lut_d,
                                   const float* mid_d, uint8_t* out_d, cudaStream_t s) {
  for (uint32_t li = 0; li < n_layers; li++) {
    const int t = layers[li];
    const int sw = (int)w[t], sh = (int)h[t];
    // Source and its mip chain down to the two levels the lookup blends.
    const double rho = (double)(sw > sh ? sw : sh) / size;
    const double lambda = rho > 1.0 ? std::log2(rho) : 0.0;
    const int d1 = (int)std::floor(lambda);
    std::vector<DeviceBuffer> levels(d1 + 2);
    std::vector<Level> L(d1 + 2);
    auto done = [&](lucent_status st) {
      cudaStreamSynchronize(s);
      for (DeviceBuffer& b : levels) b.release();
      return st;
    };
    lucent_status st = levels[0].reserve((size_t)sw * sh * 4);
    if (st) return done(st);
    cudaError_t e = cudaMemcpyAsync(levels[0].ptr, images[t], (size_t)sw * sh * 4, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return done(cuda_fail(e, "texture upload"));
    L[0] = {(const uint8_t*)levels[0].ptr, sw, sh};
    int nlev = 1;
    for (int k = 1; k <= d1 + 1; k++) {
      if (L[k - 1].w == 1 && L[k - 1].h == 1) break;
      const int dw = L[k - 1].w > 1 ? L[k - 1].w / 2 : 1, dh = L[k - 1].h > 1 ? L[k - 1].h / 2 : 1;
      if ((st = levels[k].reserve((size_t)dw * dh * 4))) return done(st);
      k_mip<<<grid_for((uint32_t)(dw * dh), 256), 256, 0, s>>>(L[k - 1], (uint8_t*)levels[k].ptr, dw, dh, lut_d, mid_d,
                                                               srgb ? 1 : 0);
      L[k] = {(const uint8_t*)levels[k].ptr, dw, dh};
      nlev = k + 1;
    }
    const int a = d1 < nlev - 1 ? d1 : nlev - 1, b = a + 1 < nlev ? a + 1 : a;
    const float blend = b > a ? (float)(lambda - d1) : 0.f;
    k_resample<<<grid_for((uint32_t)(size * size), 256), 256, 0, s>>>(
        L[a], L[b], blend, size, out_d + (size_t)li * size * size * 4, lut_d, mid_d, srgb ? 1 : 0);
    e = cudaStreamSynchronize(s);  // the level buffers are freed at the end of this iteration
    if (e == cudaSuccess) e = cudaGetLastError();
    done(LUCENT_OK);
    if (e != cudaSuccess) return cuda_fail(e, "texture resample");
  }
  return LUCENT_OK;
}

}  // namespace lucent
