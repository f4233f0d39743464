// buildEnvSampler (src/scene/environment.ts:52-85) on the GPU, with the alias
// table of buildAliasTable (src/math/alias.ts:17-65) built in parallel.
//
// Cell weights are the reference's binary64 values exactly: one thread per
// cell sums its texels' luminance in the reference's order, with sin(theta)
// per cell row from the host's libm (so the device's sin cannot differ), and
// no FMA contraction (explicit __dadd_rn / __dmul_rn).
//
// Vose's algorithm pops the small and large stacks from the top: lights
// (scaled pmf < 1) in descending index order, heavies the same; the current
// heavy serves lights until its residual drops below 1, then is itself
// topped up by the next heavy. In exact arithmetic that sweep has a closed
// form over prefix sums: with D(k) = sum of the first k+1 light deficits
// (1 - x) and C(j) = sum of the first j+1 heavy excesses (x - 1),
//   light k is served by the first heavy j with C(j) >= D(k-1)
//     (prob = x, alias = that heavy; none left: prob 1, alias itself);
//   heavy j is exhausted at the first light k with D(k) > C(j)
//     (prob = 1 + C(j) - D(k), alias = heavy j+1; the last heavy, or one
//     never exhausted, keeps prob 1 and aliases itself).
// The total and the prefix sums are deterministic double-double scans,
// exact to far below binary64 where the reference sums left to right in
// binary64 (its total and its running residuals carry about 1e-9 of
// rounding on a 1024 x 512 map). Measured on the large-mesh workload's HDRI
// (CPU emulation of these formulas against the host table): every alias and
// every pdf column equal, 3.3 % of keep probabilities different, by at most
// 1e-8; the table reproduces the pmf (the reference's own criterion,
// alias.test: each cell's probability within 5e-7) and never draws a
// zero-weight cell.
#include <cmath>
#include <vector>

#include "../../include/lucent.h"
#include "api_util.h"
#include "internal.h"

namespace lucent {
namespace envs {

constexpr int kScanBlock = 1024;

// Weight of cell i: mean luminance of its texels times sin(theta) of its row.
__global__ void k_weights(const float* __restrict__ rgb, uint32_t w, uint32_t h, uint32_t gw, uint32_t gh,
                          const double* __restrict__ sin_row, double* __restrict__ weight, unsigned* __restrict__ bad) {
  const uint32_t n = gw * gh;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t cy = i / gw, cx = i % gw;
    const uint64_t y0 = (uint64_t)floor(__ddiv_rn((double)cy * (double)h, (double)gh));
    const uint64_t y1v = (uint64_t)floor(__ddiv_rn((double)(cy + 1) * (double)h, (double)gh));
    const uint64_t y1 = y1v > y0 + 1 ? y1v : y0 + 1;
    const uint64_t x0 = (uint64_t)floor(__ddiv_rn((double)cx * (double)w, (double)gw));
    const uint64_t x1v = (uint64_t)floor(__ddiv_rn((double)(cx + 1) * (double)w, (double)gw));
    const uint64_t x1 = x1v > x0 + 1 ? x1v : x0 + 1;
    double sum = 0;
    for (uint64_t y = y0; y < y1; y++)
      for (uint64_t x = x0; x < x1; x++) {
        const float* p = rgb + (y * w + x) * 3;
        const double l = __dadd_rn(__dadd_rn(__dmul_rn(0.2126, (double)p[0]), __dmul_rn(0.7152, (double)p[1])),
                                   __dmul_rn(0.0722, (double)p[2]));
        sum = __dadd_rn(sum, l);
      }
    const double wt = __dmul_rn(__ddiv_rn(sum, (double)((y1 - y0) * (x1 - x0))), sin_row[cy]);
    if (!(wt >= 0) || isinf(wt)) atomicOr(bad, 1u);
    weight[i] = wt;
  }
}

// Double-double values (hi, lo) with hi = RN(hi + lo): the scans below keep
// about 106 bits, so prefix sums of up to 2^20 terms, and the differences
// of two of them, carry no rounding that matters at binary64 or binary32
// precision (a plain binary64 scan of 5e5 deficits lost about 1e-9 in the
// difference of two sums near 1e5 and moved 4 % of the keep probabilities
// by one binary32 ulp).
__device__ __forceinline__ double2 dd_two_sum(double a, double b) {
  const double s = __dadd_rn(a, b), bb = __dsub_rn(s, a);
  return make_double2(s, __dadd_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dsub_rn(b, bb)));
}
__device__ __forceinline__ double2 dd_norm(double hi, double lo) {
  const double s = __dadd_rn(hi, lo);
  return make_double2(s, __dsub_rn(lo, __dsub_rn(s, hi)));
}
__device__ __forceinline__ double2 dd_add(double2 a, double2 b) {
  double2 s = dd_two_sum(a.x, b.x);
  const double2 t = dd_two_sum(a.y, b.y);
  s = dd_norm(s.x, __dadd_rn(s.y, t.x));
  return dd_norm(s.x, __dadd_rn(s.y, t.y));
}
__device__ __forceinline__ double2 dd_neg(double2 a) { return make_double2(-a.x, -a.y); }
__device__ __forceinline__ bool dd_less(double2 a, double2 b) { return a.x < b.x || (a.x == b.x && a.y < b.y); }
// binary32 rounding of a double-double (ties to even, on the exact value).
__device__ __forceinline__ float dd_to_float(double2 a) {
  const float f = __double2float_rn(a.x);
  const double r = __dsub_rn(a.x, (double)f);  // exact: f is a rounding of a.x
  if (r == 0 || a.y == 0) return f;
  const double half = 0.5 * ((double)nextafterf(fabsf(f), INFINITY) - (double)fabsf(f));
  if (fabs(r) != half) return f;  // a.x is not a tie: a.y (far smaller) cannot move the rounding
  // a.x sits exactly halfway: the sign of a.y breaks the tie
  const bool up = (r > 0) == (a.y > 0);
  return up ? (r > 0 ? nextafterf(f, INFINITY) : nextafterf(f, -INFINITY)) : f;
}

__device__ __forceinline__ double2 as_dd(double v) { return make_double2(v, 0.0); }
__device__ __forceinline__ double2 as_dd(double2 v) { return v; }

// Block-wise inclusive scan (Hillis-Steele in double-double: a fixed order,
// deterministic); 1024 threads a block.
__device__ __forceinline__ double2 block_scan(double2 x, double2* sh) {
  const int t = threadIdx.x;
  sh[t] = x;
  __syncthreads();
  for (int o = 1; o < kScanBlock; o <<= 1) {
    const double2 y = t >= o ? sh[t - o] : make_double2(0.0, 0.0);
    __syncthreads();
    if (t >= o) sh[t] = dd_add(sh[t], y);
    __syncthreads();
  }
  return sh[t];
}

template <class T>
__global__ void __launch_bounds__(kScanBlock) k_scan_blocks(const T* __restrict__ v, uint32_t n,
                                                            double2* __restrict__ out, double2* __restrict__ part) {
  __shared__ double2 sh[kScanBlock];
  const uint32_t i = blockIdx.x * kScanBlock + threadIdx.x;
  const double2 s = block_scan(i < n ? as_dd(v[i]) : make_double2(0.0, 0.0), sh);
  if (i < n) out[i] = s;
  if (threadIdx.x == kScanBlock - 1) part[blockIdx.x] = s;
}

// Exclusive scan of the (at most 1024) block totals in place, one block.
__global__ void __launch_bounds__(kScanBlock) k_scan_parts(double2* __restrict__ part, uint32_t m) {
  __shared__ double2 sh[kScanBlock];
  const uint32_t t = threadIdx.x;
  block_scan(t < m ? part[t] : make_double2(0.0, 0.0), sh);  // ends with a barrier
  if (t < m) part[t] = t == 0 ? make_double2(0.0, 0.0) : sh[t - 1];
}

__global__ void k_scan_add(double2* __restrict__ out, uint32_t n, const double2* __restrict__ part) {
  const uint32_t i = blockIdx.x * kScanBlock + threadIdx.x;
  if (i < n && blockIdx.x > 0) out[i] = dd_add(out[i], part[blockIdx.x]);
}

// x_i = pmf_i * n with pmf = w / total (1/n for a black map); light flags for
// the index scan, taken in descending index order (position r = n - 1 - i),
// the order in which the reference pops its stacks.
__global__ void k_classify(const double* __restrict__ weight, uint32_t n, const double2* __restrict__ total_p,
                           double* __restrict__ pmf, double* __restrict__ x, double* __restrict__ light_rev) {
  const double total = total_p->x;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double p = total > 0 ? __ddiv_rn(weight[i], total) : __ddiv_rn(1.0, (double)n);
    const double xi = __dmul_rn(p, (double)n);
    pmf[i] = p;
    x[i] = xi;
    light_rev[n - 1 - i] = xi < 1 ? 1.0 : 0.0;
  }
}

// Compacts lights and heavies (descending index) with their exact deficit
// 1 - x / excess x - 1 as double-doubles.
__global__ void k_split(const double* __restrict__ x, uint32_t n, const double2* __restrict__ light_incl,
                        uint32_t* __restrict__ L, double2* __restrict__ deficit, uint32_t* __restrict__ H,
                        double2* __restrict__ excess) {
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    const uint32_t i = n - 1 - r;
    const bool light = x[i] < 1;
    const uint32_t lights_before = (uint32_t)light_incl[r].x - (light ? 1u : 0u);
    if (light) {
      L[lights_before] = i;
      deficit[lights_before] = dd_two_sum(1.0, -x[i]);
    } else {
      const uint32_t k = r - lights_before;
      H[k] = i;
      excess[k] = dd_two_sum(x[i], -1.0);
    }
  }
}

// First index in sorted a[0..m) with a[idx] >= v (lower) or > v (upper).
__device__ __forceinline__ uint32_t bound(const double2* a, uint32_t m, double2 v, bool upper) {
  uint32_t lo = 0, hi = m;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    const bool go_right = upper ? !dd_less(v, a[mid]) : dd_less(a[mid], v);
    if (go_right) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

__global__ void k_serve(const uint32_t* __restrict__ L, uint32_t nl, const double2* __restrict__ D,
                        const uint32_t* __restrict__ H, uint32_t nh, const double2* __restrict__ C,
                        const double* __restrict__ x, float* __restrict__ prob, uint32_t* __restrict__ alias) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nl + nh; k += gridDim.x * blockDim.x) {
    if (k < nl) {  // light k, served by the first heavy with C(j) >= D(k-1)
      const uint32_t i = L[k];
      const uint32_t j = bound(C, nh, k > 0 ? D[k - 1] : make_double2(0.0, 0.0), false);
      if (j < nh) {
        prob[i] = (float)x[i];
        alias[i] = H[j];
      } else {
        prob[i] = 1.f;
        alias[i] = i;
      }
    } else {  // heavy j, exhausted at the first light with D(k) > C(j)
      const uint32_t j = k - nl, i = H[j];
      const uint32_t e = bound(D, nl, C[j], true);
      if (e < nl && j + 1 < nh) {
        prob[i] = dd_to_float(dd_add(dd_add(C[j], dd_neg(D[e])), make_double2(1.0, 0.0)));
        alias[i] = H[j + 1];
      } else {
        prob[i] = 1.f;
        alias[i] = i;
      }
    }
  }
}

// 4 floats per cell: keep probability, alias cell, pdfUV, alias pdfUV.
__global__ void k_table(const float* __restrict__ prob, const uint32_t* __restrict__ alias,
                        const double* __restrict__ pmf, uint32_t n, float4* __restrict__ table) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t a = alias[i];
    table[i] = make_float4(prob[i], (float)a, (float)__dmul_rn(pmf[i], (double)n), (float)__dmul_rn(pmf[a], (double)n));
  }
}

// Inclusive double-double scan of v[0..n) into out (n <= 1024 * 1024); part:
// 1024 double-doubles.
template <class T>
static void scan(const T* v, uint32_t n, double2* out, double2* part, cudaStream_t s) {
  const uint32_t blocks = (n + kScanBlock - 1) / kScanBlock;
  k_scan_blocks<T><<<blocks, kScanBlock, 0, s>>>(v, n, out, part);
  k_scan_parts<<<1, kScanBlock, 0, s>>>(part, blocks);
  k_scan_add<<<blocks, kScanBlock, 0, s>>>(out, n, part);
}

}  // namespace envs

// Grid of the sampler for a w x h map (environment.ts:53-54).
void env_grid(uint32_t w, uint32_t h, uint32_t max_w, uint32_t& gw, uint32_t& gh) {
  gw = std::max(1u, std::min(w, max_w));
  gh = std::max(1u, std::min(h, (uint32_t)std::floor((double)h * gw / w + 0.5)));
}

lucent_status gpu_env_sampler(const float* rgb_d, uint32_t w, uint32_t h, uint32_t max_w, uint32_t& gw, uint32_t& gh,
                              float4* table_d, double& total, cudaStream_t s) {
  using namespace envs;
  env_grid(w, h, max_w, gw, gh);
  const uint32_t n = gw * gh;
  if (n > (uint32_t)kScanBlock * kScanBlock)
    return fail(LUCENT_ERR_UNSUPPORTED, "%u sampler cells; the device build takes at most %u", n,
                (uint32_t)kScanBlock * kScanBlock);
  std::vector<double> sin_row(gh);
  for (uint32_t cy = 0; cy < gh; cy++) sin_row[cy] = std::sin(M_PI * (cy + 0.5) / gh);
  // Scratch, carved in 256-byte aligned pieces: sin rows, 4 arrays of n
  // doubles, 5 of n double-doubles, 3 of n uint32, the scans' block totals
  // and the error word.
  const size_t dbl = 8 * (size_t)n, dd = 16 * (size_t)n;
  auto piece = [](size_t sz) { return (sz + 255) & ~(size_t)255; };
  const size_t bytes = piece(8 * (size_t)gh) + 4 * piece(dbl) + 5 * piece(dd) + 3 * piece(4 * (size_t)n) +
                       piece(16 * (size_t)kScanBlock) + piece(16);
  DeviceBuffer buf;
  lucent_status st = buf.reserve(bytes);
  if (st) return st;
  char* b = (char*)buf.ptr;
  char* const end = b + bytes;
  auto take = [&](size_t sz) {
    char* p = b;
    b += piece(sz);
    return p;
  };
  double* sin_d = (double*)take(8 * (size_t)gh);
  double* weight = (double*)take(dbl);
  double* pmf = (double*)take(dbl);
  double* x = (double*)take(dbl);
  double* light = (double*)take(dbl);
  double2* wsum = (double2*)take(dd);
  double2* light_incl = (double2*)take(dd);
  double2* deficit = (double2*)take(dd);
  double2* excess = (double2*)take(dd);
  double2* DC = (double2*)take(dd);  // D in [0, nl), C in [nl, n)
  uint32_t* L = (uint32_t*)take(4 * (size_t)n);
  uint32_t* H = (uint32_t*)take(4 * (size_t)n);
  uint32_t* alias = (uint32_t*)take(4 * (size_t)n);
  double2* part = (double2*)take(16 * (size_t)kScanBlock);
  unsigned* bad = (unsigned*)take(16);
  if (b > end) {  // the pieces above must add up to `bytes`
    buf.release();
    return fail(LUCENT_ERR_DEVICE, "environment sampler scratch layout");
  }
  float* prob = (float*)wsum;  // wsum is dead once the total is read
  const int g = grid_for(n, 256);
  cudaError_t e = cudaMemcpyAsync(sin_d, sin_row.data(), 8 * (size_t)gh, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(bad, 0, 4, s);
  if (e != cudaSuccess) {
    buf.release();
    return cuda_fail(e, "environment sampler upload");
  }
  k_weights<<<g, 256, 0, s>>>(rgb_d, w, h, gw, gh, sin_d, weight, bad);
  scan(weight, n, wsum, part, s);  // total = the last inclusive sum
  k_classify<<<g, 256, 0, s>>>(weight, n, wsum + (n - 1), pmf, x, light);
  scan(light, n, light_incl, part, s);
  uint32_t nl = 0;
  unsigned bad_h = 0;
  double2 nl_d = {0, 0}, total_d = {0, 0};
  e = cudaMemcpyAsync(&nl_d, light_incl + (n - 1), 16, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&total_d, wsum + (n - 1), 16, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&bad_h, bad, 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    buf.release();
    return cuda_fail(e, "environment sampler weights");
  }
  if (bad_h) {
    buf.release();
    return fail(LUCENT_ERR_INVALID, "environment weights must be finite and >= 0");
  }
  total = total_d.x;
  nl = (uint32_t)nl_d.x;
  const uint32_t nh = n - nl;
  k_split<<<g, 256, 0, s>>>(x, n, light_incl, L, deficit, H, excess);
  if (nl) scan(deficit, nl, DC, part, s);
  if (nh) scan(excess, nh, DC + nl, part, s);
  k_serve<<<g, 256, 0, s>>>(L, nl, DC, H, nh, DC + nl, x, prob, alias);
  k_table<<<g, 256, 0, s>>>(prob, alias, pmf, n, table_d);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  buf.release();
  return e == cudaSuccess ? LUCENT_OK : cuda_fail(e, "environment sampler build");
}

}  // namespace lucent

using namespace lucent;

extern "C" lucent_status lucent_env_sampler_device(const float* rgb_d, uint32_t width, uint32_t height,
                                                   uint32_t max_width, uint32_t* gw, uint32_t* gh, float* table_d,
                                                   double* total, void* stream) {
  clear_error();
  if (!rgb_d || !gw || !gh || !table_d || width == 0 || height == 0 || max_width == 0)
    return fail(LUCENT_ERR_INVALID, "null argument or empty image");
  double t = 0;
  lucent_status st = gpu_env_sampler(rgb_d, width, height, max_width, *gw, *gh, (float4*)table_d, t,
                                     (cudaStream_t)stream);
  if (!st && total) *total = t;
  return st;
}
