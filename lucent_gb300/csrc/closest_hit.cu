// BVH API instantiation of the shared traversal kernels (traverse.cuh):
// rays as 6 floats (or doubles) each, results per ray, hit ids equal to the
// reference's intersectBVH (src/math/bvh.ts:265-320).
#include "internal.h"
#include "traverse_wide.cuh"

namespace lucent {

__device__ __forceinline__ void load_ray6(const float* rays, uint32_t i, float3& o, float3& d) {
  const float2* r2 = reinterpret_cast<const float2*>(rays) + (size_t)i * 3;
  const float2 a = __ldg(r2), b = __ldg(r2 + 1), c = __ldg(r2 + 2);
  o = make_float3(a.x, a.y, b.x);
  d = make_float3(b.y, c.x, c.y);
}

// Rays from a float array; results in prim/t/u/v (binary64 values rounded to
// binary32). The triangle's source index sits in v0.w.
struct ApiPolicy {
  const float* rays;
  uint32_t n;
  const float4* tris;
  int32_t* prim;
  float *tout, *uout, *vout;
  double tmin;
  __device__ uint32_t count() const { return n; }
  __device__ void ray(uint32_t k, float3& o, float3& d) const { load_ray6(rays, k, o, d); }
  __device__ uint32_t key(uint32_t) const { return 0; }
  static constexpr bool kMultiScene = false;
  static constexpr int kThreads = 128, kMinBlocks = 7;  // closest-hit block shape
  // Lanes of a wide-kernel warp that wait before it fetches new rays
  // (measured on 10^6 random rays into a 65,536-triangle soup: 4 over 1, 8, 16).
  static constexpr int kRefillMin = 4;
  __device__ bool alpha(int, int, uint32_t, float, float) const { return true; }
  __device__ AlphaAnswer alpha_fast(int, int, uint32_t) const { return kAlphaBlock; }
  __device__ bool alpha_any() const { return false; }
  // The hit triangle, encoded -3 - slot until k_refine_api computes its
  // values with the warp converged (lanes finish their rays at different
  // steps, so per-ray arithmetic here would run one lane at a time).
  __device__ void finish(uint32_t k, int slot) const { prim[k] = -3 - slot; }
  __device__ void hit(uint32_t k, int slot, double t, double u, double v) const {
    prim[k] = __float_as_int(__ldg(tris + 3 * (size_t)slot).w);
    if (tout) tout[k] = __double2float_rn(t);
    if (uout) uout[k] = __double2float_rn(u);
    if (vout) vout[k] = __double2float_rn(v);
  }
  __device__ void miss(uint32_t k) const {
    prim[k] = -1;
    if (tout) tout[k] = __int_as_float(0x7f800000);
    if (uout) uout[k] = 0.f;
    if (vout) vout[k] = 0.f;
  }
  __device__ void fail(uint32_t k) const { prim[k] = -2; }
};

// f64-ray API: rays as 6 doubles, outputs in binary64 (always the exact path).
__global__ void k_closest_exact_d(TravArgs A, const double* __restrict__ rays, uint32_t n, int32_t* __restrict__ prim,
                                  double* __restrict__ tout, double* __restrict__ uout, double* __restrict__ vout) {
  ApiPolicy P{};
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double* r = rays + (size_t)i * 6;
    int slot;
    double t = 0, u = 0, v = 0;
    if (!trace_exact(A, P, bvh_of(A, P, i), {r[0], r[1], r[2]}, {r[3], r[4], r[5]}, 0, slot, t, u, v)) {
      prim[i] = -2;
    } else if (slot < 0) {
      prim[i] = -1;
      tout[i] = __longlong_as_double(0x7ff0000000000000ll);
      uout[i] = vout[i] = 0;
    } else {
      prim[i] = __float_as_int(__ldg(A.tris + 3 * (size_t)slot).w);
      tout[i] = t;
      uout[i] = u;
      vout[i] = v;
    }
  }
}

// The values of the hits the traversal found (prim = -3 - slot): the
// reference's binary64 t, u, v rounded to binary32, from double-float
// arithmetic where its bound proves the roundings of all three, else from
// binary64; prim becomes the triangle's source index. One thread per ray.
__global__ void k_refine_api(ApiPolicy P) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < P.n; k += gridDim.x * blockDim.x) {
    const int32_t code = P.prim[k];
    if (code > -3) continue;
    const int slot = -3 - code;
    float3 o, d;
    P.ray(k, o, d);
    const float4 a = __ldg(P.tris + 3 * (size_t)slot), b = __ldg(P.tris + 3 * (size_t)slot + 1),
                 c = __ldg(P.tris + 3 * (size_t)slot + 2);
    float3 tuv;
    if (tri_df32(o, d, a, b, c, true, tuv)) {
      P.hit(k, slot, tuv.x, tuv.y, tuv.z);
    } else {
      const Tri64 h = tri_f64(o, d, a, b, c, P.tmin, __longlong_as_double(0x7ff0000000000000ll));
      P.hit(k, slot, h.t, h.u, h.v);
    }
  }
}

// Reference nodes (8 floats, leftFirst/count as floats) -> device Node layout.
__global__ void k_pack_nodes(const float* __restrict__ ref, uint32_t count, Node* __restrict__ out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    const float* r = ref + (size_t)i * 8;
    Node nd;
    nd.lo = make_float4(r[0], r[1], r[2], __int_as_float((int)r[3]));
    nd.hi = make_float4(r[4], r[5], r[6], __int_as_float((int)r[7]));
    out[i] = nd;
  }
}

// Triangles gathered into leaf (slot) order, source index in v0.w.
__global__ void k_gather_tris(const float* __restrict__ pos, const uint32_t* __restrict__ tri_indices,
                              uint32_t tri_count, float4* __restrict__ out) {
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < tri_count; s += gridDim.x * blockDim.x) {
    const uint32_t src = tri_indices[s];
    const float* p = pos + (size_t)src * 9;
    out[3 * (size_t)s] = make_float4(p[0], p[1], p[2], __int_as_float((int)src));
    out[3 * (size_t)s + 1] = make_float4(p[3], p[4], p[5], 0.f);
    out[3 * (size_t)s + 2] = make_float4(p[6], p[7], p[8], 0.f);
  }
}

// Inverse of the two kernels above: back to the reference's layout.
__global__ void k_unpack(const Node* __restrict__ nodes, uint32_t count, const float4* __restrict__ tris,
                         uint32_t tri_count, float* __restrict__ ref, uint32_t* __restrict__ tri_indices) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count || i < tri_count; i += gridDim.x * blockDim.x) {
    if (i < count) {
      const Node nd = nodes[i];
      float* r = ref + (size_t)i * 8;
      r[0] = nd.lo.x, r[1] = nd.lo.y, r[2] = nd.lo.z, r[3] = (float)node_first(nd);
      r[4] = nd.hi.x, r[5] = nd.hi.y, r[6] = nd.hi.z, r[7] = (float)node_count(nd);
    }
    if (i < tri_count) tri_indices[i] = (uint32_t)__float_as_int(tris[3 * (size_t)i].w);
  }
}

int grid_for(uint32_t n, int block) {
  int g = (int)((n + block - 1) / block);
  return g < 1 ? 1 : (g > 65535 * 16 ? 65535 * 16 : g);
}

int persistent_blocks(const void* kernel, int block) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, block, 0);
  return (sms > 0 ? sms : 152) * (per > 0 ? per : 2);
}

void launch_pack_nodes(const float* ref_d, uint32_t count, Node* out_d, cudaStream_t s) {
  k_pack_nodes<<<grid_for(count, 256), 256, 0, s>>>(ref_d, count, out_d);
}

void launch_gather_tris(const float* pos_d, const uint32_t* idx_d, uint32_t tri_count, float4* out_d,
                        cudaStream_t s) {
  k_gather_tris<<<grid_for(tri_count, 256), 256, 0, s>>>(pos_d, idx_d, tri_count, out_d);
}

void launch_unpack(const Node* nodes, uint32_t count, const float4* tris, uint32_t tri_count, float* ref_d,
                   uint32_t* idx_d, cudaStream_t s) {
  k_unpack<<<grid_for(count > tri_count ? count : tri_count, 256), 256, 0, s>>>(nodes, count, tris, tri_count, ref_d,
                                                                                idx_d);
}

void launch_closest(const Node* nodes, uint32_t node_count, const float4* tris, const float* rays_d, uint32_t n,
                    double tMin, double tMax, int32_t* prim, float* t, float* u, float* v, uint32_t* queue,
                    uint32_t* queue_len, uint32_t* work, unsigned* err, bool exact_only, bool top_levels,
                    cudaStream_t s, const Node* wide) {
  if (n == 0) return;
  const ApiPolicy P{rays_d, n, tris, prim, t, u, v, tMin};
  TravArgs A{nodes, node_count, tris, tMin, tMax, queue, queue_len, work, err, nullptr, top_levels ? 1 : 0};
  if (exact_only) {
    TravArgs E = A;
    E.queue = nullptr;
    k_closest_exact_t<ApiPolicy><<<grid_for(n, 128), 128, 0, s>>>(E, P);
    return;
  }
  static int blocks = 0, wide_blocks = 0;
  if (!blocks) {
    blocks = persistent_blocks((const void*)k_closest_fast_t<ApiPolicy>, ApiPolicy::kThreads);
    wide_blocks = persistent_blocks((const void*)k_closest_wide_t<ApiPolicy>, ApiPolicy::kThreads);
  }
  const int want = (int)((n + ApiPolicy::kThreads - 1) / ApiPolicy::kThreads);
  if (wide) {
    A.wide = wide;
    A.top_scenes = 0;
    k_closest_wide_t<ApiPolicy><<<want < wide_blocks ? want : wide_blocks, ApiPolicy::kThreads, 0, s>>>(A, P);
  } else {
    k_closest_fast_t<ApiPolicy><<<want < blocks ? want : blocks, ApiPolicy::kThreads, top_smem_bytes(A.top_scenes), s>>>(A, P);
  }
  // Slow path over the rays the fast kernel queued (length read on the device).
  k_closest_exact_t<ApiPolicy><<<grid_for(n < 4096 ? n : 4096, 128), 128, 0, s>>>(A, P);
  k_refine_api<<<grid_for(n, 256), 256, 0, s>>>(P);
}

void launch_wide_view(const Node* nodes, uint32_t node_count, Node* wide, cudaStream_t s) {
  launch_build_wide(nodes, node_count, wide, s);
}

void launch_closest_d(const Node* nodes, uint32_t node_count, const float4* tris, const double* rays_d, uint32_t n,
                      double tMin, double tMax, int32_t* prim, double* t, double* u, double* v, unsigned* err,
                      cudaStream_t s) {
  if (n == 0) return;
  TravArgs A{nodes, node_count, tris, tMin, tMax, nullptr, nullptr, nullptr, err};
  k_closest_exact_d<<<grid_for(n, 128), 128, 0, s>>>(A, rays_d, n, prim, t, u, v);
}

}  // namespace lucent
