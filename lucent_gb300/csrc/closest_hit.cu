// Closest-hit traversal whose results equal the reference's CPU intersector,
// intersectBVH (src/math/bvh.ts:265-320), bit for bit in the hit id.
//
// Both kernels walk the BVH in the reference's order (explicit stack, left
// child first, box test when a node is popped) and make the reference's
// decisions: the slab test with the running closest distance and a two-sided
// Moller-Trumbore with strict t < closest. `closest_exact` makes every decision
// in binary64. `closest_fast` makes each decision with f32 arithmetic whose
// error is bounded, and falls back to binary64 only when the bound cannot
// decide; accepted hits are always recomputed in binary64, so the distance it
// carries forward is the reference's value.
#include "closest_hit.cuh"
#include "internal.h"

namespace lucent {

__device__ __forceinline__ void load_ray(const float* rays, uint32_t i, float3& o, float3& d) {
  const float2* r2 = reinterpret_cast<const float2*>(rays) + (size_t)i * 3;
  const float2 a = __ldg(r2), b = __ldg(r2 + 1), c = __ldg(r2 + 2);
  o = make_float3(a.x, a.y, b.x);
  d = make_float3(b.y, c.x, c.y);
}

__device__ __forceinline__ Node load_node(const Node* nodes, int n) {
  const float4* p = reinterpret_cast<const float4*>(nodes) + 2 * (size_t)n;
  Node r;
  r.lo = __ldg(p);
  r.hi = __ldg(p + 1);
  return r;
}

struct HitOut {
  int slot;
  double t, u, v;
};

// Entire reference algorithm in binary64 (slow path and the f64-ray API).
__device__ bool trace_exact(const Node* nodes, uint32_t node_limit, const float4* tris, D3 o, D3 d, double tMin,
                            double tMax, HitOut& h, unsigned* err) {
  const D3 inv = {ddiv(1.0, d.x), ddiv(1.0, d.y), ddiv(1.0, d.z)};
  int stack[kTsStack];
  int sp = 0;
  stack[sp++] = 0;
  double closest = tMax;
  h.slot = -1;
  uint32_t iters = 0;
  while (sp > 0) {
    if (++iters > node_limit) {  // a valid BVH visits each node at most once per ray
      atomicOr(err, kErrIterations);
      return false;
    }
    const int n = stack[--sp];
    const Node nd = load_node(nodes, n);
    if (ts_slab_culled(nd.lo, nd.hi, o, inv, closest)) continue;
    const int cnt = node_count(nd), first = node_first(nd);
    if (cnt > 0) {
      for (int k = 0; k < cnt; k++) {
        const int slot = first + k;
        const float4 a = __ldg(tris + 3 * (size_t)slot), b = __ldg(tris + 3 * (size_t)slot + 1),
                     c = __ldg(tris + 3 * (size_t)slot + 2);
        double t, u, v;
        if (ts_triangle(o, d, d3f(a), d3f(b), d3f(c), tMin, closest, t, u, v)) {
          closest = t;
          h = {slot, t, u, v};
        }
      }
    } else {
      if (sp + 2 > kTsStack) {
        atomicOr(err, kErrStack);
        return false;
      }
      stack[sp++] = first + 1;
      stack[sp++] = first;
    }
  }
  return true;
}

__device__ __forceinline__ void write_hit(const float4* tris, const HitOut& h, bool ok, uint32_t i,
                                          int32_t* prim, float* tout, float* uout, float* vout) {
  if (!ok) {
    prim[i] = -2;  // traversal aborted (error word set)
  } else if (h.slot < 0) {
    prim[i] = -1;
    if (tout) tout[i] = __int_as_float(0x7f800000);
    if (uout) uout[i] = 0.f;
    if (vout) vout[i] = 0.f;
  } else {
    prim[i] = __float_as_int(__ldg(tris + 3 * (size_t)h.slot).w);
    if (tout) tout[i] = __double2float_rn(h.t);
    if (uout) uout[i] = __double2float_rn(h.u);
    if (vout) vout[i] = __double2float_rn(h.v);
  }
}

// Slow path: rays listed in `queue` (or all rays when queue == nullptr).
__global__ void k_closest_exact(const Node* __restrict__ nodes, uint32_t node_limit, const float4* __restrict__ tris,
                                const float* __restrict__ rays, uint32_t n, const uint32_t* __restrict__ queue,
                                const uint32_t* __restrict__ queue_len, double tMin, double tMax,
                                int32_t* __restrict__ prim, float* __restrict__ tout, float* __restrict__ uout,
                                float* __restrict__ vout, unsigned* err) {
  const uint32_t limit = queue ? *queue_len : n;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < limit; k += gridDim.x * blockDim.x) {
    const uint32_t i = queue ? queue[k] : k;
    float3 o, d;
    load_ray(rays, i, o, d);
    HitOut h;
    const bool ok = trace_exact(nodes, node_limit, tris, {o.x, o.y, o.z}, {d.x, d.y, d.z}, tMin, tMax, h, err);
    write_hit(tris, h, ok, i, prim, tout, uout, vout);
  }
}

// f64-ray API: rays as 6 doubles, outputs in double.
__global__ void k_closest_exact_d(const Node* __restrict__ nodes, uint32_t node_limit, const float4* __restrict__ tris,
                                  const double* __restrict__ rays, uint32_t n, double tMin, double tMax,
                                  int32_t* __restrict__ prim, double* __restrict__ tout, double* __restrict__ uout,
                                  double* __restrict__ vout, unsigned* err) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double* r = rays + (size_t)i * 6;
    HitOut h;
    const bool ok = trace_exact(nodes, node_limit, tris, {r[0], r[1], r[2]}, {r[3], r[4], r[5]}, tMin, tMax, h, err);
    if (!ok) {
      prim[i] = -2;
    } else if (h.slot < 0) {
      prim[i] = -1;
      tout[i] = __longlong_as_double(0x7ff0000000000000ll);
      uout[i] = vout[i] = 0;
    } else {
      prim[i] = __float_as_int(__ldg(tris + 3 * (size_t)h.slot).w);
      tout[i] = h.t;
      uout[i] = h.u;
      vout[i] = h.v;
    }
  }
}

// Fast path: persistent warps, one ray per lane, lanes refill from a global
// counter as their rays finish. The reference's traversal order is kept:
// both children of an inner node are tested with the current closest `c`
// (exactly what the reference's pop of the left child, and of the right one if
// the left is culled, would test); a right child that passes is pushed with an
// upper bound on its entry distance, and is re-tested when popped only if `c`
// has since dropped below that bound (the cull test is monotone in `c`).
// `c` is carried as binary32 bounds [c_lo, c_hi] of the reference's binary64
// value; the binary64 value itself is computed only when a decision needs it.
// Rays outside the bounded-error range are queued for the slow path.
struct PendingNode {
  int node;
  float ehi;
};

__device__ __forceinline__ D3 inv_exact(float3 d) {
  return {ddiv(1.0, (double)d.x), ddiv(1.0, (double)d.y), ddiv(1.0, (double)d.z)};
}

__global__ void __launch_bounds__(256, 3) k_closest_fast(const Node* __restrict__ nodes, uint32_t node_limit,
                                                      const float4* __restrict__ tris,
                                                      const float* __restrict__ rays, uint32_t n, double tMin,
                                                      double tMax, int32_t* __restrict__ prim,
                                                      float* __restrict__ tout, float* __restrict__ uout,
                                                      float* __restrict__ vout, uint32_t* __restrict__ queue,
                                                      uint32_t* __restrict__ queue_len,
                                                      uint32_t* __restrict__ work, unsigned* err) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const float tmin_lo = __double2float_rd(tMin), tmin_hi = __double2float_ru(tMin);
  const float cmax_lo = __double2float_rd(tMax), cmax_hi = __double2float_ru(tMax);
  const double INF64 = __longlong_as_double(0x7ff0000000000000ll);

  bool active = false, exhausted = false, have_cur = false, c_exact = true;
  uint32_t ri = 0, iters = 0;
  Ray32 r;
  float c_lo = 0.f, c_hi = 0.f;
  double c64 = tMax;
  int best = -1, sp = 0;
  Node cur;
  PendingNode stack[kTsStack];

  while (true) {
    // Lanes without a ray take the next ones (one atomic per warp).
    const bool need = !active && !exhausted;
    const unsigned m = __ballot_sync(FULL, need);
    if (m) {
      const int leader = __ffs(m) - 1;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(work, (uint32_t)__popc(m));
      base = __shfl_sync(FULL, base, leader);
      if (need) {
        ri = base + __popc(m & lt);
        if (ri >= n) {
          exhausted = true;
        } else {
          float3 o, d;
          load_ray(rays, ri, o, d);
          if (!safe_ray(o, d)) {
            queue[atomicAdd(queue_len, 1u)] = ri;
          } else {
            r = make_ray32(o, d);
            c_lo = cmax_lo;
            c_hi = cmax_hi;
            c64 = tMax;
            c_exact = true;
            best = -1;
            sp = 0;
            iters = 0;
            // The reference pops the root first and tests its box.
            cur = load_node(nodes, 0);
            SlabClass cl = classify_slab(r, cur.lo, cur.hi, c_lo, c_hi);
            if (cl == kAmbiguous)
              cl = ts_slab_culled(cur.lo, cur.hi, {o.x, o.y, o.z}, inv_exact(d), c64) ? kCulled : kPass;
            have_cur = cl != kCulled;
            active = true;
          }
        }
      }
    }
    if (__all_sync(FULL, exhausted)) break;
    if (!active) continue;

    // Binary64 value of c, computed on demand (the reference's t of `best`).
    auto exact_c = [&]() {
      if (!c_exact) {
        const float4 a = __ldg(tris + 3 * (size_t)best), b = __ldg(tris + 3 * (size_t)best + 1),
                     c = __ldg(tris + 3 * (size_t)best + 2);
        double t, u, v;
        ts_triangle({r.o.x, r.o.y, r.o.z}, {r.d.x, r.d.y, r.d.z}, d3f(a), d3f(b), d3f(c), tMin, INF64, t, u, v);
        c64 = t;
        c_exact = true;
        c_lo = __double2float_rd(t);
        c_hi = __double2float_ru(t);
      }
      return c64;
    };
    auto slab_decide = [&](const Node& nd, SlabClass cl) {
      if (cl != kAmbiguous) return cl;
      return ts_slab_culled(nd.lo, nd.hi, {r.o.x, r.o.y, r.o.z}, inv_exact(r.d), exact_c()) ? kCulled : kPass;
    };

    if (!have_cur) {
      if (sp == 0) {  // traversal finished: write the hit in the reference's binary64
        if (best < 0) {
          prim[ri] = -1;
          if (tout) tout[ri] = __int_as_float(0x7f800000);
          if (uout) uout[ri] = 0.f;
          if (vout) vout[ri] = 0.f;
        } else {
          const float4 a = __ldg(tris + 3 * (size_t)best), b = __ldg(tris + 3 * (size_t)best + 1),
                       c = __ldg(tris + 3 * (size_t)best + 2);
          double t = 0, u = 0, v = 0;
          ts_triangle({r.o.x, r.o.y, r.o.z}, {r.d.x, r.d.y, r.d.z}, d3f(a), d3f(b), d3f(c), tMin, INF64, t, u, v);
          prim[ri] = __float_as_int(a.w);
          if (tout) tout[ri] = __double2float_rn(t);
          if (uout) uout[ri] = __double2float_rn(u);
          if (vout) vout[ri] = __double2float_rn(v);
        }
        active = false;
        continue;
      }
      const PendingNode e = stack[--sp];
      const Node nd = load_node(nodes, e.node);
      if (e.ehi > c_lo) {
        if (slab_decide(nd, classify_slab(r, nd.lo, nd.hi, c_lo, c_hi)) == kCulled) continue;
      }
      cur = nd;
      have_cur = true;
    }
    if (++iters > node_limit) {  // a valid BVH visits each node at most once per ray
      atomicOr(err, kErrIterations);
      prim[ri] = -2;
      active = false;
      have_cur = false;
      continue;
    }
    const int cnt = node_count(cur), first = node_first(cur);
    if (cnt > 0) {
      for (int k = 0; k < cnt; k++) {
        const int slot = first + k;
        const float4 a = __ldg(tris + 3 * (size_t)slot), b = __ldg(tris + 3 * (size_t)slot + 1),
                     c = __ldg(tris + 3 * (size_t)slot + 2);
        float tl, th;
        const TriClass tc = mt_classify(r, a, b, c, tmin_lo, tmin_hi, c_lo, c_hi, tl, th);
        if (tc == kTriReject) continue;
        if (tc == kTriAccept) {
          best = slot;
          c_exact = false;
          c_lo = tl;
          c_hi = th;
          continue;
        }
        double t, u, v;
        const double cc = exact_c();
        if (ts_triangle({r.o.x, r.o.y, r.o.z}, {r.d.x, r.d.y, r.d.z}, d3f(a), d3f(b), d3f(c), tMin, cc, t, u, v)) {
          best = slot;
          c64 = t;
          c_exact = true;
          c_lo = __double2float_rd(t);
          c_hi = __double2float_ru(t);
        }
      }
      have_cur = false;
    } else {
      // Children pair (first, first + 1): one contiguous 64-byte read.
      const Node L = load_node(nodes, first), R = load_node(nodes, first + 1);
      float ehl, ehr;
      const SlabClass cl = slab_decide(L, classify_slab_e(r, L.lo, L.hi, c_lo, c_hi, ehl));
      const SlabClass cr = slab_decide(R, classify_slab_e(r, R.lo, R.hi, c_lo, c_hi, ehr));
      if (cl == kPass) {
        if (cr == kPass) {
          if (sp >= kTsStack) {  // cannot happen for BVHs shallower than the reference's stack
            atomicOr(err, kErrStack);
            prim[ri] = -2;
            active = false;
            have_cur = false;
            continue;
          }
          stack[sp++] = {first + 1, ehr};
        }
        cur = L;
      } else if (cr == kPass) {
        cur = R;
      } else {
        have_cur = false;
      }
    }
  }
}

// Reference nodes (8 floats, leftFirst/count as floats) -> device Node layout,
// with the triangles gathered into leaf (slot) order.
__global__ void k_pack_nodes(const float* __restrict__ ref, uint32_t count, Node* __restrict__ out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    const float* r = ref + (size_t)i * 8;
    Node nd;
    nd.lo = make_float4(r[0], r[1], r[2], __int_as_float((int)r[3]));
    nd.hi = make_float4(r[4], r[5], r[6], __int_as_float((int)r[7]));
    out[i] = nd;
  }
}

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

static int grid_for(uint32_t n, int block) {
  int g = (int)((n + block - 1) / block);
  return g < 1 ? 1 : (g > 65535 * 16 ? 65535 * 16 : g);
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

void launch_closest(const Node* nodes, uint32_t node_count, const float4* tris, const float* rays_d, uint32_t n, double tMin,
                    double tMax, int32_t* prim, float* t, float* u, float* v, uint32_t* queue, uint32_t* queue_len,
                    uint32_t* work, unsigned* err, bool exact_only, cudaStream_t s) {
  if (n == 0) return;
  if (exact_only) {
    k_closest_exact<<<grid_for(n, 128), 128, 0, s>>>(nodes, node_count, tris, rays_d, n, nullptr, nullptr, tMin, tMax, prim,
                                                      t, u, v, err);
    return;
  }
  static int blocks = 0;
  if (!blocks) {  // persistent grid: every SM filled to the kernel's occupancy
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_closest_fast, 256, 0);
    blocks = (sms > 0 ? sms : 152) * (per > 0 ? per : 2);
  }
  const int want = (int)((n + 255) / 256);
  k_closest_fast<<<want < blocks ? want : blocks, 256, 0, s>>>(nodes, node_count, tris, rays_d, n, tMin, tMax, prim,
                                                                t, u, v, queue, queue_len, work, err);
  // Slow path over the queued rays; the queue length is read on the device.
  k_closest_exact<<<grid_for(n < 4096 ? n : 4096, 128), 128, 0, s>>>(nodes, node_count, tris, rays_d, n, queue, queue_len,
                                                                      tMin, tMax, prim, t, u, v, err);
}

void launch_closest_d(const Node* nodes, uint32_t node_count, const float4* tris, const double* rays_d, uint32_t n, double tMin,
                      double tMax, int32_t* prim, double* t, double* u, double* v, unsigned* err, cudaStream_t s) {
  if (n == 0) return;
  k_closest_exact_d<<<grid_for(n, 128), 128, 0, s>>>(nodes, node_count, tris, rays_d, n, tMin, tMax, prim, t, u, v, err);
}

}  // namespace lucent
