// Shared device helpers for the Lucent GB300 kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define LUCENT_DEV __device__ __forceinline__

namespace lucent {

// ---------------------------------------------------------------------------
// Binary64 arithmetic that can never be contracted into an FMA, so results
// equal JavaScript's `number` arithmetic operation by operation.
// ---------------------------------------------------------------------------
LUCENT_DEV double dadd(double a, double b) { return __dadd_rn(a, b); }
LUCENT_DEV double dsub(double a, double b) { return __dsub_rn(a, b); }
LUCENT_DEV double dmul(double a, double b) { return __dmul_rn(a, b); }
LUCENT_DEV double ddiv(double a, double b) { return __ddiv_rn(a, b); }

struct D3 {
  double x, y, z;
};
LUCENT_DEV D3 d3sub(D3 a, D3 b) { return {dsub(a.x, b.x), dsub(a.y, b.y), dsub(a.z, b.z)}; }
// dot (src/math/vec3.ts:20): ((a0*b0 + a1*b1) + a2*b2)
LUCENT_DEV double d3dot(D3 a, D3 b) { return dadd(dadd(dmul(a.x, b.x), dmul(a.y, b.y)), dmul(a.z, b.z)); }
// cross (src/math/vec3.ts:21-25)
LUCENT_DEV D3 d3cross(D3 a, D3 b) {
  return {dsub(dmul(a.y, b.z), dmul(a.z, b.y)), dsub(dmul(a.z, b.x), dmul(a.x, b.z)),
          dsub(dmul(a.x, b.y), dmul(a.y, b.x))};
}
LUCENT_DEV D3 d3f(float4 v) { return {(double)v.x, (double)v.y, (double)v.z}; }

// intersectTriangle (src/math/ray.ts:22-45), binary64, two-sided.
LUCENT_DEV bool ts_triangle(D3 o, D3 d, D3 v0, D3 v1, D3 v2, double tMin, double tMax, double& t, double& u,
                            double& v) {
  const D3 e1 = d3sub(v1, v0), e2 = d3sub(v2, v0);
  const D3 p = d3cross(d, e2);
  const double det = d3dot(e1, p);
  if (fabs(det) < 1e-12) return false;
  const double invDet = ddiv(1.0, det);
  const D3 s = d3sub(o, v0);
  const double uu = dmul(d3dot(s, p), invDet);
  if (uu < 0 || uu > 1) return false;
  const D3 q = d3cross(s, e1);
  const double vv = dmul(d3dot(d, q), invDet);
  if (vv < 0 || dadd(uu, vv) > 1) return false;
  const double tt = dmul(d3dot(e2, q), invDet);
  if (tt <= tMin || tt >= tMax) return false;
  t = tt;
  u = uu;
  v = vv;
  return true;
}

// AABB.intersect (src/math/aabb.ts:84-98) as a culling predicate: true when
// the reference returns Infinity. NaN comparisons are false, as in JS.
LUCENT_DEV bool ts_slab_culled(float4 mn, float4 mx, D3 o, D3 inv, double tMax) {
  double tmin = 0, tmax = tMax;
  const double lo[3] = {(double)mn.x, (double)mn.y, (double)mn.z};
  const double hi[3] = {(double)mx.x, (double)mx.y, (double)mx.z};
  const double oo[3] = {o.x, o.y, o.z};
  const double iv[3] = {inv.x, inv.y, inv.z};
#pragma unroll
  for (int i = 0; i < 3; i++) {
    double t0 = dmul(dsub(lo[i], oo[i]), iv[i]);
    double t1 = dmul(dsub(hi[i], oo[i]), iv[i]);
    if (t0 > t1) {
      const double s = t0;
      t0 = t1;
      t1 = s;
    }
    if (t0 > tmin) tmin = t0;
    if (t1 < tmax) tmax = t1;
    if (tmax < tmin) return true;
  }
  return false;
}

// ---------------------------------------------------------------------------
// Device layouts.
//   Node (32 B, two float4): (min.xyz, int leftFirst), (max.xyz, int count),
//   the reference's 8-float node (src/math/bvh.ts:6-16) with the two integer
//   fields stored as int bits instead of floats.
//   Triangle (48 B, three float4) in BVH leaf (slot) order:
//   (v0, int source index), (v1, int material/light word), (v2, int flags).
// ---------------------------------------------------------------------------
struct Node {
  float4 lo;  // w: leftFirst (int bits)
  float4 hi;  // w: count (int bits)
};

LUCENT_DEV int node_first(const Node& n) { return __float_as_int(n.lo.w); }
LUCENT_DEV int node_count(const Node& n) { return __float_as_int(n.hi.w); }

constexpr int kTsStack = 64;  // the reference's Int32Array(64) (bvh.ts:276)

// Alpha test answers of the binary32 traversal kernels: the hit counts, it
// passes through, or it needs a texture lookup done by the binary64 kernel.
enum AlphaAnswer { kAlphaPass = 0, kAlphaBlock = 1, kAlphaDefer = 2 };

// Device error word bits (read by the host after a launch).
enum : unsigned {
  kErrStack = 1u,       // a traversal needed more than the reference's 64 stack entries
  kErrIterations = 2u,  // a bounded loop hit its iteration cap
  kErrQueue = 4u,       // a work queue overflowed
  kErrTree = 8u,        // a caller-supplied device tree failed its check (no-allocation entry point)
};

}  // namespace lucent
