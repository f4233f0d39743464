// Binary64 vector, slab and triangle arithmetic of the reference's CPU code
// (src/math/vec3.ts, src/math/aabb.ts, src/math/ray.ts), shared by the oracle
// files. Compiled with -ffp-contract=off: each operation rounds once, as in JS.
#pragma once
#include <cmath>
#include <limits>
#include <utility>

namespace orc {

const double INF = std::numeric_limits<double>::infinity();

struct V3 {
  double x, y, z;
};
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }

// intersectTriangle, src/math/ray.ts:22-45.
inline bool tri_hit(V3 o, V3 d, V3 v0, V3 v1, V3 v2, double tMin, double tMax, double& t, double& u, double& v) {
  V3 e1 = sub(v1, v0);
  V3 e2 = sub(v2, v0);
  V3 p = cross(d, e2);
  double det = dot(e1, p);
  if (std::fabs(det) < 1e-12) return false;
  double invDet = 1.0 / det;
  V3 s = sub(o, v0);
  double uu = dot(s, p) * invDet;
  if (uu < 0 || uu > 1) return false;
  V3 q = cross(s, e1);
  double vv = dot(d, q) * invDet;
  if (vv < 0 || uu + vv > 1) return false;
  double tt = dot(e2, q) * invDet;
  if (tt <= tMin || tt >= tMax) return false;
  t = tt;
  u = uu;
  v = vv;
  return true;
}

// AABB.intersect, src/math/aabb.ts:84-98: entry distance or +inf.
inline double slab(const double* mn, const double* mx, const double* o, const double* inv, double tMax) {
  double tmin = 0;
  double tmax = tMax;
  for (int i = 0; i < 3; i++) {
    double t0 = (mn[i] - o[i]) * inv[i];
    double t1 = (mx[i] - o[i]) * inv[i];
    if (t0 > t1) std::swap(t0, t1);
    if (t0 > tmin) tmin = t0;
    if (t1 < tmax) tmax = t1;
    if (tmax < tmin) return INF;
  }
  return tmin;
}

}  // namespace orc
