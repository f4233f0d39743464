/*
 * Lucent oracle, BVH / ray / alias / environment / sheen part.
 *
 * TEST INFRASTRUCTURE ONLY: this is the checker that tests/, the smoke entry
 * point and bench.py's CPU-baseline leg compare the CUDA product against. The
 * product never links it.
 *
 * Restates, in C++ with JavaScript's number semantics (binary64 arithmetic,
 * binary32 rounding at every Float32Array store), the reference's:
 *   src/math/bvh.ts, src/math/aabb.ts, src/math/ray.ts, src/math/alias.ts,
 *   src/scene/environment.ts, src/scene/sheen.ts.
 * Build flags (see oracle/build_oracle.py): -O2 -ffp-contract=off -fno-fast-math.
 */
#include "lucent_oracle.h"
#include "oracle_core.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

namespace {

// Binary64 vector / slab / triangle arithmetic (vec3.ts, aabb.ts, ray.ts).
using namespace orc;

inline V3 vtx(const float* pos, uint32_t tri, int k) {
  const float* p = pos + (uint64_t)tri * 9 + k * 3;
  return {(double)p[0], (double)p[1], (double)p[2]};
}

struct Hit {
  int32_t id;
  double t, u, v;
};

// intersectBVH, src/math/bvh.ts:265-320. Returns false on a stack overflow
// (the reference's Int32Array(64) would silently drop the push).
bool bvh_closest(const float* nodes, const uint32_t* tri, uint32_t triCount, const float* pos, V3 o, V3 d,
                 double tMin, double tMax, Hit& out) {
  out = {-1, INF, 0, 0};
  if (triCount == 0) return true;
  const double org[3] = {o.x, o.y, o.z};
  const double inv[3] = {1.0 / d.x, 1.0 / d.y, 1.0 / d.z};
  int32_t stack[64];
  int sp = 0;
  stack[sp++] = 0;
  double closest = tMax;
  while (sp > 0) {
    int32_t n = stack[--sp];
    const float* nd = nodes + (uint64_t)n * 8;
    const double mn[3] = {nd[0], nd[1], nd[2]};
    const double mx[3] = {nd[4], nd[5], nd[6]};
    if (slab(mn, mx, org, inv, closest) == INF) continue;
    const double leftFirst = nd[3];
    const double count = nd[7];
    if (count > 0) {
      for (int i = 0; i < (int)count; i++) {
        uint32_t t = tri[(uint64_t)leftFirst + i];
        double th, uh, vh;
        if (tri_hit(o, d, vtx(pos, t, 0), vtx(pos, t, 1), vtx(pos, t, 2), tMin, closest, th, uh, vh)) {
          closest = th;
          out = {(int32_t)t, th, uh, vh};
        }
      }
    } else {
      if (sp + 2 > 64) return false;
      stack[sp++] = (int32_t)leftFirst + 1;
      stack[sp++] = (int32_t)leftFirst;
    }
  }
  return true;
}

template <class F>
void parallel_for(uint64_t n, int threads, F&& f) {
  if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
  if (n < 1024 || threads == 1) {
    f(0, n);
    return;
  }
  std::vector<std::thread> pool;
  std::atomic<uint64_t> next(0);
  const uint64_t chunk = 256;
  for (int k = 0; k < threads; k++) {
    pool.emplace_back([&]() {
      for (;;) {
        uint64_t b = next.fetch_add(chunk);
        if (b >= n) break;
        f(b, std::min(n, b + chunk));
      }
    });
  }
  for (auto& t : pool) t.join();
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------------------
// buildBVH, src/math/bvh.ts:52-252.
// ---------------------------------------------------------------------------
int orc_build_bvh(const float* positions, uint64_t n_floats, int max_leaf, int bins, float* nodes,
                  uint32_t* node_count_out, uint32_t* triIndices, double* bounds_out) {
  if (n_floats % 9 != 0) return ORC_ERR_INVALID;  // bvh.ts:54-57
  if (bins < 2 || max_leaf < 1) return ORC_ERR_INVALID;
  const uint64_t triCount = n_floats / 9;

  // Per-triangle bounds and centroids (bvh.ts:59-73): Float32Array stores.
  std::vector<float> tb(triCount * 6), cen(triCount * 3);
  for (uint64_t i = 0; i < triCount; i++) {
    for (int a = 0; a < 3; a++) {
      const float p0 = positions[i * 9 + a], p1 = positions[i * 9 + 3 + a], p2 = positions[i * 9 + 6 + a];
      const float lo = std::min(p0, std::min(p1, p2));
      const float hi = std::max(p0, std::max(p1, p2));
      tb[i * 6 + a] = lo;
      tb[i * 6 + 3 + a] = hi;
      cen[i * 3 + a] = (float)(((double)lo + (double)hi) * 0.5);
    }
  }
  for (uint64_t i = 0; i < triCount; i++) triIndices[i] = (uint32_t)i;

  uint32_t nodeCount = 0;
  std::vector<double> binBox(3 * bins * 6);
  std::vector<uint32_t> binCount(3 * bins);
  std::vector<double> rightArea(bins);
  std::vector<uint32_t> rightCount(bins);
  double box[6], cbox[6];
  bool splittable[3] = {false, false, false};
  double binScale[3] = {0, 0, 0};

  auto boxArea = [](double x0, double y0, double z0, double x1, double y1, double z1) {  // bvh.ts:35-40
    const double dx = x1 - x0, dy = y1 - y0, dz = z1 - z0;
    return dx < 0 ? 0.0 : 2 * (dx * dy + dy * dz + dz * dx);
  };
  auto writeNode = [&](uint32_t idx, const double* b, double leftFirst, double count) {  // bvh.ts:91-101
    float* o = nodes + (uint64_t)idx * 8;
    o[0] = (float)b[0];
    o[1] = (float)b[1];
    o[2] = (float)b[2];
    o[3] = (float)leftFirst;
    o[4] = (float)b[3];
    o[5] = (float)b[4];
    o[6] = (float)b[5];
    o[7] = (float)count;
  };
  auto measure = [&](uint64_t start, uint64_t end) {  // bvh.ts:104-119
    for (int a = 0; a < 3; a++) {
      box[a] = INF;
      box[a + 3] = -INF;
      cbox[a] = INF;
      cbox[a + 3] = -INF;
    }
    for (uint64_t i = start; i < end; i++) {
      const uint32_t t = triIndices[i];
      for (int a = 0; a < 3; a++) {
        const double lo = tb[t * 6 + a], hi = tb[t * 6 + 3 + a], c = cen[t * 3 + a];
        if (lo < box[a]) box[a] = lo;
        if (hi > box[a + 3]) box[a + 3] = hi;
        if (c < cbox[a]) cbox[a] = c;
        if (c > cbox[a + 3]) cbox[a + 3] = c;
      }
    }
  };
  auto binOf = [&](uint32_t t, int axis) -> int {  // bvh.ts:122-123
    const double f = std::floor(((double)cen[t * 3 + axis] - cbox[axis]) * binScale[axis]);
    return (int)std::min((double)(bins - 1), f);
  };
  auto partition = [&](uint64_t start, uint64_t end, int axis, int split) -> uint64_t {  // bvh.ts:126-140
    int64_t i = (int64_t)start, j = (int64_t)end - 1;
    while (i <= j) {
      if (binOf(triIndices[i], axis) <= split) {
        i++;
      } else {
        std::swap(triIndices[i], triIndices[j]);
        j--;
      }
    }
    return (uint64_t)i;
  };

  const uint32_t root = nodeCount++;
  if (triCount == 0) {  // bvh.ts:143-147
    for (double& b : box) b = 0;
    writeNode(root, box, 0, 0);
    *node_count_out = nodeCount;
    for (int k = 0; k < 6; k++) bounds_out[k] = 0;
    return ORC_OK;
  }

  struct Task {
    uint32_t node;
    uint64_t start, end;
  };
  std::vector<Task> stack;
  stack.push_back({root, 0, triCount});
  while (!stack.empty()) {
    const Task tk = stack.back();
    stack.pop_back();
    const uint64_t start = tk.start, end = tk.end, count = end - start;
    measure(start, end);

    if (count <= (uint64_t)max_leaf) {  // bvh.ts:157-160
      writeNode(tk.node, box, (double)start, (double)count);
      continue;
    }

    // bvh.ts:163-174: longest centroid axis; bin all 3 axes only for >= 512.
    const int longest = cbox[3] - cbox[0] >= cbox[4] - cbox[1] && cbox[3] - cbox[0] >= cbox[5] - cbox[2] ? 0
                        : cbox[4] - cbox[1] >= cbox[5] - cbox[2]                                      ? 1
                                                                                                       : 2;
    for (int a = 0; a < 3; a++) {
      const double extent = cbox[a + 3] - cbox[a];
      splittable[a] = extent > 1e-9 && (count >= 512 || a == longest);
      binScale[a] = (double)bins / extent;
      if (!splittable[a]) continue;
      for (int k = a * bins; k < (a + 1) * bins; k++) {
        for (int c = 0; c < 3; c++) {
          binBox[k * 6 + c] = INF;
          binBox[k * 6 + 3 + c] = -INF;
        }
        binCount[k] = 0;
      }
    }
    for (uint64_t i = start; i < end; i++) {  // bvh.ts:175-189
      const uint32_t t = triIndices[i];
      for (int a = 0; a < 3; a++) {
        if (!splittable[a]) continue;
        const int k = a * bins + binOf(t, a);
        binCount[k]++;
        const int o = k * 6;
        for (int c = 0; c < 3; c++) {
          const double lo = tb[t * 6 + c], hi = tb[t * 6 + 3 + c];
          if (lo < binBox[o + c]) binBox[o + c] = lo;
          if (hi > binBox[o + 3 + c]) binBox[o + 3 + c] = hi;
        }
      }
    }

    double bestCost = INF;  // bvh.ts:191-223
    int bestAxis = -1, bestBin = -1;
    for (int a = 0; a < 3; a++) {
      if (!splittable[a]) continue;
      double x0 = INF, y0 = INF, z0 = INF, x1 = -INF, y1 = -INF, z1 = -INF;
      uint64_t n = 0;
      for (int b = bins - 1; b > 0; b--) {
        const int o = (a * bins + b) * 6;
        x0 = std::min(x0, binBox[o]);
        y0 = std::min(y0, binBox[o + 1]);
        z0 = std::min(z0, binBox[o + 2]);
        x1 = std::max(x1, binBox[o + 3]);
        y1 = std::max(y1, binBox[o + 4]);
        z1 = std::max(z1, binBox[o + 5]);
        n += binCount[a * bins + b];
        rightArea[b] = boxArea(x0, y0, z0, x1, y1, z1);
        rightCount[b] = (uint32_t)n;
      }
      x0 = INF, y0 = INF, z0 = INF, x1 = -INF, y1 = -INF, z1 = -INF;
      uint64_t leftN = 0;
      for (int b = 0; b < bins - 1; b++) {
        const int o = (a * bins + b) * 6;
        x0 = std::min(x0, binBox[o]);
        y0 = std::min(y0, binBox[o + 1]);
        z0 = std::min(z0, binBox[o + 2]);
        x1 = std::max(x1, binBox[o + 3]);
        y1 = std::max(y1, binBox[o + 4]);
        z1 = std::max(z1, binBox[o + 5]);
        leftN += binCount[a * bins + b];
        const uint64_t rn = rightCount[b + 1];
        if (leftN == 0 || rn == 0) continue;
        const double cost = boxArea(x0, y0, z0, x1, y1, z1) * (double)leftN + rightArea[b + 1] * (double)rn;
        if (cost < bestCost) {
          bestCost = cost;
          bestAxis = a;
          bestBin = b;
        }
      }
    }

    const double leafCost = (double)count * boxArea(box[0], box[1], box[2], box[3], box[4], box[5]);
    const bool unprofitable = bestAxis < 0 || bestCost >= leafCost;  // bvh.ts:227-232
    if (unprofitable && count <= (uint64_t)max_leaf * 4) {
      writeNode(tk.node, box, (double)start, (double)count);
      continue;
    }

    uint64_t mid = unprofitable ? ((start + end) >> 1) : partition(start, end, bestAxis, bestBin);
    if (mid == start || mid == end) mid = (start + end) >> 1;  // bvh.ts:236

    const uint32_t left = nodeCount++;
    const uint32_t right = nodeCount++;
    writeNode(tk.node, box, (double)left, 0);
    stack.push_back({right, mid, end});  // bvh.ts:242: right pushed first, left popped first
    stack.push_back({left, start, mid});
  }

  measure(0, triCount);  // bvh.ts:245-251
  *node_count_out = nodeCount;
  for (int k = 0; k < 6; k++) bounds_out[k] = box[k];
  return ORC_OK;
}

int orc_bvh_depth(const float* nodes, uint32_t node_count) {
  if (node_count == 0) return -1;
  std::vector<std::pair<uint32_t, int>> st{{0u, 0}};
  int depth = 0;
  while (!st.empty()) {
    auto [n, dd] = st.back();
    st.pop_back();
    if (n >= node_count) return -1;
    depth = std::max(depth, dd);
    const float* nd = nodes + (uint64_t)n * 8;
    if (nd[7] > 0 || node_count == 1) continue;
    const uint32_t l = (uint32_t)nd[3];
    st.push_back({l, dd + 1});
    st.push_back({l + 1, dd + 1});
  }
  return depth;
}

int orc_intersect_bvh(const float* nodes, uint32_t node_count, const uint32_t* tri, uint32_t tri_count,
                      const float* positions, const double* rays, uint64_t n, double t_min, double t_max,
                      int32_t* id_out, double* t_out, double* u_out, double* v_out, int threads) {
  (void)node_count;
  std::atomic<int> overflow(0);
  parallel_for(n, threads, [&](uint64_t b, uint64_t e) {
    for (uint64_t r = b; r < e; r++) {
      const double* ry = rays + r * 6;
      Hit h;
      if (!bvh_closest(nodes, tri, tri_count, positions, {ry[0], ry[1], ry[2]}, {ry[3], ry[4], ry[5]}, t_min,
                       t_max, h))
        overflow = 1;
      id_out[r] = h.id;
      if (t_out) t_out[r] = h.t;
      if (u_out) u_out[r] = h.u;
      if (v_out) v_out[r] = h.v;
    }
  });
  return overflow ? ORC_ERR_STACK : ORC_OK;
}

int orc_intersect_bvh_f32(const float* nodes, uint32_t node_count, const uint32_t* tri, uint32_t tri_count,
                          const float* positions, const float* rays, uint64_t n, double t_min, double t_max,
                          int32_t* id_out, double* t_out, double* u_out, double* v_out, int threads) {
  (void)node_count;
  std::atomic<int> overflow(0);
  parallel_for(n, threads, [&](uint64_t b, uint64_t e) {
    for (uint64_t r = b; r < e; r++) {
      const float* ry = rays + r * 6;
      Hit h;
      if (!bvh_closest(nodes, tri, tri_count, positions, {ry[0], ry[1], ry[2]}, {ry[3], ry[4], ry[5]}, t_min,
                       t_max, h))
        overflow = 1;
      id_out[r] = h.id;
      if (t_out) t_out[r] = h.t;
      if (u_out) u_out[r] = h.u;
      if (v_out) v_out[r] = h.v;
    }
  });
  return overflow ? ORC_ERR_STACK : ORC_OK;
}

// Work counts of intersectBVH's own order (bvh.ts:283-318): nodes popped and
// triangles tested per ray.
int orc_ts_traversal_counts(const float* nodes, const uint32_t* tri, uint32_t tri_count, const float* positions,
                            const float* rays, uint64_t n, double t_min, double t_max, uint32_t* popped_out,
                            uint32_t* tests_out, int threads) {
  parallel_for(n, threads, [&](uint64_t b, uint64_t e) {
    for (uint64_t r = b; r < e; r++) {
      const float* ry = rays + r * 6;
      const V3 o{ry[0], ry[1], ry[2]}, d{ry[3], ry[4], ry[5]};
      const double org[3] = {o.x, o.y, o.z};
      const double inv[3] = {1.0 / d.x, 1.0 / d.y, 1.0 / d.z};
      uint32_t popped = 0, tests = 0;
      if (tri_count) {
        int32_t stack[64];
        int sp = 0;
        stack[sp++] = 0;
        double closest = t_max;
        while (sp > 0) {
          const int32_t nn = stack[--sp];
          popped++;
          const float* nd = nodes + (uint64_t)nn * 8;
          const double mn[3] = {nd[0], nd[1], nd[2]}, mx[3] = {nd[4], nd[5], nd[6]};
          if (slab(mn, mx, org, inv, closest) == INF) continue;
          if (nd[7] > 0) {
            for (int i = 0; i < (int)nd[7]; i++) {
              const uint32_t t = tri[(uint64_t)nd[3] + i];
              tests++;
              double th, uh, vh;
              if (tri_hit(o, d, vtx(positions, t, 0), vtx(positions, t, 1), vtx(positions, t, 2), t_min, closest,
                          th, uh, vh))
                closest = th;
            }
          } else if (sp + 2 <= 64) {
            stack[sp++] = (int32_t)nd[3] + 1;
            stack[sp++] = (int32_t)nd[3];
          }
        }
      }
      popped_out[r] = popped;
      tests_out[r] = tests;
    }
  });
  return ORC_OK;
}

int orc_intersect_all(const float* positions, uint32_t tri_count, const double* rays, uint64_t n, double t_min,
                      double t_max, int32_t* id_out, double* t_out, double* u_out, double* v_out, int threads) {
  parallel_for(n, threads, [&](uint64_t b, uint64_t e) {
    for (uint64_t r = b; r < e; r++) {
      const double* ry = rays + r * 6;
      const V3 o{ry[0], ry[1], ry[2]}, d{ry[3], ry[4], ry[5]};
      Hit best{-1, INF, 0, 0};
      double closest = t_max;
      for (uint32_t t = 0; t < tri_count; t++) {  // bvh.ts:332-346
        double th, uh, vh;
        if (tri_hit(o, d, vtx(positions, t, 0), vtx(positions, t, 1), vtx(positions, t, 2), t_min, closest, th,
                    uh, vh)) {
          closest = th;
          best = {(int32_t)t, th, uh, vh};
        }
      }
      id_out[r] = best.id;
      if (t_out) t_out[r] = best.t;
      if (u_out) u_out[r] = best.u;
      if (v_out) v_out[r] = best.v;
    }
  });
  return ORC_OK;
}

int orc_intersect_triangle(const double* origin, const double* dir, const double* v0, const double* v1,
                           const double* v2, double t_min, double t_max, double* t, double* u, double* v) {
  double th, uh, vh;
  const V3 o{origin[0], origin[1], origin[2]}, d{dir[0], dir[1], dir[2]};
  if (!tri_hit(o, d, {v0[0], v0[1], v0[2]}, {v1[0], v1[1], v1[2]}, {v2[0], v2[1], v2[2]}, t_min, t_max, th, uh,
               vh))
    return 0;
  *t = th;
  *u = uh;
  *v = vh;
  return 1;
}

int orc_intersect_sphere(const double* origin, const double* dir, const double* center, double radius,
                         double t_min, double t_max, double* tout) {  // ray.ts:48-67
  const V3 o{origin[0], origin[1], origin[2]}, d{dir[0], dir[1], dir[2]}, c{center[0], center[1], center[2]};
  const V3 oc = sub(o, c);
  const double b = dot(oc, d);
  const double cc = dot(oc, oc) - radius * radius;
  const double disc = b * b - cc;
  if (disc < 0) return 0;
  const double sq = std::sqrt(disc);
  double t = -b - sq;
  if (t <= t_min || t >= t_max) {
    t = -b + sq;
    if (t <= t_min || t >= t_max) return 0;
  }
  *tout = t;
  return 1;
}

double orc_aabb_intersect(const double* bmin, const double* bmax, const double* origin, const double* inv_dir,
                          double t_max) {
  return slab(bmin, bmax, origin, inv_dir, t_max);
}

// ---------------------------------------------------------------------------
// GLSL traversal work counts, src/shaders/scene.glsl:218-267 (f32, near-first,
// stack 40, iteration cap 8192, EPS = 1e-6 handled by t_min).
// ---------------------------------------------------------------------------
int orc_glsl_traversal_counts(const float* nodes, uint32_t node_count, const float* geo, uint32_t tri_count,
                              const float* rays, uint64_t n, float t_min, uint32_t* inner_out,
                              uint32_t* tris_out, int32_t* slot_out, int threads) {
  (void)node_count;
  const float FINF = 1e30f;  // common.glsl:7 INF
  parallel_for(n, threads, [&](uint64_t b, uint64_t e) {
    for (uint64_t r = b; r < e; r++) {
      const float* ry = rays + r * 6;
      const float ro[3] = {ry[0], ry[1], ry[2]}, rd[3] = {ry[3], ry[4], ry[5]};
      const float inv[3] = {1.0f / rd[0], 1.0f / rd[1], 1.0f / rd[2]};
      uint32_t inner = 0, tests = 0;
      int32_t best = -1;
      float closest = FINF;
      auto hitAABB = [&](const float* a, const float* bb) -> float {  // scene.glsl:153-161
        float tn = 0.0f, tf = closest;
        float tmn[3], tmx[3];
        for (int i = 0; i < 3; i++) {
          const float t0 = (a[i] - ro[i]) * inv[i], t1 = (bb[i] - ro[i]) * inv[i];
          tmn[i] = std::min(t0, t1);
          tmx[i] = std::max(t0, t1);
        }
        tn = std::max(std::max(tmn[0], tmn[1]), std::max(tmn[2], 0.0f));
        tf = std::min(std::min(tmx[0], tmx[1]), std::min(tmx[2], closest));
        return tf >= tn ? tn : FINF;
      };
      if (tri_count > 0) {
        int stack[40];
        int sp = 0;
        int node = 0;
        for (int iter = 0; iter < 8192; iter++) {
          const float* nd = nodes + (uint64_t)node * 8;
          const int leftFirst = (int)nd[3];
          const int count = (int)nd[7];
          if (count > 0) {
            for (int k = 0; k < count; k++) {
              const int slot = leftFirst + k;
              const float* g = geo + (uint64_t)slot * 12;
              tests++;
              // hitTriangle, scene.glsl:113-130 in f32.
              const float e1[3] = {g[4] - g[0], g[5] - g[1], g[6] - g[2]};
              const float e2[3] = {g[8] - g[0], g[9] - g[1], g[10] - g[2]};
              const float p[3] = {rd[1] * e2[2] - rd[2] * e2[1], rd[2] * e2[0] - rd[0] * e2[2],
                                  rd[0] * e2[1] - rd[1] * e2[0]};
              const float det = e1[0] * p[0] + e1[1] * p[1] + e1[2] * p[2];
              if (std::fabs(det) < 1e-12f) continue;
              const float invDet = 1.0f / det;
              const float s[3] = {ro[0] - g[0], ro[1] - g[1], ro[2] - g[2]};
              const float u = (s[0] * p[0] + s[1] * p[1] + s[2] * p[2]) * invDet;
              if (u < 0.0f || u > 1.0f) continue;
              const float q[3] = {s[1] * e1[2] - s[2] * e1[1], s[2] * e1[0] - s[0] * e1[2],
                                  s[0] * e1[1] - s[1] * e1[0]};
              const float v = (rd[0] * q[0] + rd[1] * q[1] + rd[2] * q[2]) * invDet;
              if (v < 0.0f || u + v > 1.0f) continue;
              const float t = (e2[0] * q[0] + e2[1] * q[1] + e2[2] * q[2]) * invDet;
              if (t <= t_min || t >= closest) continue;
              closest = t;
              best = slot;
            }
            if (sp == 0) break;
            node = stack[--sp];
            continue;
          }
          inner++;
          int left = leftFirst, right = leftFirst + 1;
          const float* la = nodes + (uint64_t)left * 8;
          const float* ra = nodes + (uint64_t)right * 8;
          float tl = hitAABB(la, la + 4), tr = hitAABB(ra, ra + 4);
          if (tl > tr) {
            std::swap(tl, tr);
            std::swap(left, right);
          }
          if (tl == FINF) {
            if (sp == 0) break;
            node = stack[--sp];
          } else {
            node = left;
            if (tr != FINF && sp < 40) stack[sp++] = right;
          }
        }
      }
      if (inner_out) inner_out[r] = inner;
      if (tris_out) tris_out[r] = tests;
      if (slot_out) slot_out[r] = best;
    }
  });
  return ORC_OK;
}

// ---------------------------------------------------------------------------
// buildAliasTable, src/math/alias.ts:17-65 (Vose).
// ---------------------------------------------------------------------------
int orc_build_alias(const double* weights, uint32_t n, float* prob, uint32_t* alias, double* pmf,
                    double* total_out) {
  if (n == 0) return ORC_ERR_INVALID;
  double total = 0;
  for (uint32_t i = 0; i < n; i++) {
    const double w = weights[i];
    if (!(w >= 0) || !std::isfinite(w)) return ORC_ERR_INVALID;
    total += w;
  }
  for (uint32_t i = 0; i < n; i++) pmf[i] = total > 0 ? weights[i] / total : 1.0 / n;
  std::vector<double> scaled(n);
  std::vector<uint32_t> small(n), large(n);
  uint32_t ns = 0, nl = 0;
  for (uint32_t i = 0; i < n; i++) {
    scaled[i] = pmf[i] * n;
    if (scaled[i] < 1)
      small[ns++] = i;
    else
      large[nl++] = i;
  }
  for (uint32_t i = 0; i < n; i++) {
    prob[i] = 0;
    alias[i] = 0;
  }
  while (ns > 0 && nl > 0) {
    const uint32_t s = small[--ns];
    const uint32_t l = large[--nl];
    prob[s] = (float)scaled[s];
    alias[s] = l;
    scaled[l] = scaled[l] + scaled[s] - 1;
    if (scaled[l] < 1)
      small[ns++] = l;
    else
      large[nl++] = l;
  }
  while (nl > 0) {
    const uint32_t l = large[--nl];
    prob[l] = 1;
    alias[l] = l;
  }
  while (ns > 0) {
    const uint32_t s = small[--ns];
    prob[s] = 1;
    alias[s] = s;
  }
  *total_out = total;
  return ORC_OK;
}

// ---------------------------------------------------------------------------
// buildEnvSampler, src/scene/environment.ts:50-85.
// ---------------------------------------------------------------------------
int orc_build_env_sampler(const float* rgb, uint32_t width, uint32_t height, uint32_t max_width, uint32_t* gw_out,
                          uint32_t* gh_out, float* table, double* total_out) {
  if (width == 0 || height == 0) return ORC_ERR_INVALID;
  const uint32_t gw = std::max(1u, std::min(width, max_width));
  const double ghr = std::floor((double)height * gw / width + 0.5);  // Math.round for positive values
  const uint32_t gh = std::max(1u, std::min(height, (uint32_t)ghr));
  std::vector<double> weights((uint64_t)gw * gh);
  for (uint32_t cy = 0; cy < gh; cy++) {
    const uint64_t y0 = (uint64_t)std::floor((double)cy * height / gh);
    const uint64_t y1 = std::max(y0 + 1, (uint64_t)std::floor((double)(cy + 1) * height / gh));
    const double sinTheta = std::sin((M_PI * (cy + 0.5)) / gh);
    for (uint32_t cx = 0; cx < gw; cx++) {
      const uint64_t x0 = (uint64_t)std::floor((double)cx * width / gw);
      const uint64_t x1 = std::max(x0 + 1, (uint64_t)std::floor((double)(cx + 1) * width / gw));
      double sum = 0;
      for (uint64_t y = y0; y < y1; y++)
        for (uint64_t x = x0; x < x1; x++) {
          const float* p = rgb + (y * width + x) * 3;
          sum += 0.2126 * (double)p[0] + 0.7152 * (double)p[1] + 0.0722 * (double)p[2];
        }
      weights[(uint64_t)cy * gw + cx] = (sum / (double)((y1 - y0) * (x1 - x0))) * sinTheta;
    }
  }
  const uint32_t n = gw * gh;
  std::vector<float> prob(n);
  std::vector<uint32_t> alias(n);
  std::vector<double> pmf(n);
  double total = 0;
  const int st = orc_build_alias(weights.data(), n, prob.data(), alias.data(), pmf.data(), &total);
  if (st) return st;
  for (uint32_t i = 0; i < n; i++) {
    const uint32_t a = alias[i];
    table[(uint64_t)i * 4] = prob[i];
    table[(uint64_t)i * 4 + 1] = (float)a;
    table[(uint64_t)i * 4 + 2] = (float)(pmf[i] * n);
    table[(uint64_t)i * 4 + 3] = (float)(pmf[a] * n);
  }
  *gw_out = gw;
  *gh_out = gh;
  *total_out = total;
  return ORC_OK;
}

// ---------------------------------------------------------------------------
// Sheen albedo, src/scene/sheen.ts:13-60.
// ---------------------------------------------------------------------------
static double charlieD(double alpha, double cosH) {
  const double inv = 1 / alpha;
  const double sin2 = std::max(0.0, 1 - cosH * cosH);
  return ((2 + inv) * std::pow(sin2, inv * 0.5)) / (2 * M_PI);
}
static double neubeltV(double cosL, double cosV) { return 1 / (4 * (cosL + cosV - cosL * cosV)); }

// bakeSky (src/scene/environment.ts:106-132): gradient sky plus the sun's
// glow into a width x width/2 equirect map; every store rounds to binary32
// (Float32Array), then the glow is added and the intensity applied as the
// reference does, each a separate rounded store. directionFromUV :88-93,
// fromSpherical src/math/vec3.ts:57-60.
void orc_bake_sky(uint32_t width, const double* zenith, const double* horizon, const double* ground,
                  double intensity, int enabled, double sun_elevation_deg, double sun_azimuth_deg,
                  const double* sun_color, double sun_intensity, double sun_angular_radius_deg, float* out) {
  const uint32_t height = width / 2;
  const size_t n = (size_t)width * height * 3;
  for (size_t i = 0; i < n; i++) out[i] = 0.0f;
  if (!enabled || !(intensity > 0)) return;
  const double pi = 3.141592653589793;
  const double el = sun_elevation_deg * pi / 180, az = sun_azimuth_deg * pi / 180;
  const double ce = std::cos(el);
  const double sd[3] = {ce * std::sin(az), std::sin(el), ce * std::cos(az)};
  const bool sun_on = sun_intensity > 0 && sun_elevation_deg > -sun_angular_radius_deg;
  for (uint32_t y = 0; y < height; y++) {
    for (uint32_t x = 0; x < width; x++) {
      const double u = (x + 0.5) / width, v = (y + 0.5) / height;
      const double phi = (u - 0.5) * 2 * pi, theta = v * pi;
      const double st = std::sin(theta);
      const double d[3] = {st * std::cos(phi), std::cos(theta), st * std::sin(phi)};
      const double t = d[1];
      float* o = out + ((size_t)y * width + x) * 3;
      for (int c = 0; c < 3; c++)
        o[c] = (float)(t >= 0 ? horizon[c] + (zenith[c] - horizon[c]) * std::pow(t, 0.55)
                              : horizon[c] + (ground[c] - horizon[c]) * std::min(1.0, -t * 4));
      if (sun_on) {
        const double s = std::max(0.0, d[0] * sd[0] + d[1] * sd[1] + d[2] * sd[2]);
        const double glow = 0.12 * std::pow(s, 24) + 0.5 * std::pow(s, 400);
        for (int c = 0; c < 3; c++) o[c] = (float)((double)o[c] + sun_color[c] * glow);
      }
      for (int c = 0; c < 3; c++) o[c] = (float)((double)o[c] * intensity);
    }
  }
}

double orc_sheen_albedo(double cosV, double roughness, int steps) {
  const double r = std::max(0.07, roughness);
  const double alpha = r * r;
  const double v0 = std::sqrt(std::max(0.0, 1 - cosV * cosV)), v2 = cosV;
  const int phiSteps = steps / 2;
  const double dTheta = M_PI / 2 / steps;
  const double dPhi = M_PI / phiSteps;
  double e = 0;
  for (int i = 0; i < steps; i++) {
    const double th = (i + 0.5) * dTheta;
    const double ch = std::cos(th), sh = std::sin(th);
    const double d = charlieD(alpha, ch);
    for (int j = 0; j < phiSteps; j++) {
      const double ph = (j + 0.5) * dPhi;
      const double h0 = sh * std::cos(ph), h2 = ch;
      const double vh = v0 * h0 + v2 * h2;
      if (vh <= 0) continue;
      const double cosL = 2 * vh * h2 - v2;
      if (cosL <= 0) continue;
      e += d * neubeltV(cosL, cosV) * cosL * 4 * vh * sh * dTheta * dPhi;
    }
  }
  return std::min(1.0, 2 * e);
}

void orc_sheen_lut(int size, int steps, float* out) {
  for (int y = 0; y < size; y++)
    for (int x = 0; x < size; x++) {
      const double cosV = std::max(1e-3, (double)x / (size - 1));
      out[y * size + x] = (float)orc_sheen_albedo(cosV, (double)y / (size - 1), steps);
    }
}

}  // extern "C"
