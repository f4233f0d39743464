// Four-wide traversal over the reference's binary BVH, with the reference's
// decisions and order.
//
// The wide view holds, for every inner binary node n, four records: the
// grandchildren of n in the reference's visiting order (left subtree first),
// where a child of n that is a leaf stands in for its two (absent)
// grandchildren. One expansion therefore descends two levels with one
// 128-byte read instead of two dependent 64-byte reads, and skips the box
// tests of n's inner children.
//
// Skipping those tests changes no decision. A child's box lies inside its
// parent's (the builder's parent bounds are the union of its children's), so
// per axis the child's entry distance is >= the parent's and its exit <= the
// parent's, in binary32 and binary64 alike (rounding is monotone, and the
// fast path only takes rays whose inverse direction is finite). The
// reference's cull test, max(0, entries) > min(closest, exits), therefore
// culls a grandchild whenever it culls the child above it, and testing the
// grandchild alone gives the reference's answer for it. The other rules are
// those of the binary kernel: the first record that passes continues at once
// (nothing between the parent's test and the reference's pop of it can lower
// the closest distance), the others are pushed with an upper bound on their
// entry distance and re-tested on pop only if the closest distance has
// dropped below it.
//
// A record is a binary node record: box, then (lo.w) its own binary index for
// an inner node (count 0) or its first triangle slot for a leaf (count > 0);
// count -1 marks an unused record.
#pragma once
#include "traverse.cuh"

namespace lucent {

constexpr int kWide = 4;
// Pending records: at most 3 per expansion, one expansion per two levels of a
// tree at most 62 deep (the reference's 64-entry stack less the root and one).
constexpr int kWideStack = 96;

__device__ __forceinline__ Node wide_record(const Node* nodes, int c) {
  Node r = load_node(nodes, c);
  if (node_count(r) == 0) r.lo.w = __int_as_float(c);
  return r;
}

// Fills wide[4 n .. 4 n + 3] for every binary node n (unused records for leaves).
static __global__ void k_build_wide(const Node* nodes, uint32_t n_nodes, Node* wide) {
  const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= n_nodes) return;
  const float inf = __int_as_float(0x7f800000);
  Node rec[kWide];
  for (int k = 0; k < kWide; k++) rec[k] = {make_float4(inf, inf, inf, 0.f), make_float4(-inf, -inf, -inf, __int_as_float(-1))};
  const Node nd = load_node(nodes, n);
  const int f = node_first(nd);
  if (node_count(nd) == 0 && f > 0 && (uint32_t)f + 1 < n_nodes) {
    int m = 0;
    for (int c = f; c <= f + 1; c++) {
      const Node cn = load_node(nodes, c);
      const int g = node_first(cn);
      if (node_count(cn) > 0) {
        rec[m++] = cn;
      } else if (g > 0 && (uint32_t)g + 1 < n_nodes) {
        rec[m++] = wide_record(nodes, g);
        rec[m++] = wide_record(nodes, g + 1);
      }
    }
  }
  float4* out = reinterpret_cast<float4*>(wide + (size_t)kWide * n);
  for (int k = 0; k < kWide; k++) {
    out[2 * k] = rec[k].lo;
    out[2 * k + 1] = rec[k].hi;
  }
}

static inline void launch_build_wide(const Node* nodes, uint32_t n_nodes, Node* wide, cudaStream_t s) {
  if (n_nodes) k_build_wide<<<(n_nodes + 255) / 256, 256, 0, s>>>(nodes, n_nodes, wide);
}

struct WidePending {
  int rec;    // index of the record in the wide array (4 n + k)
  float ehi;  // upper bound on its entry distance when it was pushed
};

// The running closest of a closest-hit ray: the reference's binary64
// `closest` lies in [lo, hi]; `exact`: c64 is the binary64 t of `best`;
// `pend`: a triangle met at a distance tied with it within the binary32
// bounds (kTriNearC), not yet compared in binary64, [lo, hi] then spanning
// both candidates' distances.
struct Closest {
  double c64;
  float lo, hi;
  int best, pend;
  int exact;
};

// The reference's binary64 `closest`, for the decisions the binary32 bounds
// leave open: the binary64 t of `best` if not yet known, then the deferred
// tie resolved as the reference's test resolves it (taken iff its binary64
// t is below). Out of line, one copy for every such decision of the kernel.
static __device__ __noinline__ Closest closest_exact(Closest s, float3 o, float3 d, const float4* __restrict__ tris,
                                                     double tmin, unsigned long long* stats) {
  const D3 O{o.x, o.y, o.z}, Dd{d.x, d.y, d.z};
  double t, u, v;
  if (!s.exact) {
    if (stats) atomicAdd(stats + 3, 1ull);
    const float4* g = tris + 3 * (size_t)s.best;
    ts_triangle(O, Dd, d3f(__ldg(g)), d3f(__ldg(g + 1)), d3f(__ldg(g + 2)), tmin,
                __longlong_as_double(0x7ff0000000000000ll), t, u, v);
    s.c64 = t;
    s.exact = 1;
  }
  if (s.pend >= 0) {
    if (stats) atomicAdd(stats + 2, 1ull);
    const float4* g = tris + 3 * (size_t)s.pend;
    if (ts_triangle(O, Dd, d3f(__ldg(g)), d3f(__ldg(g + 1)), d3f(__ldg(g + 2)), tmin, s.c64, t, u, v)) {
      s.best = s.pend;
      s.c64 = t;
    }
    s.pend = -1;
  }
  s.lo = __double2float_rd(s.c64);
  s.hi = __double2float_ru(s.c64);
  return s;
}

// Closest hit over the wide view: k_closest_fast_t's persistent warps, per-lane
// refill, bounded-error binary32 decisions and binary64 fallbacks, with each
// inner step expanding four records (bv.wide must be set). Two deferrals keep
// binary64 off the common path: a distance tie (Closest::pend), and a leaf
// whose own slab test the binary32 bounds leave open (`cond`), which is
// visited and decided in binary64 only if one of its triangles is not
// certainly rejected (otherwise the leaf changes nothing either way).
template <class Pol>
__global__ void __launch_bounds__(Pol::kThreads, Pol::kMinBlocks) k_closest_wide_t(TravArgs A, Pol P) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const float tmin_lo = __double2float_rd(A.tMin), tmin_hi = __double2float_ru(A.tMin);
  const float cmax_lo = __double2float_rd(A.tMax), cmax_hi = __double2float_ru(A.tMax);
  const float INF32 = __int_as_float(0x7f800000);
  const uint32_t n = P.count();
  const bool use_alpha = P.alpha_any();

  bool active = false, exhausted = false, have_cur = false, cond = false;
  uint32_t ri = 0, iters = 0, key = 0;
  Ray32 r;
  Closest S{A.tMax, 0.f, 0.f, -1, -1, 1};
  int sp = 0;
  BvhView bv{A.nodes, A.tris, A.node_limit, 0, A.wide};
  Node cur;
  WidePending stack[kWideStack];

  while (true) {
    const bool need = !active && !exhausted;
    const unsigned m = __ballot_sync(FULL, need);
    // Refill once Pol::kRefillMin lanes wait (or none is busy): each refill
    // stalls the whole warp on the atomic and the new rays' loads.
    if (m && (__popc(m) >= Pol::kRefillMin || __ballot_sync(FULL, active) == 0)) {
      const int leader = __ffs(m) - 1;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(A.work, (uint32_t)__popc(m));
      base = __shfl_sync(FULL, base, leader);
      if (need) {
        ri = base + __popc(m & lt);
        if (ri >= n) {
          exhausted = true;
        } else {
          float3 o, d;
          P.ray(ri, o, d);
          if (!safe_ray(o, d)) {
            A.queue[atomicAdd(A.queue_len, 1u)] = ri;
          } else {
            r = make_ray32(o, d);
            key = use_alpha ? P.key(ri) : 0u;  // read only where alpha tests use it
            if constexpr (Pol::kMultiScene) bv = P.bvh(ri);
            S = Closest{A.tMax, cmax_lo, cmax_hi, -1, -1, 1};
            cond = false;
            sp = 0;
            iters = 0;
            count_stat(A, 0);
            cur = wide_record(bv.nodes, 0);  // the reference pops the root first and tests its box
            SlabClass cl = classify_slab(r, cur.lo, cur.hi, S.lo, S.hi);
            if (cl == kAmbiguous) {
              count_stat(A, 1);
              cl = slab_f64_culled(cur.lo, cur.hi, o, d, A.tMax) ? kCulled : kPass;
            }
            have_cur = cl != kCulled;
            active = true;
          }
        }
      }
    }
    if (__all_sync(FULL, exhausted)) break;
    if (!active) continue;

    auto exact_c = [&]() {  // the reference's binary64 `closest`, on demand
      if (!S.exact || S.pend >= 0) S = closest_exact(S, r.o, r.d, bv.tris, A.tMin, A.stats);
      return S.c64;
    };

    if (!have_cur) {
      if (sp == 0) {  // finished
        if (S.pend >= 0) exact_c();
        if (S.best < 0) {
          P.miss(ri);
        } else {
          // Only the triangle: its t, u, v are computed afterwards with the
          // warp converged (lanes finish their rays at different steps, and
          // work at this point stalls the warp for each lane in turn).
          P.finish(ri, S.best);
        }
        active = false;
        continue;
      }
      const WidePending e = stack[--sp];
      const Node nd = load_node(bv.wide, e.rec);
      cond = false;
      if (e.ehi > S.lo) {  // open leaves were pushed with ehi = inf: always re-tested
        const SlabClass cl = classify_slab(r, nd.lo, nd.hi, S.lo, S.hi);
        if (cl == kCulled) continue;
        if (cl == kAmbiguous) {
          if (node_count(nd) > 0) {
            cond = true;
          } else {
            count_stat(A, 1);
            if (slab_f64_culled(nd.lo, nd.hi, r.o, r.d, exact_c())) continue;
          }
        }
      }
      cur = nd;
      have_cur = true;
    }
    if (++iters > bv.node_limit) {  // a valid BVH visits each node at most once per ray
      atomicOr(A.err, kErrIterations);
      P.fail(ri);
      active = false;
      have_cur = false;
      continue;
    }
    const int cnt = node_count(cur), first = node_first(cur);
    if (cnt > 0) {
      bool defer = false;
      for (int k = 0; k < cnt; k++) {
        const int slot = first + k;
        const float4 a = __ldg(bv.tris + 3 * (size_t)slot), b = __ldg(bv.tris + 3 * (size_t)slot + 1),
                     c = __ldg(bv.tris + 3 * (size_t)slot + 2);
        float tl, th;
        float3 est;
        const TriClass tc = mt_classify(r, a, b, c, tmin_lo, tmin_hi, S.lo, S.hi, tl, th, est);
        if (tc == kTriReject) continue;
        if (cond) {  // this triangle may count: first the leaf's own test, as the reference made it
          cond = false;
          count_stat(A, 1);
          if (slab_f64_culled(cur.lo, cur.hi, r.o, r.d, exact_c())) break;
        }
        if (use_alpha) {
          const AlphaAnswer aa = P.alpha_fast(bv.scene, slot, key);
          if (aa == kAlphaDefer) {
            defer = true;
            break;
          }
          if (aa == kAlphaPass) continue;
        }
        if (tc == kTriAccept) {
          S.best = slot;
          S.pend = -1;
          S.exact = 0;
          S.lo = tl;
          S.hi = th;
          continue;
        }
        if (tc == kTriNearC && S.pend < 0) {  // defer: a later certain hit below both makes it moot
          S.pend = slot;
          S.lo = fminf(S.lo, tl);
          S.hi = fmaxf(S.hi, th);
          continue;
        }
        count_stat(A, 2);
        const double cc = exact_c();
        const Tri64 h = tri_f64(r.o, r.d, a, b, c, A.tMin, cc);
        if (h.hit) {
          S.best = slot;
          S.c64 = h.t;
          S.lo = __double2float_rd(h.t);
          S.hi = __double2float_ru(h.t);
        }
      }
      have_cur = false;
      if (defer) {  // a textured alpha test: the binary64 kernel traces this ray
        A.queue[atomicAdd(A.queue_len, 1u)] = ri;
        active = false;
        continue;
      }
    } else {
      // Expand the four records of `cur`: binary32 tests of all four, then
      // binary64 for inner records they leave open (one place in the code),
      // then, as the reference's order has it, the first passing record
      // continues and the others are pushed in reverse order. A leaf left
      // open passes conditionally (`cond`).
      const int base = kWide * first;
      unsigned pass = 0, open_leaf = 0, open_inner = 0;
      float eh[kWide];
#pragma unroll
      for (int k = 0; k < kWide; k++) {
        const Node s = load_node(bv.wide, base + k);
        eh[k] = 0.f;
        if (node_count(s) < 0) continue;
        const SlabClass cl = classify_slab_e(r, s.lo, s.hi, S.lo, S.hi, eh[k]);
        if (cl == kPass) pass |= 1u << k;
        else if (cl == kAmbiguous) (node_count(s) > 0 ? open_leaf : open_inner) |= 1u << k;
      }
      if (open_inner) {
        const double cc = exact_c();
        for (int k = 0; k < kWide; k++) {
          if (!(open_inner >> k & 1u)) continue;
          count_stat(A, 1);
          const Node s = load_node(bv.wide, base + k);
          if (!slab_f64_culled(s.lo, s.hi, r.o, r.d, cc)) pass |= 1u << k;
        }
      }
      pass |= open_leaf;
      if (!pass) {
        have_cur = false;
        continue;
      }
      const int go = __ffs(pass) - 1;
      bool overflow = false;
#pragma unroll
      for (int k = kWide - 1; k > 0; k--) {
        if (k <= go || !(pass >> k & 1u)) continue;
        if (sp >= kWideStack) overflow = true;
        else stack[sp++] = {base + k, (open_leaf >> k & 1u) ? INF32 : eh[k]};
      }
      if (overflow) {  // unreachable for trees the reference's stack can traverse
        atomicOr(A.err, kErrStack);
        P.fail(ri);
        active = false;
        have_cur = false;
        continue;
      }
      cur = load_node(bv.wide, base + go);
      cond = open_leaf >> go & 1u;
    }
  }
}

// Any hit over the wide view: one ray per thread (grid-stride), as
// k_anyhit_fast_t. With the cull distance fixed at tMax the answer does not
// depend on visiting order, and a leaf is reached exactly when its own box
// passes (a culled ancestor implies a culled leaf), so testing every
// expanded record once gives the reference's answer. Pushed records have
// passed their test; a pop only expands or tests triangles.
template <class Pol>
__global__ void __launch_bounds__(256, 4) k_anyhit_wide_t(TravArgs A, Pol P) {
  const float tmin_lo = __double2float_rd(A.tMin), tmin_hi = __double2float_ru(A.tMin);
  const uint32_t n = P.count();
  const bool use_alpha = P.alpha_any();
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    float3 o, d;
    P.ray(k, o, d);
    if (!safe_ray(o, d)) {
      A.queue[atomicAdd(A.queue_len, 1u)] = k;
      continue;
    }
    const Ray32 r = make_ray32(o, d);
    const uint32_t key = P.key(k);
    const float tmax32 = P.tmax32(k);  // binary32, so its bounds are itself
    BvhView bv = bvh_of(A, P, k);
    if constexpr (!Pol::kMultiScene) bv.wide = A.wide;
    const float c_lo = tmax32, c_hi = tmax32;
    auto passes = [&](const Node& nd) {
      SlabClass cl = classify_slab(r, nd.lo, nd.hi, c_lo, c_hi);
      if (cl == kAmbiguous) cl = ts_slab_culled(nd.lo, nd.hi, {o.x, o.y, o.z}, inv_exact(d), (double)tmax32) ? kCulled : kPass;
      return cl == kPass;
    };
    int stack[kWideStack];  // indices of records that passed their box test
    int sp = 0;
    bool occ = false, ok = true, defer = false;
    uint32_t iters = 0;
    Node cur = wide_record(bv.nodes, 0);
    bool have = passes(cur);
    while (have) {
      if (++iters > bv.node_limit) {
        atomicOr(A.err, kErrIterations);
        ok = false;
        break;
      }
      const int cnt = node_count(cur), first = node_first(cur);
      if (cnt > 0) {
        for (int q = 0; q < cnt && !occ && !defer; q++) {
          const int slot = first + q;
          const float4 a = __ldg(bv.tris + 3 * (size_t)slot), b = __ldg(bv.tris + 3 * (size_t)slot + 1),
                       c = __ldg(bv.tris + 3 * (size_t)slot + 2);
          float tl, th;
          float3 est;
          const TriClass tc = mt_classify(r, a, b, c, tmin_lo, tmin_hi, c_lo, c_hi, tl, th, est);
          if (tc == kTriReject) continue;
          if (use_alpha) {
            const AlphaAnswer aa = P.alpha_fast(bv.scene, slot, key);
            if (aa == kAlphaDefer) {
              defer = true;
              continue;
            }
            if (aa == kAlphaPass) continue;
          }
          if (tc == kTriAccept) {
            occ = true;
          } else {
            double t, u, v;
            occ = ts_triangle({o.x, o.y, o.z}, {d.x, d.y, d.z}, d3f(a), d3f(b), d3f(c), A.tMin, (double)tmax32, t, u, v);
          }
        }
        if (occ || defer) break;
      } else {
        const int base = kWide * first;
#pragma unroll
        for (int q = 0; q < kWide; q++) {
          const Node s = load_node(bv.wide, base + q);
          if (node_count(s) < 0 || !passes(s)) continue;
          if (sp >= kWideStack) ok = false;
          else stack[sp++] = base + q;
        }
        if (!ok) {  // unreachable for trees the reference's stack can traverse
          atomicOr(A.err, kErrStack);
          break;
        }
      }
      have = sp > 0;
      if (have) cur = load_node(bv.wide, stack[--sp]);
    }
    if (defer && ok) {  // a textured alpha test: the binary64 kernel answers this ray
      A.queue[atomicAdd(A.queue_len, 1u)] = k;
      continue;
    }
    P.shadow(k, ok ? occ : true);
  }
}

}  // namespace lucent
