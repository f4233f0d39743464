// Traversal kernels shared by the BVH API and the renderer, templated on a
// policy that supplies rays and consumes hits.
//
// Closest hit reproduces the reference's CPU intersector, intersectBVH
// (src/math/bvh.ts:265-320): its traversal order (explicit stack, left child
// first, a node's box tested against the running closest distance `c` when it
// is popped) and its binary64 decisions. Each decision is first tried with
// binary32 arithmetic whose error is bounded (closest_hit.cuh); binary64 runs
// only when the bound cannot decide. The traversal reports the hit triangle
// only; its t, u, v are computed afterwards, one ray per thread: the BVH
// API's are the reference's binary64 values rounded to binary32 (tri_df32),
// the renderer's binary32 estimates like the GLSL's own hitTriangle.
//
// Any hit (shadow rays) answers: does some triangle pass the reference's
// binary64 Moller-Trumbore in (tMin, tMax) inside boxes its slab test at tMax
// accepts? With `c` fixed at tMax the answer does not depend on visiting order.
//
// Policies:
//   uint32_t count() const                        rays in this launch
//   void ray(uint32_t k, float3& o, float3& d)   k-th ray
//   uint32_t key(uint32_t k) const                alpha any-hit key (RNG state)
//   bool alpha(int scene, int slot, uint32_t key, float bu, float bv)
//                                                 true if a hit on `slot` at barycentrics (bu, bv) counts
//   AlphaAnswer alpha_fast(int scene, int slot, uint32_t key)
//                                                 the same without texture lookups (kAlphaDefer: ask alpha)
//   static constexpr int kRefillMin               (closest hit) lanes a warp lets wait before it fetches rays
//   static constexpr bool kMultiScene             rays of several scenes in one launch:
//   BvhView bvh(uint32_t k) const                 then the k-th ray's BVH (else TravArgs'),
//   BvhView scene_bvh(int s) const                and scene s's BVH
//   bool alpha_any() const                        false: no alpha-tested triangles
//   void finish(uint32_t k, int slot)             (closest) the hit triangle; its t, u, v are the policy's
//                                                 to compute later, with the warp converged
//   void hit(uint32_t k, int slot, double t, double u, double v)   a hit with its binary64 values
//   void miss(uint32_t k); void fail(uint32_t k)
//   float tmax32(uint32_t k) const                (any hit) the ray's tMax, a binary32 value
//   void shadow(uint32_t k, bool occluded)        (any hit)
#pragma once
#include "closest_hit.cuh"

namespace lucent {

__device__ __forceinline__ Node load_node(const Node* nodes, int n) {
  const float4* p = reinterpret_cast<const float4*>(nodes) + 2 * (size_t)n;
  Node r;
  r.lo = __ldg(p);
  r.hi = __ldg(p + 1);
  return r;
}

__device__ __forceinline__ D3 inv_exact(float3 d) {
  return {ddiv(1.0, (double)d.x), ddiv(1.0, (double)d.y), ddiv(1.0, (double)d.z)};
}

// Binary64 fallbacks of the fast closest-hit kernel, kept out of line: they
// run for a few percent of rays, and inlined they raise the register
// allocation (and the spills) of the binary32 loop around them. (The any-hit
// kernel measured faster with them inline.)
struct Tri64 {
  double t, u, v;
  bool hit;
};
static __device__ __noinline__ Tri64 tri_f64(float3 o, float3 d, float4 a, float4 b, float4 c, double tMin, double tMax) {
  Tri64 r{0.0, 0.0, 0.0, false};
  r.hit = ts_triangle({o.x, o.y, o.z}, {d.x, d.y, d.z}, d3f(a), d3f(b), d3f(c), tMin, tMax, r.t, r.u, r.v);
  return r;
}
static __device__ __noinline__ bool slab_f64_culled(float4 mn, float4 mx, float3 o, float3 d, double tMax) {
  return ts_slab_culled(mn, mx, {o.x, o.y, o.z}, inv_exact(d), tMax);
}

struct TravArgs {
  const Node* nodes;
  uint32_t node_limit;
  const float4* tris;  // 3 float4 per slot, vertices in xyz
  double tMin, tMax;
  uint32_t* queue;     // rays outside the bounded-error range (slow path)
  uint32_t* queue_len;
  uint32_t* work;      // persistent-kernel ray counter (zeroed before launch)
  unsigned* err;
  // Optional counters (nullptr = off): rays, binary64 slab decisions,
  // binary64 triangle decisions, binary64 closest values, binary64 final hits.
  unsigned long long* stats = nullptr;
  // Scenes (0, 1, ... top_scenes - 1) whose top BVH levels each block stages
  // in shared memory (0 = off); the launch passes top_smem_bytes(top_scenes).
  int top_scenes = 0;
  // Four-wide view of `nodes` (traverse_wide.cuh) for the wide kernels.
  const Node* wide = nullptr;
};


__device__ __forceinline__ void count_stat(const TravArgs& A, int k) {
  if (A.stats) atomicAdd(A.stats + k, 1ull);
}

// The BVH one ray traverses: the launch's (TravArgs) or, for policies that
// trace the rays of several scenes in one launch, its scene's.
struct BvhView {
  const Node* nodes;
  const float4* tris;
  uint32_t node_limit;
  int scene;
  const Node* wide = nullptr;  // four-wide view (traverse_wide.cuh), when built
};
template <class Pol>
__device__ __forceinline__ BvhView bvh_of(const TravArgs& A, const Pol& P, uint32_t k) {
  if constexpr (Pol::kMultiScene)
    return P.bvh(k);
  else
    return {A.nodes, A.tris, A.node_limit, 0};
}

// Top BVH levels in shared memory. The top kTopDepth + 1 levels of a tree
// (63 nodes, 2016 bytes) are copied at block start in breadth-first order,
// 1-based: treelet node b has children 2b and 2b + 1, stored side by side.
// Nodes are numbered depth-first in memory, so the treelet is a second copy,
// reached by carrying each node's treelet index beside it (a stack entry
// holds -b for treelet node b). Only where the nodes are read changes: the
// decisions and their order do not.
constexpr int kTopDepth = 5, kTopNodes = (1 << (kTopDepth + 1)) - 1, kTopMaxScenes = 8;
inline size_t top_smem_bytes(int scenes) { return (size_t)scenes * kTopNodes * sizeof(Node); }

// Treelet node b (1-based) of a tree: the path from the root follows the bits
// of b below its leading one (0 = left child). Nodes under a leaf, or past
// the node array, are absent: an inverted box, never read by a traversal of
// a valid tree.
__device__ __forceinline__ Node top_node(const Node* nodes, uint32_t limit, int b) {
  const float inf = __int_as_float(0x7f800000);
  const Node absent{make_float4(inf, inf, inf, 0.f), make_float4(-inf, -inf, -inf, 0.f)};
  if (limit == 0) return absent;
  int n = 0;
  for (int d = 30 - __clz(b); d >= 0; d--) {
    const Node nd = load_node(nodes, n);
    const int f = node_first(nd);
    if (node_count(nd) > 0 || f < 0 || (uint32_t)f + 1 >= limit) return absent;
    n = f + ((b >> d) & 1);
  }
  return load_node(nodes, n);
}

template <class Pol>
__device__ __forceinline__ BvhView scene_bvh_of(const TravArgs& A, const Pol& P, int s) {
  if constexpr (Pol::kMultiScene)
    return P.scene_bvh(s);
  else
    return {A.nodes, A.tris, A.node_limit, 0};
}

// Fills the block's treelets (all threads of the block must call it).
template <class Pol>
__device__ __forceinline__ void stage_top(const TravArgs& A, const Pol& P, Node* s_top) {
  for (int i = threadIdx.x; i < A.top_scenes * kTopNodes; i += blockDim.x) {
    const BvhView v = scene_bvh_of(A, P, i / kTopNodes);
    s_top[i] = top_node(v.nodes, v.node_limit, i % kTopNodes + 1);
  }
  __syncthreads();
}

struct PendingNode {
  int node;
  float ehi;
};

// Entire reference algorithm in binary64 for one ray (slow path, f64 rays).
// Returns false if the traversal was aborted (error word set).
template <class Pol>
__device__ bool trace_exact(const TravArgs& A, const Pol& P, const BvhView& bv, D3 o, D3 d, uint32_t key, int& slot,
                            double& t_out, double& u_out, double& v_out) {
  const D3 inv = {ddiv(1.0, d.x), ddiv(1.0, d.y), ddiv(1.0, d.z)};
  int stack[kTsStack];
  int sp = 0;
  stack[sp++] = 0;
  double closest = A.tMax;
  slot = -1;
  uint32_t iters = 0;
  while (sp > 0) {
    if (++iters > bv.node_limit) {
      atomicOr(A.err, kErrIterations);
      return false;
    }
    const int n = stack[--sp];
    const Node nd = load_node(bv.nodes, n);
    if (ts_slab_culled(nd.lo, nd.hi, o, inv, closest)) continue;
    const int cnt = node_count(nd), first = node_first(nd);
    if (cnt > 0) {
      for (int k = 0; k < cnt; k++) {
        const int s = first + k;
        const float4 a = __ldg(bv.tris + 3 * (size_t)s), b = __ldg(bv.tris + 3 * (size_t)s + 1),
                     c = __ldg(bv.tris + 3 * (size_t)s + 2);
        double t, u, v;
        if (ts_triangle(o, d, d3f(a), d3f(b), d3f(c), A.tMin, closest, t, u, v) &&
            P.alpha(bv.scene, s, key, (float)u, (float)v)) {
          closest = t;
          slot = s;
          t_out = t;
          u_out = u;
          v_out = v;
        }
      }
    } else {
      if (sp + 2 > kTsStack) {
        atomicOr(A.err, kErrStack);
        return false;
      }
      stack[sp++] = first + 1;
      stack[sp++] = first;
    }
  }
  return true;
}

template <class Pol>
__global__ void k_closest_exact_t(TravArgs A, Pol P) {
  const uint32_t limit = A.queue ? *A.queue_len : P.count();
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < limit; q += gridDim.x * blockDim.x) {
    const uint32_t k = A.queue ? A.queue[q] : q;
    float3 o, d;
    P.ray(k, o, d);
    int slot;
    double t = 0, u = 0, v = 0;
    if (!trace_exact(A, P, bvh_of(A, P, k), {o.x, o.y, o.z}, {d.x, d.y, d.z}, P.key(k), slot, t, u, v))
      P.fail(k);
    else if (slot < 0)
      P.miss(k);
    else
      P.hit(k, slot, t, u, v);
  }
}

// Fast path: persistent warps, one ray per lane; lanes refill from A.work as
// their rays finish. Both children of an inner node are tested with the
// current `c` (what the reference tests when it pops the left child, and the
// right one if the left is culled); a right child that passes is pushed with
// an upper bound on its entry distance and re-tested on pop only if `c` has
// dropped below it (the cull test is monotone in `c`). `c` is carried as
// binary32 bounds [c_lo, c_hi] of the reference's binary64 value.
// Block shape of the fast closest-hit kernel, per policy (Pol::kThreads,
// Pol::kMinBlocks): the register budget 65,536 / (threads x blocks) per
// thread sets the resident warps per SM. Deep traversals of long rays (the
// BVH API) gain from 28 warps at 72 registers; the renderer's short rays
// lose more to the extra spills and keep 24 warps at 80 (measured).
template <class Pol>
__global__ void __launch_bounds__(Pol::kThreads, Pol::kMinBlocks) k_closest_fast_t(TravArgs A, Pol P) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const float tmin_lo = __double2float_rd(A.tMin), tmin_hi = __double2float_ru(A.tMin);
  const float cmax_lo = __double2float_rd(A.tMax), cmax_hi = __double2float_ru(A.tMax);
  const double INF64 = __longlong_as_double(0x7ff0000000000000ll);
  const uint32_t n = P.count();
  const bool use_alpha = P.alpha_any();

  bool active = false, exhausted = false, have_cur = false, c_exact = true;
  uint32_t ri = 0, iters = 0, key = 0;
  Ray32 r;
  float c_lo = 0.f, c_hi = 0.f;
  double c64 = A.tMax;  // binary64 t of `best` when c_exact
  // pend: a triangle met at a distance tied with c within the binary32
  // bounds (kTriNearC), not yet compared in binary64; [c_lo, c_hi] then
  // spans both candidates' distances.
  int best = -1, pend = -1, sp = 0;
  BvhView bv{A.nodes, A.tris, A.node_limit, 0};  // multi-scene policies set it per ray below
  Node cur;
  PendingNode stack[kTsStack];
  extern __shared__ float4 s_top4[];
  Node* const s_top = reinterpret_cast<Node*>(s_top4);
  stage_top(A, P, s_top);
  const Node* sb = nullptr;  // this ray's treelet (null: its scene has none staged)
  int ctb = 0;               // treelet index of `cur` (0: not in the treelet)

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
            c_lo = cmax_lo;
            c_hi = cmax_hi;
            c64 = A.tMax;
            c_exact = true;
            best = -1;
            pend = -1;
            sp = 0;
            iters = 0;
            count_stat(A, 0);
            sb = bv.scene < A.top_scenes ? s_top + bv.scene * kTopNodes : nullptr;
            ctb = sb ? 1 : 0;
            cur = sb ? sb[0] : load_node(bv.nodes, 0);  // the reference pops the root first and tests its box
            SlabClass cl = classify_slab(r, cur.lo, cur.hi, c_lo, c_hi);
            if (cl == kAmbiguous) {
              count_stat(A, 1);
              cl = slab_f64_culled(cur.lo, cur.hi, o, d, c64) ? kCulled : kPass;
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
      if (!c_exact) {
        count_stat(A, 3);
        const float4 a = __ldg(bv.tris + 3 * (size_t)best), b = __ldg(bv.tris + 3 * (size_t)best + 1),
                     c = __ldg(bv.tris + 3 * (size_t)best + 2);
        const Tri64 h = tri_f64(r.o, r.d, a, b, c, A.tMin, INF64);
        c64 = h.t;
        c_exact = true;
        c_lo = __double2float_rd(h.t);
        c_hi = __double2float_ru(h.t);
      }
      if (pend >= 0) {  // the deferred tie: the reference took it iff its binary64 t is below c
        count_stat(A, 2);
        const float4 a = __ldg(bv.tris + 3 * (size_t)pend), b = __ldg(bv.tris + 3 * (size_t)pend + 1),
                     c = __ldg(bv.tris + 3 * (size_t)pend + 2);
        const Tri64 h = tri_f64(r.o, r.d, a, b, c, A.tMin, c64);
        if (h.hit) {
          best = pend;
          c64 = h.t;
        }
        pend = -1;
        c_lo = __double2float_rd(c64);
        c_hi = __double2float_ru(c64);
      }
      return c64;
    };
    auto slab_decide = [&](const Node& nd, SlabClass cl) {
      if (cl != kAmbiguous) return cl;
      count_stat(A, 1);
      return slab_f64_culled(nd.lo, nd.hi, r.o, r.d, exact_c()) ? kCulled : kPass;
    };

    if (!have_cur) {
      if (sp == 0) {  // finished
        if (pend >= 0) exact_c();
        if (best < 0) {
          P.miss(ri);
        } else {
          // Only the triangle: its t, u, v are computed afterwards with the
          // warp converged (lanes finish their rays at different steps, and
          // work at this point stalls the warp for each lane in turn).
          P.finish(ri, best);
        }
        active = false;
        continue;
      }
      const PendingNode e = stack[--sp];
      const Node nd = e.node < 0 ? sb[-e.node - 1] : load_node(bv.nodes, e.node);
      if (e.ehi > c_lo && slab_decide(nd, classify_slab(r, nd.lo, nd.hi, c_lo, c_hi)) == kCulled) continue;
      cur = nd;
      ctb = e.node < 0 ? -e.node : 0;
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
        const TriClass tc = mt_classify(r, a, b, c, tmin_lo, tmin_hi, c_lo, c_hi, tl, th, est);
        if (tc == kTriReject) continue;
        if (use_alpha) {  // depends on (key, slot) only, unless a texture must be sampled
          const AlphaAnswer aa = P.alpha_fast(bv.scene, slot, key);
          if (aa == kAlphaDefer) {
            defer = true;
            break;
          }
          if (aa == kAlphaPass) continue;
        }
        if (tc == kTriAccept) {
          best = slot;
          pend = -1;
          c_exact = false;
          c_lo = tl;
          c_hi = th;
          continue;
        }
        if (tc == kTriNearC && pend < 0) {  // defer: a later certain hit below both makes it moot
          pend = slot;
          c_lo = fminf(c_lo, tl);
          c_hi = fmaxf(c_hi, th);
          continue;
        }
        count_stat(A, 2);
        const double cc = exact_c();
        const Tri64 h = tri_f64(r.o, r.d, a, b, c, A.tMin, cc);
        if (h.hit) {
          best = slot;
          c64 = h.t;
          c_exact = true;
            c_lo = __double2float_rd(h.t);
          c_hi = __double2float_ru(h.t);
        }
      }
      have_cur = false;
      if (defer) {  // a textured alpha test: the binary64 kernel traces this ray
        A.queue[atomicAdd(A.queue_len, 1u)] = ri;
        active = false;
        continue;
      }
    } else {
      // One 64-byte pair, from the treelet while its children are in it.
      const bool in_top = ctb > 0 && 2 * ctb + 1 <= kTopNodes;
      const Node L = in_top ? sb[2 * ctb - 1] : load_node(bv.nodes, first);
      const Node R = in_top ? sb[2 * ctb] : load_node(bv.nodes, first + 1);
      const int ltb = in_top ? 2 * ctb : 0;
      float ehl, ehr;
      const SlabClass cl = slab_decide(L, classify_slab_e(r, L.lo, L.hi, c_lo, c_hi, ehl));
      const SlabClass cr = slab_decide(R, classify_slab_e(r, R.lo, R.hi, c_lo, c_hi, ehr));
      if (cl == kPass) {
        if (cr == kPass) {
          if (sp >= kTsStack) {  // unreachable for trees shallower than the reference's stack
            atomicOr(A.err, kErrStack);
            P.fail(ri);
            active = false;
            have_cur = false;
            continue;
          }
          stack[sp++] = {ltb ? -(ltb + 1) : first + 1, ehr};
        }
        cur = L;
        ctb = ltb;
      } else if (cr == kPass) {
        cur = R;
        ctb = ltb ? ltb + 1 : 0;
      } else {
        have_cur = false;
      }
    }
  }
}

// Any hit in binary64 (slow path).
template <class Pol>
__device__ bool any_exact(const TravArgs& A, const Pol& P, const BvhView& bv, D3 o, D3 d, uint32_t key, double tMax,
                          bool& ok) {
  const D3 inv = {ddiv(1.0, d.x), ddiv(1.0, d.y), ddiv(1.0, d.z)};
  int stack[kTsStack];
  int sp = 0;
  stack[sp++] = 0;
  uint32_t iters = 0;
  ok = true;
  while (sp > 0) {
    if (++iters > bv.node_limit) {
      atomicOr(A.err, kErrIterations);
      ok = false;
      return false;
    }
    const int n = stack[--sp];
    const Node nd = load_node(bv.nodes, n);
    if (ts_slab_culled(nd.lo, nd.hi, o, inv, tMax)) continue;
    const int cnt = node_count(nd), first = node_first(nd);
    if (cnt > 0) {
      for (int k = 0; k < cnt; k++) {
        const int s = first + k;
        const float4 a = __ldg(bv.tris + 3 * (size_t)s), b = __ldg(bv.tris + 3 * (size_t)s + 1),
                     c = __ldg(bv.tris + 3 * (size_t)s + 2);
        double t, u, v;
        if (ts_triangle(o, d, d3f(a), d3f(b), d3f(c), A.tMin, tMax, t, u, v) &&
            P.alpha(bv.scene, s, key, (float)u, (float)v))
          return true;
      }
    } else if (sp + 2 <= kTsStack) {
      stack[sp++] = first + 1;
      stack[sp++] = first;
    } else {
      atomicOr(A.err, kErrStack);
      ok = false;
      return false;
    }
  }
  return false;
}

// Any-hit rays carry their own tMax: P.tmax32(k).
template <class Pol>
__global__ void k_anyhit_exact_t(TravArgs A, Pol P) {
  const uint32_t limit = *A.queue_len;
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < limit; q += gridDim.x * blockDim.x) {
    const uint32_t k = A.queue[q];
    float3 o, d;
    P.ray(k, o, d);
    bool ok;
    const bool occ = any_exact(A, P, bvh_of(A, P, k), {o.x, o.y, o.z}, {d.x, d.y, d.z}, P.key(k), (double)P.tmax32(k), ok);
    P.shadow(k, ok ? occ : true);
  }
}

// Fast any hit: one ray per thread (grid-stride), depth-first, exits on the
// first triangle the reference's test certainly (or, in binary64, exactly)
// accepts. Culling at the fixed tMax.
template <class Pol>
__global__ void __launch_bounds__(256, 4) k_anyhit_fast_t(TravArgs A, Pol P) {
  const float tmin_lo = __double2float_rd(A.tMin), tmin_hi = __double2float_ru(A.tMin);
  const uint32_t n = P.count();
  const bool use_alpha = P.alpha_any();
  extern __shared__ float4 s_top4[];
  Node* const s_top = reinterpret_cast<Node*>(s_top4);
  stage_top(A, P, s_top);
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
    const BvhView bv = bvh_of(A, P, k);
    const float c_lo = tmax32, c_hi = tmax32;
    const Node* sb = bv.scene < A.top_scenes ? s_top + bv.scene * kTopNodes : nullptr;
    int stack[kTsStack];  // node index, or -b for treelet node b
    int sp = 0;
    stack[sp++] = sb ? -1 : 0;
    bool occ = false, ok = true, defer = false;
    uint32_t iters = 0;
    while (sp > 0 && !occ && !defer) {
      if (++iters > bv.node_limit) {
        atomicOr(A.err, kErrIterations);
        ok = false;
        break;
      }
      const int e = stack[--sp];
      const Node nd = e < 0 ? sb[-e - 1] : load_node(bv.nodes, e);
      SlabClass cl = classify_slab(r, nd.lo, nd.hi, c_lo, c_hi);
      if (cl == kAmbiguous) cl = ts_slab_culled(nd.lo, nd.hi, {o.x, o.y, o.z}, inv_exact(d), (double)tmax32) ? kCulled : kPass;
      if (cl == kCulled) continue;
      const int cnt = node_count(nd), first = node_first(nd);
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
      } else {
        if (sp + 2 > kTsStack) {
          atomicOr(A.err, kErrStack);
          ok = false;
          break;
        }
        const bool in_top = e < 0 && 2 * (-e) + 1 <= kTopNodes;
        stack[sp++] = in_top ? 2 * e - 1 : first + 1;  // -(2b + 1)
        stack[sp++] = in_top ? 2 * e : first;          // -(2b)
      }
    }
    if (defer && ok) {  // a textured alpha test: the binary64 kernel answers this ray
      A.queue[atomicAdd(A.queue_len, 1u)] = k;
      continue;
    }
    P.shadow(k, ok ? occ : true);
  }
}

int persistent_blocks(const void* kernel, int block);

}  // namespace lucent
