// GPU binned-SAH BVH builder whose output equals the reference's buildBVH
// (src/math/bvh.ts:52-252): same node array, same triIndices permutation.
//
// Why the result is the reference's:
//  * every per-node quantity the reference computes is either an exact
//    reduction (min/max of binary32 values, integer counts), which any order
//    reproduces, or binary64 arithmetic evaluated here in the reference's own
//    operation order (this file is compiled with -fmad=false);
//  * the SAH choice is the reference's first strict minimum (axis-major, bin
//    ascending): a parallel argmin with ties broken by candidate index;
//  * the in-place partition (bvh.ts:126-140) is sequential, but its final
//    permutation has a closed form computable from prefix counts (see
//    partition_dest below);
//  * nodes are built in any order under temporary ids and renumbered at the
//    end: the k-th inner node in left-first DFS preorder owns children
//    (2k+1, 2k+2) (bvh.ts:238-242).
// Big nodes (> 2048 triangles) are processed level by level with one block
// per chunk of triangles; smaller nodes level by level too, one warp per node,
// every node of a level in parallel (k_small_level).
#include <cfloat>

#include "common.cuh"
#include "internal.h"

namespace lucent {
namespace build {

constexpr int kMaxBins = 32;
constexpr int kChunk = 4096;  // triangles per block in the big-node pipeline

struct Task {
  uint32_t start, end;
  int32_t node;
  int32_t pad;
};

struct NodeRec {
  float lo[3], hi[3];
  uint32_t first, count;  // leaf range (count > 0) or 0
  int32_t left, right;    // temporary ids of the children, -1 for a leaf
};

struct Prims {
  const float4* lo;  // (min.xyz, centroid.x)
  const float4* hi;  // (max.xyz, centroid.y)
  const float* cz;   // centroid.z
};

__device__ __forceinline__ unsigned ord(float f) {
  const unsigned b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float unord(unsigned u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

__device__ __forceinline__ float cen_of(const Prims& p, uint32_t t, int a) {
  return a == 0 ? p.lo[t].w : a == 1 ? p.hi[t].w : p.cz[t];
}

// boxArea (bvh.ts:35-40), binary64, reference operation order.
__device__ __forceinline__ double box_area(double x0, double y0, double z0, double x1, double y1, double z1) {
  const double dx = x1 - x0, dy = y1 - y0, dz = z1 - z0;
  return dx < 0 ? 0.0 : 2 * ((dx * dy + dy * dz) + dz * dx);
}

// Per-node split setup shared by every thread that bins (bvh.ts:163-174).
struct Split {
  double cmin[3], scale[3];
  bool splittable[3];
};

__device__ __forceinline__ Split make_split(const float* cbox, uint32_t count, int bins) {
  Split s;
  const double e0 = (double)cbox[3] - (double)cbox[0], e1 = (double)cbox[4] - (double)cbox[1],
               e2 = (double)cbox[5] - (double)cbox[2];
  const int longest = e0 >= e1 && e0 >= e2 ? 0 : e1 >= e2 ? 1 : 2;
  const double ext[3] = {e0, e1, e2};
#pragma unroll
  for (int a = 0; a < 3; a++) {
    s.cmin[a] = (double)cbox[a];
    s.splittable[a] = ext[a] > 1e-9 && (count >= 512 || a == longest);
    s.scale[a] = (double)bins / ext[a];
  }
  return s;
}

// binOf (bvh.ts:122-123).
__device__ __forceinline__ int bin_of(const Split& s, float c, int a, int bins) {
  const double f = floor(((double)c - s.cmin[a]) * s.scale[a]);
  const int b = (int)fmin((double)(bins - 1), f);
  return b < 0 ? 0 : b;  // no-op for finite inputs (f >= 0); keeps any input in bounds
}

// Bins of one node: counts and binary32 bounds (as order-preserving uints).
struct BinsView {
  unsigned* cnt;  // [3*bins]
  unsigned* box;  // [3*bins*6]: min xyz (ord), max xyz (ord)
};

__device__ __forceinline__ void bins_clear(BinsView b, int bins, int tid, int nthreads) {
  for (int k = tid; k < 3 * bins; k += nthreads) {
    b.cnt[k] = 0;
    for (int c = 0; c < 3; c++) {
      b.box[k * 6 + c] = 0xffffffffu;
      b.box[k * 6 + 3 + c] = 0u;
    }
  }
}

__device__ __forceinline__ void bins_add(BinsView b, const Prims& p, const Split& s, uint32_t t, int bins) {
  const float4 lo = p.lo[t], hi = p.hi[t];
  const float cz = p.cz[t];
  const float c[3] = {lo.w, hi.w, cz};
  const unsigned ol[3] = {ord(lo.x), ord(lo.y), ord(lo.z)};
  const unsigned oh[3] = {ord(hi.x), ord(hi.y), ord(hi.z)};
#pragma unroll
  for (int a = 0; a < 3; a++) {
    if (!s.splittable[a]) continue;
    const int k = a * bins + bin_of(s, c[a], a, bins);
    atomicAdd(&b.cnt[k], 1u);
#pragma unroll
    for (int q = 0; q < 3; q++) {
      atomicMin(&b.box[k * 6 + q], ol[q]);
      atomicMax(&b.box[k * 6 + 3 + q], oh[q]);
    }
  }
}

// SAH sweep (bvh.ts:191-223) by one warp: lane l evaluates candidates
// l, l+32, ...; candidate c = a*(bins-1) + b splits axis a after bin b. The
// reference keeps the first strict minimum in (a, b) order.
struct Choice {
  double cost;
  int axis, bin;
  uint32_t left_count;
};

__device__ Choice warp_sah(const unsigned* cnt, const unsigned* box, const Split& s, int bins, int lane) {
  double best = __longlong_as_double(0x7ff0000000000000ll);
  int bestc = 0x7fffffff;
  uint32_t bestn = 0;
  const int ncand = 3 * (bins - 1);
  for (int c = lane; c < ncand; c += 32) {
    const int a = c / (bins - 1), b = c % (bins - 1);
    if (!s.splittable[a]) continue;
    unsigned lmin[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, lmax[3] = {0, 0, 0};
    unsigned rmin[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, rmax[3] = {0, 0, 0};
    uint32_t ln = 0, rn = 0;
    for (int k = 0; k < bins; k++) {
      const int o = (a * bins + k) * 6;
      const unsigned n = cnt[a * bins + k];
      if (k <= b) {
        ln += n;
        for (int q = 0; q < 3; q++) {
          lmin[q] = min(lmin[q], box[o + q]);
          lmax[q] = max(lmax[q], box[o + 3 + q]);
        }
      } else {
        rn += n;
        for (int q = 0; q < 3; q++) {
          rmin[q] = min(rmin[q], box[o + q]);
          rmax[q] = max(rmax[q], box[o + 3 + q]);
        }
      }
    }
    if (ln == 0 || rn == 0) continue;
    // Empty bins contribute +-inf in the reference; only non-empty sides are
    // costed, so the unions above are finite.
    const double la = box_area(unord(lmin[0]), unord(lmin[1]), unord(lmin[2]), unord(lmax[0]), unord(lmax[1]),
                               unord(lmax[2]));
    const double ra = box_area(unord(rmin[0]), unord(rmin[1]), unord(rmin[2]), unord(rmax[0]), unord(rmax[1]),
                               unord(rmax[2]));
    const double cost = la * (double)ln + ra * (double)rn;
    if (cost < best) {  // candidates of one lane arrive in increasing c
      best = cost;
      bestc = c;
      bestn = ln;
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const double oc = __shfl_xor_sync(0xffffffffu, best, off);
    const int oi = __shfl_xor_sync(0xffffffffu, bestc, off);
    const uint32_t on = __shfl_xor_sync(0xffffffffu, bestn, off);
    if (oc < best || (oc == best && oi < bestc)) {
      best = oc;
      bestc = oi;
      bestn = on;
    }
  }
  Choice ch;
  ch.cost = best;
  ch.axis = bestc == 0x7fffffff ? -1 : bestc / (bins - 1);
  ch.bin = bestc == 0x7fffffff ? -1 : bestc % (bins - 1);
  ch.left_count = bestn;
  return ch;
}

// Destination of the element at relative position r after the reference's
// in-place partition (bvh.ts:126-140). n elements, L left-goers, m = number
// of right-goers in [0, L) = number of left-goers in [L, n).
//   front left-goer            stays
//   k-th front right-goer      -> n-1 (k = 0) or Q[k-1]-1
//   j-th back left-goer (from the end) -> P[j]
//   back right-goer with a back left-goer below it -> r-1
//   other back right-goers     -> r-1, except r = L -> Q[m-1]-1 (or n-1 if m = 0)
// with P[k] the k-th front right-goer's position (ascending) and Q[j] the
// j-th back left-goer's position counted from the end (Q[j] = Qasc[m-1-j]).
// Returns n (an impossible destination) if the counts are inconsistent; the
// caller then raises the error word instead of writing out of bounds.
__device__ __forceinline__ uint32_t partition_dest(uint32_t r, bool left, uint32_t L, uint32_t n, uint32_t m,
                                                   uint32_t rank_fr, uint32_t rank_bl_asc, uint32_t bl_before,
                                                   const int32_t* P, const int32_t* Qasc) {
  uint32_t d;
  if (r < L) {
    if (left) return r;
    if (rank_fr == 0) return n - 1;
    if (rank_fr > m) return n;
    d = (uint32_t)Qasc[m - rank_fr] - 1u;
  } else if (left) {
    if (rank_bl_asc >= m) return n;
    d = (uint32_t)P[m - 1 - rank_bl_asc];
  } else if (bl_before > 0 || r != L) {
    return r - 1;
  } else {
    d = m > 0 ? (uint32_t)Qasc[0] - 1u : n - 1;
  }
  return d < n ? d : n;
}

struct Ctx {
  Prims p;
  uint32_t* tri;
  uint32_t* tmp;
  int32_t* P;
  int32_t* Q;
  NodeRec* recs;
  uint32_t* rec_count;
  Task* small;        // subtrees finished by one warp
  uint32_t* small_count;
  Task* big_next;     // next level of big nodes
  uint32_t* big_next_count;
  uint32_t cap;       // capacity of each task list
  uint32_t rec_cap;   // capacity of recs (2N - 1)
  int max_leaf, bins;
  unsigned* err;
};

__device__ __forceinline__ void write_rec(NodeRec* r, const float* box, uint32_t first, uint32_t count, int left,
                                          int right) {
#pragma unroll
  for (int q = 0; q < 3; q++) {
    r->lo[q] = box[q];
    r->hi[q] = box[3 + q];
  }
  r->first = first;
  r->count = count;
  r->left = left;
  r->right = right;
}

__device__ __forceinline__ void push_task(Task* list, uint32_t* count, uint32_t cap, Task t, unsigned* err) {
  const uint32_t i = atomicAdd(count, 1u);
  if (i < cap)
    list[i] = t;
  else
    atomicOr(err, kErrQueue);
}

// ---------------------------------------------------------------------------
// Per-triangle bounds and centroids (bvh.ts:59-73) and the identity order.
// ---------------------------------------------------------------------------
__global__ void k_prim_bounds(const float* __restrict__ pos, uint32_t n, float4* __restrict__ lo4,
                              float4* __restrict__ hi4, float* __restrict__ cz, uint32_t* __restrict__ tri) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float* p = pos + (size_t)i * 9;
    float lo[3], hi[3], c[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
      const float p0 = p[a], p1 = p[3 + a], p2 = p[6 + a];
      lo[a] = fminf(p0, fminf(p1, p2));
      hi[a] = fmaxf(p0, fmaxf(p1, p2));
      c[a] = __double2float_rn(((double)lo[a] + (double)hi[a]) * 0.5);
    }
    lo4[i] = make_float4(lo[0], lo[1], lo[2], c[0]);
    hi4[i] = make_float4(hi[0], hi[1], hi[2], c[1]);
    cz[i] = c[2];
    tri[i] = i;
  }
}

// ---------------------------------------------------------------------------
// Warp-level node processing (used for every node of <= 2048 triangles).
// ---------------------------------------------------------------------------
__device__ __forceinline__ float warp_min(float v) {
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__device__ void warp_measure(const Ctx& cx, uint32_t start, uint32_t end, int lane, float* box, float* cbox) {
  float b[6] = {FLT_MAX * 2, FLT_MAX * 2, FLT_MAX * 2, -FLT_MAX * 2, -FLT_MAX * 2, -FLT_MAX * 2};
  float c[6] = {b[0], b[1], b[2], b[3], b[4], b[5]};
  for (uint32_t i = start + lane; i < end; i += 32) {
    const uint32_t t = cx.tri[i];
    const float4 lo = cx.p.lo[t], hi = cx.p.hi[t];
    const float cz = cx.p.cz[t];
    b[0] = fminf(b[0], lo.x), b[1] = fminf(b[1], lo.y), b[2] = fminf(b[2], lo.z);
    b[3] = fmaxf(b[3], hi.x), b[4] = fmaxf(b[4], hi.y), b[5] = fmaxf(b[5], hi.z);
    c[0] = fminf(c[0], lo.w), c[1] = fminf(c[1], hi.w), c[2] = fminf(c[2], cz);
    c[3] = fmaxf(c[3], lo.w), c[4] = fmaxf(c[4], hi.w), c[5] = fmaxf(c[5], cz);
  }
#pragma unroll
  for (int q = 0; q < 3; q++) {
    box[q] = warp_min(b[q]);
    box[3 + q] = warp_max(b[3 + q]);
    cbox[q] = warp_min(c[q]);
    cbox[3 + q] = warp_max(c[3 + q]);
  }
}

// Partition of [start, end) by one warp; returns mid.
__device__ uint32_t warp_partition(const Ctx& cx, uint32_t start, uint32_t end, const Split& s, int axis, int split,
                                   uint32_t L, int lane) {
  const uint32_t n = end - start;
  const unsigned lt = (1u << lane) - 1u;
  int32_t* P = cx.P + start;
  int32_t* Qa = cx.Q + start;
  // Pass 1: positions of front right-goers (P) and back left-goers (Qasc).
  uint32_t fr = 0, bl = 0;
  for (uint32_t base = 0; base < n; base += 32) {
    const uint32_t r = base + lane;
    bool left = false;
    if (r < n) left = bin_of(s, cen_of(cx.p, cx.tri[start + r], axis), axis, cx.bins) <= split;
    const bool is_fr = r < n && r < L && !left, is_bl = r < n && r >= L && left;
    const unsigned mfr = __ballot_sync(0xffffffffu, is_fr), mbl = __ballot_sync(0xffffffffu, is_bl);
    if (is_fr) P[fr + __popc(mfr & lt)] = (int32_t)r;
    if (is_bl) Qa[bl + __popc(mbl & lt)] = (int32_t)r;
    fr += __popc(mfr);
    bl += __popc(mbl);
  }
  const uint32_t m = fr;
  if (m != bl) atomicOr(cx.err, kErrQueue);  // impossible for a consistent binning
  __syncwarp();
  // Pass 2: destinations, scattered into tmp.
  fr = 0;
  bl = 0;
  for (uint32_t base = 0; base < n; base += 32) {
    const uint32_t r = base + lane;
    bool left = false;
    uint32_t t = 0;
    if (r < n) {
      t = cx.tri[start + r];
      left = bin_of(s, cen_of(cx.p, t, axis), axis, cx.bins) <= split;
    }
    const bool is_fr = r < n && r < L && !left, is_bl = r < n && r >= L && left;
    const unsigned mfr = __ballot_sync(0xffffffffu, is_fr), mbl = __ballot_sync(0xffffffffu, is_bl);
    const uint32_t rfr = fr + __popc(mfr & lt), rbl = bl + __popc(mbl & lt);
    if (r < n) {
      uint32_t d = partition_dest(r, left, L, n, m, rfr, rbl, rbl, P, Qa);
      if (d >= n) {
        atomicOr(cx.err, kErrQueue);
        d = r;
      }
      cx.tmp[start + d] = t;
    }
    fr += __popc(mfr);
    bl += __popc(mbl);
  }
  __syncwarp();
  for (uint32_t r = lane; r < n; r += 32) cx.tri[start + r] = cx.tmp[start + r];
  __syncwarp();
  return start + L;
}

// Processes one node with a warp. Returns true if it split; children tasks
// are written to *lt and *rt (temporary ids already allocated).
__device__ bool warp_node(const Ctx& cx, Task tk, int lane, unsigned* cnt, unsigned* box_s, Task* lt, Task* rt) {
  const uint32_t start = tk.start, end = tk.end, count = end - start;
  float box[6], cbox[6];
  warp_measure(cx, start, end, lane, box, cbox);
  NodeRec* rec = cx.recs + tk.node;
  if (count <= (uint32_t)cx.max_leaf) {  // bvh.ts:157-160
    if (lane == 0) write_rec(rec, box, start, count, -1, -1);
    return false;
  }
  const Split s = make_split(cbox, count, cx.bins);
  BinsView bv{cnt, box_s};
  bins_clear(bv, cx.bins, lane, 32);
  __syncwarp();
  for (uint32_t i = start + lane; i < end; i += 32) bins_add(bv, cx.p, s, cx.tri[i], cx.bins);
  __syncwarp();
  const Choice ch = warp_sah(cnt, box_s, s, cx.bins, lane);
  __syncwarp();
  const double leafCost = (double)count * box_area(box[0], box[1], box[2], box[3], box[4], box[5]);
  const bool unprofitable = ch.axis < 0 || ch.cost >= leafCost;  // bvh.ts:227-232
  if (unprofitable && count <= (uint32_t)cx.max_leaf * 4) {
    if (lane == 0) write_rec(rec, box, start, count, -1, -1);
    return false;
  }
  uint32_t mid = unprofitable ? ((start + end) >> 1)
                              : warp_partition(cx, start, end, s, ch.axis, ch.bin, ch.left_count, lane);
  if (mid == start || mid == end) mid = (start + end) >> 1;  // bvh.ts:236
  int id = 0;
  if (lane == 0) id = (int)atomicAdd(cx.rec_count, 2u);
  id = __shfl_sync(0xffffffffu, id, 0);
  if ((uint32_t)id + 2 > cx.rec_cap) {  // impossible for non-empty children; never write past recs
    if (lane == 0) {
      atomicOr(cx.err, kErrQueue);
      write_rec(rec, box, start, count, -1, -1);
    }
    return false;
  }
  if (lane == 0) write_rec(rec, box, 0, 0, id, id + 1);
  *lt = {start, mid, id, 0};
  *rt = {mid, end, id + 1, 0};
  return true;
}

// One level of the small nodes: warp w processes task w of `in` (grid-stride
// over *n_in), and a node that splits appends its two children to `out`. The
// host launches levels until no task is left, so every small node of a level
// runs in parallel instead of one warp walking a whole subtree.
__global__ void __launch_bounds__(128) k_small_level(Ctx cx, const Task* __restrict__ in,
                                                     const uint32_t* __restrict__ n_in, Task* __restrict__ out,
                                                     uint32_t* __restrict__ n_out) {
  __shared__ unsigned cnt_s[4][3 * kMaxBins];
  __shared__ unsigned box_s[4][3 * kMaxBins * 6];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t nt = min(*n_in, cx.cap);
  for (uint32_t w = blockIdx.x * 4 + warp; w < nt; w += gridDim.x * 4) {
    Task a, b;
    if (!warp_node(cx, in[w], lane, cnt_s[warp], box_s[warp], &a, &b)) continue;
    if (lane == 0) {
      const uint32_t k = atomicAdd(n_out, 2u);
      if (k + 2 <= cx.cap) {
        out[k] = a;
        out[k + 1] = b;
      } else {
        atomicOr(cx.err, kErrQueue);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Big-node pipeline (one level): chunks of kChunk triangles per block.
// ---------------------------------------------------------------------------
struct Chunk {
  uint32_t task, begin, end;  // absolute element range inside the task
  uint32_t pad;
};

struct BigInfo {  // per big task
  float box[6], cbox[6];
  Split split;
  int axis, bin, leaf, partition;
  uint32_t L, m, mid;
};

__device__ __forceinline__ float block_min(float v, float* sh) {
  v = warp_min(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  v = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : FLT_MAX * 2;
  if (w == 0) v = warp_min(v);
  return v;
}
__device__ __forceinline__ float block_max(float v, float* sh) {
  v = warp_max(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  v = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : -FLT_MAX * 2;
  if (w == 0) v = warp_max(v);
  return v;
}

__global__ void __launch_bounds__(256) k_big_measure(Ctx cx, const Chunk* __restrict__ chunks,
                                                     float* __restrict__ partial) {
  __shared__ float sh[32];
  const Chunk ck = chunks[blockIdx.x];
  float b[6] = {FLT_MAX * 2, FLT_MAX * 2, FLT_MAX * 2, -FLT_MAX * 2, -FLT_MAX * 2, -FLT_MAX * 2};
  float c[6] = {b[0], b[1], b[2], b[3], b[4], b[5]};
  for (uint32_t i = ck.begin + threadIdx.x; i < ck.end; i += blockDim.x) {
    const uint32_t t = cx.tri[i];
    const float4 lo = cx.p.lo[t], hi = cx.p.hi[t];
    const float cz = cx.p.cz[t];
    b[0] = fminf(b[0], lo.x), b[1] = fminf(b[1], lo.y), b[2] = fminf(b[2], lo.z);
    b[3] = fmaxf(b[3], hi.x), b[4] = fmaxf(b[4], hi.y), b[5] = fmaxf(b[5], hi.z);
    c[0] = fminf(c[0], lo.w), c[1] = fminf(c[1], hi.w), c[2] = fminf(c[2], cz);
    c[3] = fmaxf(c[3], lo.w), c[4] = fmaxf(c[4], hi.w), c[5] = fmaxf(c[5], cz);
  }
  float out[12];
  for (int q = 0; q < 3; q++) {
    out[q] = block_min(b[q], sh);
    out[3 + q] = block_max(b[3 + q], sh);
    out[6 + q] = block_min(c[q], sh);
    out[9 + q] = block_max(c[3 + q], sh);
  }
  if (threadIdx.x == 0)
    for (int q = 0; q < 12; q++) partial[blockIdx.x * 12 + q] = out[q];
}

// One warp per big task: reduce the chunk partials and set up the split.
__global__ void k_big_setup(Ctx cx, const Task* __restrict__ tasks, uint32_t ntasks,
                            const uint32_t* __restrict__ chunk_first, const float* __restrict__ partial,
                            BigInfo* __restrict__ info) {
  const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= ntasks) return;
  float v[12];
  for (int q = 0; q < 12; q++) v[q] = (q % 6) < 3 ? FLT_MAX * 2 : -FLT_MAX * 2;
  for (uint32_t c = chunk_first[w] + lane; c < chunk_first[w + 1]; c += 32)
    for (int q = 0; q < 12; q++) v[q] = (q % 6) < 3 ? fminf(v[q], partial[c * 12 + q]) : fmaxf(v[q], partial[c * 12 + q]);
  for (int q = 0; q < 12; q++) v[q] = (q % 6) < 3 ? warp_min(v[q]) : warp_max(v[q]);
  if (lane == 0) {
    BigInfo& I = info[w];
    for (int q = 0; q < 6; q++) {
      I.box[q] = v[q];
      I.cbox[q] = v[6 + q];
    }
    const uint32_t count = tasks[w].end - tasks[w].start;
    I.leaf = count <= (uint32_t)cx.max_leaf;
    I.split = make_split(I.cbox, count, cx.bins);
  }
}

__global__ void __launch_bounds__(256) k_big_bins(Ctx cx, const Chunk* __restrict__ chunks,
                                                  const BigInfo* __restrict__ info, unsigned* __restrict__ pbins) {
  __shared__ unsigned cnt[3 * kMaxBins];
  __shared__ unsigned box[3 * kMaxBins * 6];
  const Chunk ck = chunks[blockIdx.x];
  const BigInfo& I = info[ck.task];
  if (I.leaf) return;
  BinsView bv{cnt, box};
  bins_clear(bv, cx.bins, threadIdx.x, blockDim.x);
  __syncthreads();
  const Split s = I.split;
  for (uint32_t i = ck.begin + threadIdx.x; i < ck.end; i += blockDim.x) bins_add(bv, cx.p, s, cx.tri[i], cx.bins);
  __syncthreads();
  const int per = 3 * cx.bins * 7;
  for (int k = threadIdx.x; k < 3 * cx.bins; k += blockDim.x) {
    pbins[(size_t)blockIdx.x * per + k] = cnt[k];
    for (int q = 0; q < 6; q++) pbins[(size_t)blockIdx.x * per + 3 * cx.bins + k * 6 + q] = box[k * 6 + q];
  }
}

// One warp per big task: merge bins, SAH, leaf / split decision.
__global__ void k_big_sah(Ctx cx, const Task* __restrict__ tasks, uint32_t ntasks,
                          const uint32_t* __restrict__ chunk_first, const unsigned* __restrict__ pbins,
                          BigInfo* __restrict__ info) {
  __shared__ unsigned cnt_s[4][3 * kMaxBins];
  __shared__ unsigned box_s[4][3 * kMaxBins * 6];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t w = blockIdx.x * 4 + warp;
  if (w >= ntasks) return;
  BigInfo& I = info[w];
  if (I.leaf) {
    if (lane == 0) {
      I.partition = 0;
      write_rec(cx.recs + tasks[w].node, I.box, tasks[w].start, tasks[w].end - tasks[w].start, -1, -1);
    }
    return;
  }
  const int bins = cx.bins, per = 3 * bins * 7;
  unsigned* cnt = cnt_s[warp];
  unsigned* box = box_s[warp];
  for (int k = lane; k < 3 * bins; k += 32) {
    unsigned n = 0, mn[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, mx[3] = {0, 0, 0};
    for (uint32_t c = chunk_first[w]; c < chunk_first[w + 1]; c++) {
      const unsigned* pb = pbins + (size_t)c * per;
      n += pb[k];
      for (int q = 0; q < 3; q++) {
        mn[q] = min(mn[q], pb[3 * bins + k * 6 + q]);
        mx[q] = max(mx[q], pb[3 * bins + k * 6 + 3 + q]);
      }
    }
    cnt[k] = n;
    for (int q = 0; q < 3; q++) {
      box[k * 6 + q] = mn[q];
      box[k * 6 + 3 + q] = mx[q];
    }
  }
  __syncwarp();
  const Choice ch = warp_sah(cnt, box, I.split, bins, lane);
  if (lane != 0) return;
  const uint32_t start = tasks[w].start, end = tasks[w].end, count = end - start;
  const double leafCost = (double)count * box_area(I.box[0], I.box[1], I.box[2], I.box[3], I.box[4], I.box[5]);
  const bool unprofitable = ch.axis < 0 || ch.cost >= leafCost;
  if (unprofitable && count <= (uint32_t)cx.max_leaf * 4) {
    I.leaf = 1;
    I.partition = 0;
    write_rec(cx.recs + tasks[w].node, I.box, start, count, -1, -1);
    return;
  }
  I.partition = !unprofitable;
  I.axis = ch.axis;
  I.bin = ch.bin;
  I.L = ch.left_count;
  I.mid = unprofitable ? ((start + end) >> 1) : start + ch.left_count;
  if (I.mid == start || I.mid == end) I.mid = (start + end) >> 1;
}

// Counts of front right-goers / back left-goers per chunk.
__device__ __forceinline__ bool goes_left(const Ctx& cx, const BigInfo& I, uint32_t t) {
  return bin_of(I.split, cen_of(cx.p, t, I.axis), I.axis, cx.bins) <= I.bin;
}

__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  uint32_t r = 0;
  for (int k = 0; k < (int)(blockDim.x >> 5); k++) r += sh[k];
  return r;
}

__global__ void __launch_bounds__(256) k_big_count(Ctx cx, const Chunk* __restrict__ chunks, const Task* __restrict__ tasks,
                                                   const BigInfo* __restrict__ info, uint32_t* __restrict__ pcount) {
  __shared__ uint32_t sh[32];
  const Chunk ck = chunks[blockIdx.x];
  const BigInfo& I = info[ck.task];
  if (!I.partition) return;
  const uint32_t start = tasks[ck.task].start;
  uint32_t fr = 0, bl = 0;
  for (uint32_t i = ck.begin + threadIdx.x; i < ck.end; i += blockDim.x) {
    const bool left = goes_left(cx, I, cx.tri[i]);
    const uint32_t r = i - start;
    fr += (r < I.L && !left);
    bl += (r >= I.L && left);
  }
  fr = block_sum(fr, sh);
  bl = block_sum(bl, sh);
  if (threadIdx.x == 0) {
    pcount[2 * blockIdx.x] = fr;
    pcount[2 * blockIdx.x + 1] = bl;
  }
}

// Exclusive scan of chunk counts per task (one thread per task; few chunks).
__global__ void k_big_scan(const Task* __restrict__ tasks, uint32_t ntasks, const uint32_t* __restrict__ chunk_first,
                           uint32_t* __restrict__ pcount, BigInfo* __restrict__ info, unsigned* err) {
  const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= ntasks || !info[w].partition) return;
  uint32_t fr = 0, bl = 0;
  for (uint32_t c = chunk_first[w]; c < chunk_first[w + 1]; c++) {
    const uint32_t a = pcount[2 * c], b = pcount[2 * c + 1];
    pcount[2 * c] = fr;
    pcount[2 * c + 1] = bl;
    fr += a;
    bl += b;
  }
  if (fr != bl) atomicOr(err, kErrQueue);
  info[w].m = fr;
}

// Block-wide exclusive scan of two flags; returns ranks and the block totals.
__device__ __forceinline__ void block_scan2(bool f0, bool f1, uint32_t* sh, uint32_t& r0, uint32_t& r1,
                                            uint32_t& t0, uint32_t& t1) {
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
  const unsigned b0 = __ballot_sync(0xffffffffu, f0), b1 = __ballot_sync(0xffffffffu, f1);
  const unsigned lt = (1u << l) - 1u;
  __syncthreads();
  if (l == 0) {
    sh[w] = __popc(b0);
    sh[32 + w] = __popc(b1);
  }
  __syncthreads();
  uint32_t o0 = 0, o1 = 0, s0 = 0, s1 = 0;
  for (int k = 0; k < nw; k++) {
    if (k < w) {
      o0 += sh[k];
      o1 += sh[32 + k];
    }
    s0 += sh[k];
    s1 += sh[32 + k];
  }
  r0 = o0 + __popc(b0 & lt);
  r1 = o1 + __popc(b1 & lt);
  t0 = s0;
  t1 = s1;
}

// mode 0: write P / Qasc; mode 1: scatter to tmp.
__global__ void __launch_bounds__(256) k_big_place(Ctx cx, const Chunk* __restrict__ chunks, const Task* __restrict__ tasks,
                                                   const BigInfo* __restrict__ info,
                                                   const uint32_t* __restrict__ pcount, int mode) {
  __shared__ uint32_t sh[64];
  const Chunk ck = chunks[blockIdx.x];
  const BigInfo& I = info[ck.task];
  if (!I.partition) return;
  const uint32_t start = tasks[ck.task].start, n = tasks[ck.task].end - start;
  int32_t* P = cx.P + start;
  int32_t* Qa = cx.Q + start;
  uint32_t fr = pcount[2 * blockIdx.x], bl = pcount[2 * blockIdx.x + 1];
  const uint32_t len = ck.end - ck.begin;
  for (uint32_t base = 0; base < len; base += blockDim.x) {  // uniform trip count per block
    const uint32_t i = ck.begin + base + threadIdx.x;
    const bool valid = base + threadIdx.x < len;
    uint32_t t = 0;
    bool left = false;
    if (valid) {
      t = cx.tri[i];
      left = goes_left(cx, I, t);
    }
    const uint32_t r = i - start;
    const bool is_fr = valid && r < I.L && !left, is_bl = valid && r >= I.L && left;
    uint32_t rfr, rbl, tfr, tbl;
    block_scan2(is_fr, is_bl, sh, rfr, rbl, tfr, tbl);
    rfr += fr;
    rbl += bl;
    if (mode == 0) {
      if (is_fr) P[rfr] = (int32_t)r;
      if (is_bl) Qa[rbl] = (int32_t)r;
    } else if (valid) {
      uint32_t d = partition_dest(r, left, I.L, n, I.m, rfr, rbl, rbl, P, Qa);
      if (d >= n) {
        atomicOr(cx.err, kErrQueue);
        d = r;
      }
      cx.tmp[start + d] = t;
    }
    fr += tfr;
    bl += tbl;
  }
}

__global__ void k_big_copyback(Ctx cx, const Chunk* __restrict__ chunks, const BigInfo* __restrict__ info) {
  const Chunk ck = chunks[blockIdx.x];
  if (!info[ck.task].partition) return;
  for (uint32_t i = ck.begin + threadIdx.x; i < ck.end; i += blockDim.x) cx.tri[i] = cx.tmp[i];
}

// One thread per big task: allocate children, write the node, route children.
__global__ void k_big_finish(Ctx cx, const Task* __restrict__ tasks, uint32_t ntasks, const BigInfo* __restrict__ info,
                             uint32_t small_max) {
  const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= ntasks) return;
  const BigInfo& I = info[w];
  if (I.leaf) return;
  const Task tk = tasks[w];
  const int id = (int)atomicAdd(cx.rec_count, 2u);
  if ((uint32_t)id + 2 > cx.rec_cap) {
    atomicOr(cx.err, kErrQueue);
    write_rec(cx.recs + tk.node, I.box, tk.start, tk.end - tk.start, -1, -1);
    return;
  }
  write_rec(cx.recs + tk.node, I.box, 0, 0, id, id + 1);
  const Task kids[2] = {{tk.start, I.mid, id, 0}, {I.mid, tk.end, id + 1, 0}};
  for (int k = 0; k < 2; k++) {
    if (kids[k].end - kids[k].start <= small_max)
      push_task(cx.small, cx.small_count, cx.cap, kids[k], cx.err);
    else
      push_task(cx.big_next, cx.big_next_count, cx.cap, kids[k], cx.err);
  }
}

// ---------------------------------------------------------------------------
// Renumbering (bvh.ts:238-242): inner-node subtree counts bottom-up, DFS
// preorder ranks top-down, then the reference's node array.
// ---------------------------------------------------------------------------
}  // namespace build

using namespace build;

struct BuildScratch;

// Host orchestration lives in bvh_build_host.cu; these launchers are its
// interface to the kernels above.
void bb_prim_bounds(const float* pos, uint32_t n, float4* lo, float4* hi, float* cz, uint32_t* tri, cudaStream_t s) {
  int g = (int)((n + 255) / 256);
  if (g < 1) g = 1;
  if (g > 152 * 64) g = 152 * 64;
  k_prim_bounds<<<g, 256, 0, s>>>(pos, n, lo, hi, cz, tri);
}

}  // namespace lucent

#include "bvh_build_host.inl"
