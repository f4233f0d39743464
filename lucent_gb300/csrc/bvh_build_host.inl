// Host orchestration of the GPU BVH builder (included by bvh_build.cu).
#include <vector>

#include "api_util.h"

namespace lucent {

// Builds the BVH of `n` triangles at `pos_d` (device, 9 floats each).
// Outputs the reference's node array and triIndices on the host, the bounds,
// and (optionally) the device traversal layout: Node array + slot-order
// triangles for a lucent_bvh handle.
lucent_status gpu_build_bvh(const float* pos_d, uint32_t n, int max_leaf, int bins, cudaStream_t s,
                            std::vector<float>& nodes_ref, std::vector<uint32_t>& tri_out, double bounds[6],
                            DeviceBuffer* nodes_dev, DeviceBuffer* tris_dev) {
  using namespace build;
  if (bins < 2 || bins > kMaxBins) return fail(LUCENT_ERR_UNSUPPORTED, "bins must be in [2, %d]", kMaxBins);
  if (max_leaf < 1) return fail(LUCENT_ERR_INVALID, "maxLeafSize must be >= 1");
  if (n > (1u << 23)) return fail(LUCENT_ERR_UNSUPPORTED, "%u triangles; the limit is 2^23", n);
  tri_out.assign(n, 0);
  if (n == 0) {  // bvh.ts:143-147
    nodes_ref.assign(8, 0.f);
    for (int k = 0; k < 6; k++) bounds[k] = 0;
    if (nodes_dev) {
      lucent_status st = nodes_dev->reserve(sizeof(Node));
      if (st) return st;
      cudaMemsetAsync(nodes_dev->ptr, 0, sizeof(Node), s);
    }
    if (tris_dev) {
      lucent_status st = tris_dev->reserve(48);
      if (st) return st;
    }
    return LUCENT_OK;
  }

  const uint32_t small_max = 2048;
  const uint32_t cap = n;
  // Scratch: prim bounds, orders, partition positions, node records, lists.
  DeviceBuffer b_lo, b_hi, b_cz, b_tri, b_tmp, b_P, b_Q, b_recs, b_ctr, b_small, b_bigA, b_bigB, b_info, b_chunks,
      b_first, b_part, b_bins, b_cnt;
  auto release_all = [&]() {
    for (DeviceBuffer* b : {&b_lo, &b_hi, &b_cz, &b_tri, &b_tmp, &b_P, &b_Q, &b_recs, &b_ctr, &b_small, &b_bigA,
                            &b_bigB, &b_info, &b_chunks, &b_first, &b_part, &b_bins, &b_cnt})
      b->release();
  };
  lucent_status st = LUCENT_OK;
#define BB_TRY(x)      \
  do {                 \
    st = (x);          \
    if (st) {          \
      release_all();   \
      return st;       \
    }                  \
  } while (0)
#define BB_CUDA(x, what)                      \
  do {                                        \
    cudaError_t e_ = (x);                     \
    if (e_ != cudaSuccess) {                  \
      release_all();                          \
      return cuda_fail(e_, what);             \
    }                                         \
  } while (0)
  const uint32_t nrec = 2 * n - 1;
  BB_TRY(b_lo.reserve((size_t)n * 16));
  BB_TRY(b_hi.reserve((size_t)n * 16));
  BB_TRY(b_cz.reserve((size_t)n * 4));
  BB_TRY(b_tri.reserve((size_t)n * 4));
  BB_TRY(b_tmp.reserve((size_t)n * 4));
  BB_TRY(b_P.reserve((size_t)n * 4));
  BB_TRY(b_Q.reserve((size_t)n * 4));
  BB_TRY(b_recs.reserve((size_t)nrec * sizeof(NodeRec)));
  BB_TRY(b_ctr.reserve(64));
  BB_TRY(b_small.reserve((size_t)cap * sizeof(Task)));
  BB_TRY(b_bigA.reserve((size_t)cap * sizeof(Task)));
  BB_TRY(b_bigB.reserve((size_t)cap * sizeof(Task)));

  uint32_t* ctr = (uint32_t*)b_ctr.ptr;  // [0] rec_count [1] small_count [2] big_next_count [3] err
  Ctx cx;
  cx.p = {(const float4*)b_lo.ptr, (const float4*)b_hi.ptr, (const float*)b_cz.ptr};
  cx.tri = (uint32_t*)b_tri.ptr;
  cx.tmp = (uint32_t*)b_tmp.ptr;
  cx.P = (int32_t*)b_P.ptr;
  cx.Q = (int32_t*)b_Q.ptr;
  cx.recs = (NodeRec*)b_recs.ptr;
  cx.rec_count = ctr;
  cx.small = (Task*)b_small.ptr;
  cx.small_count = ctr + 1;
  cx.big_next_count = ctr + 2;
  cx.err = ctr + 3;
  cx.cap = cap;
  cx.rec_cap = nrec;
  cx.max_leaf = max_leaf;
  cx.bins = bins;

  bb_prim_bounds(pos_d, n, (float4*)b_lo.ptr, (float4*)b_hi.ptr, (float*)b_cz.ptr, cx.tri, s);
  const Task root = {0, n, 0, 0};
  uint32_t init[4] = {1, 0, 0, 0};
  Task* big_cur = (Task*)b_bigA.ptr;
  Task* big_nxt = (Task*)b_bigB.ptr;
  uint32_t nbig = 0;
  if (n <= small_max) {
    init[1] = 1;
    BB_CUDA(cudaMemcpyAsync(cx.small, &root, sizeof(Task), cudaMemcpyHostToDevice, s), "upload root");
  } else {
    nbig = 1;
    BB_CUDA(cudaMemcpyAsync(big_cur, &root, sizeof(Task), cudaMemcpyHostToDevice, s), "upload root");
  }
  BB_CUDA(cudaMemcpyAsync(ctr, init, sizeof init, cudaMemcpyHostToDevice, s), "init counters");

  std::vector<Task> tasks_h;
  std::vector<Chunk> chunks_h;
  std::vector<uint32_t> first_h;
  int guard = 0;
  while (nbig > 0) {
    if (++guard > 4096) {
      release_all();
      return fail(LUCENT_ERR_DEVICE, "BVH build did not converge");
    }
    tasks_h.resize(nbig);
    BB_CUDA(cudaMemcpyAsync(tasks_h.data(), big_cur, nbig * sizeof(Task), cudaMemcpyDeviceToHost, s), "read tasks");
    BB_CUDA(cudaStreamSynchronize(s), "sync tasks");
    chunks_h.clear();
    first_h.assign(nbig + 1, 0);
    for (uint32_t t = 0; t < nbig; t++) {
      first_h[t] = (uint32_t)chunks_h.size();
      for (uint32_t b = tasks_h[t].start; b < tasks_h[t].end; b += kChunk)
        chunks_h.push_back({t, b, std::min(tasks_h[t].end, b + (uint32_t)kChunk), 0});
    }
    first_h[nbig] = (uint32_t)chunks_h.size();
    const uint32_t nch = (uint32_t)chunks_h.size();
    BB_TRY(b_chunks.reserve(nch * sizeof(Chunk)));
    BB_TRY(b_first.reserve((nbig + 1) * 4));
    BB_TRY(b_part.reserve((size_t)nch * 12 * 4));
    BB_TRY(b_bins.reserve((size_t)nch * 3 * bins * 7 * 4));
    BB_TRY(b_cnt.reserve((size_t)nch * 2 * 4));
    BB_TRY(b_info.reserve((size_t)nbig * sizeof(BigInfo)));
    BB_CUDA(cudaMemcpyAsync(b_chunks.ptr, chunks_h.data(), nch * sizeof(Chunk), cudaMemcpyHostToDevice, s), "chunks");
    BB_CUDA(cudaMemcpyAsync(b_first.ptr, first_h.data(), (nbig + 1) * 4, cudaMemcpyHostToDevice, s), "chunk index");
    BB_CUDA(cudaMemsetAsync(cx.big_next_count, 0, 4, s), "reset next");
    cx.big_next = big_nxt;
    const Chunk* ch = (const Chunk*)b_chunks.ptr;
    const uint32_t* fi = (const uint32_t*)b_first.ptr;
    BigInfo* info = (BigInfo*)b_info.ptr;
    k_big_measure<<<nch, 256, 0, s>>>(cx, ch, (float*)b_part.ptr);
    k_big_setup<<<(nbig * 32 + 127) / 128, 128, 0, s>>>(cx, big_cur, nbig, fi, (const float*)b_part.ptr, info);
    k_big_bins<<<nch, 256, 0, s>>>(cx, ch, info, (unsigned*)b_bins.ptr);
    k_big_sah<<<(nbig + 3) / 4, 128, 0, s>>>(cx, big_cur, nbig, fi, (const unsigned*)b_bins.ptr, info);
    k_big_count<<<nch, 256, 0, s>>>(cx, ch, big_cur, info, (uint32_t*)b_cnt.ptr);
    k_big_scan<<<(nbig + 127) / 128, 128, 0, s>>>(big_cur, nbig, fi, (uint32_t*)b_cnt.ptr, info, cx.err);
    k_big_place<<<nch, 256, 0, s>>>(cx, ch, big_cur, info, (const uint32_t*)b_cnt.ptr, 0);
    k_big_place<<<nch, 256, 0, s>>>(cx, ch, big_cur, info, (const uint32_t*)b_cnt.ptr, 1);
    k_big_copyback<<<nch, 256, 0, s>>>(cx, ch, info);
    k_big_finish<<<(nbig + 127) / 128, 128, 0, s>>>(cx, big_cur, nbig, info, small_max);
    BB_CUDA(cudaGetLastError(), "big-node kernels");
    BB_CUDA(cudaMemcpyAsync(&nbig, cx.big_next_count, 4, cudaMemcpyDeviceToHost, s), "read next count");
    BB_CUDA(cudaStreamSynchronize(s), "sync level");
    if (nbig > cap) {
      release_all();
      return fail(LUCENT_ERR_DEVICE, "task list overflow");
    }
    std::swap(big_cur, big_nxt);
  }
  // Small nodes level by level: the tasks of a level are processed by one
  // warp each, their children form the next level. Two task lists alternate
  // (the small list and a big-node list, free by now) with their counts in
  // ctr[1] and ctr[2]; the host checks for an empty level every 8 levels.
  {
    Task* lv[2] = {cx.small, big_nxt};
    uint32_t* lc[2] = {cx.small_count, cx.big_next_count};
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int g = 8 * (sms > 0 ? sms : 152);
    int cur = 0;
    for (int level = 0;; level++) {
      if (level >= 4096) {
        release_all();
        return fail(LUCENT_ERR_DEVICE, "BVH build did not converge");
      }
      if (level % 8 == 0) {  // any task left in the current level?
        uint32_t left = 0;
        BB_CUDA(cudaMemcpyAsync(&left, lc[cur], 4, cudaMemcpyDeviceToHost, s), "read small count");
        BB_CUDA(cudaStreamSynchronize(s), "sync small count");
        if (left == 0) break;
      }
      BB_CUDA(cudaMemsetAsync(lc[cur ^ 1], 0, 4, s), "reset small count");
      k_small_level<<<g, 128, 0, s>>>(cx, lv[cur], lc[cur], lv[cur ^ 1], lc[cur ^ 1]);
      BB_CUDA(cudaGetLastError(), "small-level kernel");
      cur ^= 1;
    }
  }
  uint32_t ctr_h[4];
  BB_CUDA(cudaMemcpyAsync(ctr_h, ctr, sizeof ctr_h, cudaMemcpyDeviceToHost, s), "read counters");
  BB_CUDA(cudaStreamSynchronize(s), "build");
  if (ctr_h[3]) {
    release_all();
    return fail(LUCENT_ERR_DEVICE, "BVH build raised device error 0x%x", ctr_h[3]);
  }
  const uint32_t nr = ctr_h[0];
  if (nr > nrec || (nr & 1) == 0) {
    release_all();
    return fail(LUCENT_ERR_DEVICE, "BVH build produced %u nodes", nr);
  }
  std::vector<NodeRec> recs(nr);
  BB_CUDA(cudaMemcpyAsync(recs.data(), cx.recs, nr * sizeof(NodeRec), cudaMemcpyDeviceToHost, s), "read nodes");
  BB_CUDA(cudaMemcpyAsync(tri_out.data(), cx.tri, (size_t)n * 4, cudaMemcpyDeviceToHost, s), "read triIndices");
  BB_CUDA(cudaStreamSynchronize(s), "read results");

  // Inner-node counts bottom-up (children always have larger temporary ids),
  // then DFS-preorder ranks top-down: left = parent + 1, right = parent + 1 +
  // inner nodes of the left subtree; children of rank k get ids 2k+1, 2k+2.
  std::vector<uint32_t> ic(nr, 0), rank(nr, 0), fid(nr, 0);
  for (uint32_t x = 0; x < nr; x++) {  // children are allocated after their parent, in pairs
    const NodeRec& r = recs[x];
    if (r.left >= 0 && (r.left <= (int32_t)x || r.right != r.left + 1 || (uint32_t)r.right >= nr)) {
      release_all();
      return fail(LUCENT_ERR_DEVICE, "BVH build produced a malformed node %u", x);
    }
  }
  for (int64_t x = (int64_t)nr - 1; x >= 0; x--)
    if (recs[x].left >= 0) ic[x] = 1 + ic[recs[x].left] + ic[recs[x].right];
  nodes_ref.assign((size_t)nr * 8, 0.f);
  for (uint32_t x = 0; x < nr; x++) {
    const NodeRec& r = recs[x];
    float* o = nodes_ref.data() + (size_t)fid[x] * 8;
    o[0] = r.lo[0], o[1] = r.lo[1], o[2] = r.lo[2];
    o[4] = r.hi[0], o[5] = r.hi[1], o[6] = r.hi[2];
    if (r.left >= 0) {
      const uint32_t k = rank[x];
      rank[r.left] = k + 1;
      rank[r.right] = k + 1 + ic[r.left];
      fid[r.left] = 2 * k + 1;
      fid[r.right] = 2 * k + 2;
      o[3] = (float)(2 * k + 1);
      o[7] = 0.f;
    } else {
      o[3] = (float)r.first;
      o[7] = (float)r.count;
    }
  }
  for (int k = 0; k < 3; k++) {  // bvh.ts:245-251: measure(0, triCount) = the root's box
    bounds[k] = recs[0].lo[k];
    bounds[3 + k] = recs[0].hi[k];
  }
  if (nodes_dev || tris_dev) {
    DeviceBuffer ref;
    BB_TRY(ref.reserve((size_t)nr * 32));
    cudaError_t e = cudaMemcpyAsync(ref.ptr, nodes_ref.data(), (size_t)nr * 32, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && nodes_dev) {
      st = nodes_dev->reserve((size_t)nr * sizeof(Node));
      if (!st) launch_pack_nodes((const float*)ref.ptr, nr, (Node*)nodes_dev->ptr, s);
    }
    if (e == cudaSuccess && !st && tris_dev) {
      st = tris_dev->reserve((size_t)n * 48);
      if (!st) launch_gather_tris(pos_d, cx.tri, n, (float4*)tris_dev->ptr, s);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    ref.release();
    if (e != cudaSuccess) {
      release_all();
      return cuda_fail(e, "pack built BVH");
    }
    if (st) {
      release_all();
      return st;
    }
  }
  release_all();
  return LUCENT_OK;
#undef BB_TRY
#undef BB_CUDA
}

}  // namespace lucent
