// C ABI: status codes, thread-local error text, BVH handle for closest-hit.
#include <cmath>
#include <cstring>
#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/lucent.h"
#include "api_util.h"
#include "internal.h"

using namespace lucent;

namespace lucent {

static thread_local std::string g_last_error;

lucent_status fail(lucent_status code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

void clear_error() { g_last_error.clear(); }

lucent_status cuda_fail(cudaError_t e, const char* what) {
  cudaGetLastError();  // clear the sticky-free error state
  if (e == cudaErrorMemoryAllocation) return fail(LUCENT_ERR_OOM, "%s: %s", what, cudaGetErrorString(e));
  return fail(LUCENT_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

lucent_status DeviceBuffer::reserve(size_t bytes) {
  if (bytes <= cap) return LUCENT_OK;
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
  cap = 0;
  size_t want = bytes < 256 ? 256 : bytes;
  cudaError_t e = cudaMalloc(&ptr, want);
  if (e != cudaSuccess) {
    ptr = nullptr;
    return cuda_fail(e, "cudaMalloc");
  }
  cap = want;
  return LUCENT_OK;
}

void DeviceBuffer::release() {
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
  cap = 0;
}

}  // namespace lucent

struct lucent_bvh {
  uint32_t node_count = 0, tri_count = 0;
  // Tree depth (root = 0). Trees whose depth could overflow the reference's
  // 64-entry stack take the all-binary64 path, which reproduces the overflow.
  uint32_t depth = 0;
  int mode = LUCENT_TRAVERSE_WIDE;
  DeviceBuffer nodes, tris, scratch, stage;
  DeviceBuffer wide;  // four-wide view of `nodes` (LUCENT_TRAVERSE_WIDE), built on first use
};

extern "C" {

const char* lucent_last_error(void) { return g_last_error.c_str(); }
int32_t lucent_version(void) { return 100; }

// Depth of a (validated) reference-layout tree; root = 0.
uint32_t tree_depth(const float* nodes, uint32_t node_count, uint32_t tri_count) {
  if (tri_count == 0 || node_count == 0) return 0;
  std::vector<std::pair<uint32_t, uint32_t>> st{{0u, 0u}};
  uint32_t depth = 0;
  while (!st.empty()) {
    const auto [n, d] = st.back();
    st.pop_back();
    depth = d > depth ? d : depth;
    const float* r = nodes + (size_t)n * 8;
    if (r[7] > 0) continue;
    const uint32_t l = (uint32_t)r[3];
    st.push_back({l, d + 1});
    st.push_back({l + 1, d + 1});
  }
  return depth;
}

// Validates the reference layout so that no kernel can read out of bounds:
// children inside the array, leaf ranges inside triIndices, indices in range.
lucent_status validate_bvh(const float* nodes, uint32_t node_count, const uint32_t* tri, uint32_t tri_count) {
  if (node_count == 0) return fail(LUCENT_ERR_INVALID, "BVH has no nodes");
  if (tri_count > (1u << 23)) return fail(LUCENT_ERR_UNSUPPORTED, "%u triangles; the limit is 2^23", tri_count);
  for (uint32_t i = 0; i < tri_count; i++)
    if (tri[i] >= tri_count) return fail(LUCENT_ERR_INVALID, "triIndices[%u] = %u out of range", i, tri[i]);
  if (tri_count == 0) return LUCENT_OK;
  for (uint32_t n = 0; n < node_count; n++) {
    const float* r = nodes + (size_t)n * 8;
    const float lf = r[3], cnt = r[7];
    if (!(lf >= 0) || !(cnt >= 0) || lf != std::floor(lf) || cnt != std::floor(cnt))
      return fail(LUCENT_ERR_INVALID, "node %u has a malformed leftFirst/count", n);
    if (cnt > 0) {
      if ((double)lf + cnt > tri_count) return fail(LUCENT_ERR_INVALID, "leaf %u range past triIndices", n);
    } else if ((double)lf + 1 >= node_count || lf <= n) {
      return fail(LUCENT_ERR_INVALID, "node %u children out of range", n);
    }
    for (int k : {0, 1, 2, 4, 5, 6})
      if (!std::isfinite(r[k])) return fail(LUCENT_ERR_INVALID, "node %u has a non-finite bound", n);
  }
  return LUCENT_OK;
}

lucent_status lucent_bvh_create(const float* nodes, uint32_t node_count, const uint32_t* tri_indices,
                                uint32_t tri_count, const float* positions, lucent_bvh** out) {
  clear_error();
  if (!out || !nodes || (tri_count && (!tri_indices || !positions)))
    return fail(LUCENT_ERR_INVALID, "null argument");
  *out = nullptr;
  lucent_status st = validate_bvh(nodes, node_count, tri_indices, tri_count);
  if (st) return st;
  lucent_bvh* b = new lucent_bvh();
  b->node_count = node_count;
  b->tri_count = tri_count;
  b->depth = tree_depth(nodes, node_count, tri_count);
  DeviceBuffer ref, pos, idx;
  cudaStream_t s = 0;
  auto cleanup = [&](lucent_status code) {
    ref.release();
    pos.release();
    idx.release();
    if (code) lucent_bvh_destroy(b);
    return code;
  };
  if ((st = b->nodes.reserve((size_t)node_count * sizeof(Node)))) return cleanup(st);
  if ((st = b->tris.reserve((size_t)(tri_count ? tri_count : 1) * 48))) return cleanup(st);
  if ((st = ref.reserve((size_t)node_count * 32))) return cleanup(st);
  cudaError_t e = cudaMemcpyAsync(ref.ptr, nodes, (size_t)node_count * 32, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cleanup(cuda_fail(e, "upload nodes"));
  launch_pack_nodes((const float*)ref.ptr, node_count, (Node*)b->nodes.ptr, s);
  if (tri_count) {
    if ((st = pos.reserve((size_t)tri_count * 36)) || (st = idx.reserve((size_t)tri_count * 4))) return cleanup(st);
    e = cudaMemcpyAsync(pos.ptr, positions, (size_t)tri_count * 36, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(idx.ptr, tri_indices, (size_t)tri_count * 4, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cleanup(cuda_fail(e, "upload triangles"));
    launch_gather_tris((const float*)pos.ptr, (const uint32_t*)idx.ptr, tri_count, (float4*)b->tris.ptr, s);
  }
  e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return cleanup(cuda_fail(e, "bvh upload kernels"));
  cleanup(LUCENT_OK);
  *out = b;
  return LUCENT_OK;
}

static lucent_status build_common(const float* pos_d, uint32_t n, const lucent_bvh_opts* opts, cudaStream_t s,
                                  float* nodes_out, uint32_t* node_count_out, uint32_t* tri_out, double* bounds_out,
                                  lucent_bvh** handle_out) {
  const int max_leaf = opts ? (int)opts->max_leaf_size : 4;  // bvh.ts:33 defaults
  const int bins = opts ? (int)opts->bins : 12;
  std::vector<float> nodes;
  std::vector<uint32_t> tri;
  double bounds[6];
  lucent_bvh* b = handle_out ? new lucent_bvh() : nullptr;
  lucent_status st = gpu_build_bvh(pos_d, n, max_leaf, bins, s, nodes, tri, bounds, b ? &b->nodes : nullptr,
                                   b ? &b->tris : nullptr);
  if (st) {
    lucent_bvh_destroy(b);
    return st;
  }
  const uint32_t nc = (uint32_t)(nodes.size() / 8);
  if (nodes_out) memcpy(nodes_out, nodes.data(), nodes.size() * 4);
  if (node_count_out) *node_count_out = nc;
  if (tri_out && n) memcpy(tri_out, tri.data(), (size_t)n * 4);
  if (bounds_out) memcpy(bounds_out, bounds, sizeof bounds);
  if (b) {
    b->node_count = nc;
    b->tri_count = n;
    b->depth = tree_depth(nodes.data(), nc, n);
    *handle_out = b;
  }
  return LUCENT_OK;
}

lucent_status lucent_bvh_build(const float* positions, uint64_t n_floats, const lucent_bvh_opts* opts,
                               float* nodes_out, uint32_t* node_count_out, uint32_t* tri_indices_out,
                               double* bounds_out, lucent_bvh** handle_out, void* stream) {
  clear_error();
  if (handle_out) *handle_out = nullptr;
  if (n_floats % 9 != 0)  // bvh.ts:55-57
    return fail(LUCENT_ERR_INVALID, "positions length %llu is not a multiple of 9", (unsigned long long)n_floats);
  if (n_floats && !positions) return fail(LUCENT_ERR_INVALID, "null positions");
  const uint64_t n = n_floats / 9;
  if (n > (1u << 23)) return fail(LUCENT_ERR_UNSUPPORTED, "%llu triangles; the limit is 2^23", (unsigned long long)n);
  for (uint64_t i = 0; i < n_floats; i++)
    if (!std::isfinite(positions[i])) return fail(LUCENT_ERR_UNSUPPORTED, "positions[%llu] is not finite", (unsigned long long)i);
  cudaStream_t s = (cudaStream_t)stream;
  DeviceBuffer pos;
  lucent_status st = pos.reserve(n_floats * 4 + 4);
  if (st) return st;
  cudaError_t e = cudaMemcpyAsync(pos.ptr, positions, n_floats * 4, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) {
    pos.release();
    return cuda_fail(e, "upload positions");
  }
  st = build_common((const float*)pos.ptr, (uint32_t)n, opts, s, nodes_out, node_count_out, tri_indices_out,
                    bounds_out, handle_out);
  cudaStreamSynchronize(s);
  pos.release();
  return st;
}

lucent_status lucent_bvh_build_device(const float* positions_d, uint32_t tri_count, const lucent_bvh_opts* opts,
                                      lucent_bvh** handle_out, void* stream) {
  clear_error();
  if (!handle_out || (tri_count && !positions_d)) return fail(LUCENT_ERR_INVALID, "null argument");
  *handle_out = nullptr;
  return build_common(positions_d, tri_count, opts, (cudaStream_t)stream, nullptr, nullptr, nullptr, nullptr,
                      handle_out);
}

void lucent_bvh_destroy(lucent_bvh* b) {
  if (!b) return;
  b->nodes.release();
  b->tris.release();
  b->scratch.release();
  b->stage.release();
  delete b;
}

lucent_status lucent_bvh_info(const lucent_bvh* b, uint32_t* node_count, uint32_t* tri_count) {
  clear_error();
  if (!b) return fail(LUCENT_ERR_INVALID, "null bvh");
  if (node_count) *node_count = b->node_count;
  if (tri_count) *tri_count = b->tri_count;
  return LUCENT_OK;
}

lucent_status lucent_bvh_download(const lucent_bvh* b, float* nodes_out, uint32_t* tri_indices_out) {
  clear_error();
  if (!b || !nodes_out || (b->tri_count && !tri_indices_out)) return fail(LUCENT_ERR_INVALID, "null argument");
  DeviceBuffer tmp;
  lucent_status st = tmp.reserve((size_t)b->node_count * 32 + (size_t)b->tri_count * 4 + 16);
  if (st) return st;
  float* ref_d = (float*)tmp.ptr;
  uint32_t* idx_d = (uint32_t*)((char*)tmp.ptr + (size_t)b->node_count * 32);
  launch_unpack((const Node*)b->nodes.ptr, b->node_count, (const float4*)b->tris.ptr, b->tri_count, ref_d, idx_d, 0);
  cudaError_t e = cudaMemcpy(nodes_out, ref_d, (size_t)b->node_count * 32, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && b->tri_count)
    e = cudaMemcpy(tri_indices_out, idx_d, (size_t)b->tri_count * 4, cudaMemcpyDeviceToHost);
  tmp.release();
  return e == cudaSuccess ? LUCENT_OK : cuda_fail(e, "download bvh");
}

lucent_status lucent_bvh_set_mode(lucent_bvh* b, int32_t mode) {
  clear_error();
  if (!b) return fail(LUCENT_ERR_INVALID, "null bvh");
  if (mode != LUCENT_TRAVERSE_FAST && mode != LUCENT_TRAVERSE_EXACT && mode != LUCENT_TRAVERSE_FAST_GLOBAL &&
      mode != LUCENT_TRAVERSE_WIDE)
    return fail(LUCENT_ERR_INVALID, "bad mode %d", mode);
  b->mode = mode;
  return LUCENT_OK;
}

static lucent_status check_tmin(double t_min, double t_max) {
  if (!(t_min >= 0) || std::isnan(t_max)) return fail(LUCENT_ERR_INVALID, "t_min must be >= 0 and t_max not NaN");
  return LUCENT_OK;
}

// Scratch layout: [err word][queue length][work counter][pad..][queue: n u32]
static lucent_status prepare_scratch(lucent_bvh* b, uint32_t n, cudaStream_t s, unsigned** err, uint32_t** qlen,
                                     uint32_t** queue, uint32_t** work = nullptr) {
  lucent_status st = b->scratch.reserve(256 + (size_t)n * 4);
  if (st) return st;
  char* base = (char*)b->scratch.ptr;
  *err = (unsigned*)base;
  *qlen = (uint32_t*)(base + 4);
  if (work) *work = (uint32_t*)(base + 8);
  *queue = (uint32_t*)(base + 256);
  cudaError_t e = cudaMemsetAsync(base, 0, 12, s);
  if (e != cudaSuccess) return cuda_fail(e, "memset scratch");
  return LUCENT_OK;
}

lucent_status lucent_bvh_intersect_device(lucent_bvh* b, const float* rays_d, uint32_t n, double t_min,
                                          double t_max, int32_t* prim_d, float* t_d, float* u_d, float* v_d,
                                          void* stream) {
  clear_error();
  if (!b || (n && (!rays_d || !prim_d))) return fail(LUCENT_ERR_INVALID, "null argument");
  lucent_status st = check_tmin(t_min, t_max);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  unsigned* err;
  uint32_t *qlen, *queue, *work;
  if ((st = prepare_scratch(b, n, s, &err, &qlen, &queue, &work))) return st;
  if (n == 0) return LUCENT_OK;
  if (b->tri_count == 0) {  // bvh.ts:274: an empty BVH never hits
    cudaError_t e = cudaMemsetAsync(prim_d, 0xff, (size_t)n * 4, s);
    return e == cudaSuccess ? LUCENT_OK : cuda_fail(e, "memset");
  }
  const Node* wide = nullptr;
  if (b->mode == LUCENT_TRAVERSE_WIDE) {
    if (!b->wide.ptr) {
      if ((st = b->wide.reserve((size_t)b->node_count * 4 * sizeof(Node)))) return st;
      launch_wide_view((const Node*)b->nodes.ptr, b->node_count, (Node*)b->wide.ptr, s);
    }
    wide = (const Node*)b->wide.ptr;
  }
  launch_closest((const Node*)b->nodes.ptr, b->node_count, (const float4*)b->tris.ptr, rays_d, n, t_min, t_max, prim_d, t_d, u_d,
                 v_d, queue, qlen, work, err, b->mode == LUCENT_TRAVERSE_EXACT || b->depth + 2 > kTsStack,
                 b->mode == LUCENT_TRAVERSE_FAST, s, wide);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LUCENT_OK : cuda_fail(e, "closest-hit launch");
}

lucent_status lucent_bvh_check(lucent_bvh* b, void* stream) {
  clear_error();
  if (!b) return fail(LUCENT_ERR_INVALID, "null bvh");
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "synchronize");
  if (!b->scratch.ptr) return LUCENT_OK;
  unsigned word = 0;
  e = cudaMemcpy(&word, b->scratch.ptr, 4, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "read error word");
  if (word) {
    cudaMemset(b->scratch.ptr, 0, 4);
    if (word & kErrIterations) return fail(LUCENT_ERR_DEVICE, "traversal exceeded node_count steps (malformed BVH)");
    if (word & kErrStack)
      return fail(LUCENT_ERR_DEVICE, "traversal needed more than 64 stack entries (BVH too deep for the reference)");
    return fail(LUCENT_ERR_DEVICE, "device error word 0x%x", word);
  }
  return LUCENT_OK;
}

lucent_status lucent_bvh_intersect(lucent_bvh* b, const float* rays, uint32_t n, double t_min, double t_max,
                                   int32_t* prim_out, float* t_out, float* u_out, float* v_out, void* stream) {
  clear_error();
  if (!b || (n && (!rays || !prim_out))) return fail(LUCENT_ERR_INVALID, "null argument");
  if (n == 0) return LUCENT_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t rb = (size_t)n * 24, ob = (size_t)n * 4;
  lucent_status st = b->stage.reserve(rb + 4 * ob + 64);
  if (st) return st;
  char* base = (char*)b->stage.ptr;
  float* rays_d = (float*)base;
  int32_t* prim_d = (int32_t*)(base + rb);
  float* t_d = (float*)(base + rb + ob);
  float* u_d = (float*)(base + rb + 2 * ob);
  float* v_d = (float*)(base + rb + 3 * ob);
  cudaError_t e = cudaMemcpyAsync(rays_d, rays, rb, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "upload rays");
  if ((st = lucent_bvh_intersect_device(b, rays_d, n, t_min, t_max, prim_d, t_d, u_d, v_d, stream))) return st;
  e = cudaMemcpyAsync(prim_out, prim_d, ob, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && t_out) e = cudaMemcpyAsync(t_out, t_d, ob, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && u_out) e = cudaMemcpyAsync(u_out, u_d, ob, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && v_out) e = cudaMemcpyAsync(v_out, v_d, ob, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return cuda_fail(e, "download hits");
  if (b->tri_count == 0 && t_out)
    for (uint32_t i = 0; i < n; i++) t_out[i] = INFINITY;
  return lucent_bvh_check(b, stream);
}

lucent_status lucent_bvh_intersect_f64(lucent_bvh* b, const double* rays, uint32_t n, double t_min, double t_max,
                                       int32_t* prim_out, double* t_out, double* u_out, double* v_out,
                                       void* stream) {
  clear_error();
  if (!b || (n && (!rays || !prim_out || !t_out || !u_out || !v_out))) return fail(LUCENT_ERR_INVALID, "null argument");
  lucent_status st = check_tmin(t_min, t_max);
  if (st) return st;
  if (n == 0) return LUCENT_OK;
  if (b->tri_count == 0) {
    for (uint32_t i = 0; i < n; i++) {
      prim_out[i] = -1;
      t_out[i] = INFINITY;
      u_out[i] = v_out[i] = 0;
    }
    return LUCENT_OK;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const size_t rb = (size_t)n * 48, ob = (size_t)n * 8;
  if ((st = b->stage.reserve(rb + 4 * ob + 64))) return st;
  unsigned *err;
  uint32_t *qlen, *queue;
  if ((st = prepare_scratch(b, 0, s, &err, &qlen, &queue))) return st;
  char* base = (char*)b->stage.ptr;
  double* rays_d = (double*)base;
  int32_t* prim_d = (int32_t*)(base + rb);
  double* t_d = (double*)(base + rb + ob);
  double* u_d = (double*)(base + rb + 2 * ob);
  double* v_d = (double*)(base + rb + 3 * ob);
  cudaError_t e = cudaMemcpyAsync(rays_d, rays, rb, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "upload rays");
  launch_closest_d((const Node*)b->nodes.ptr, b->node_count, (const float4*)b->tris.ptr, rays_d, n, t_min, t_max, prim_d, t_d, u_d,
                   v_d, err, s);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(prim_out, prim_d, (size_t)n * 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(t_out, t_d, ob, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(u_out, u_d, ob, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(v_out, v_d, ob, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return cuda_fail(e, "f64 closest-hit");
  return lucent_bvh_check(b, stream);
}

}  // extern "C"
