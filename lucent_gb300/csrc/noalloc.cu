// Closest hit for callers that cannot allocate device memory.
//
// Some hosts forbid the library from calling cudaMalloc: a process whose own
// allocator has reserved the device's memory up front, a real-time loop that
// must not take the allocator's implicit synchronisation, or a plugin whose
// host owns every allocation. This entry point runs the same kernels as
// lucent_bvh_intersect_device, but the scratch those kernels need (error
// word, ray counter, slow-path queue) lives in one file-scope __device__
// array that the module carries, so nothing is allocated per call.
//
// The caller's tree is not trusted: a check kernel walks every node and
// triangle record first (children inside the node array and after their
// parent, leaf ranges inside the triangle array, finite bounds, source
// indices in range), and no traversal kernel is launched unless it passes.
// With those facts every node and triangle read of the traversal stays inside
// the caller's buffers, and the traversal's iteration cap and stack check end
// any remaining malformation as a device error.
#include "../../include/lucent.h"
#include "api_util.h"
#include "internal.h"

namespace lucent {

constexpr uint32_t kNoAllocMaxRays = 1u << 20;  // rays per call
constexpr size_t kNoAllocHeader = 256;          // error word, queue length, ray counter, first bad record

// Every GPU that loads this library keeps this array (4 MiB + 256 B) until the
// process exits. All calls share it.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocHeader + 4 * (size_t)kNoAllocMaxRays];

// Host code cannot use the array's name as a device address. The address is
// looked up on every call with the calling device current, so a module that
// was reloaded (a new primary context after cudaDeviceReset) is never served
// a stale address.
static lucent_status noalloc_scratch(void** out) {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-allocation scratch)");
  *out = p;
  return LUCENT_OK;
}

// Device-side form of validate_bvh (api.cu) over the device layouts: records
// the lowest offending record (node i, or node_count + slot for a triangle)
// in *bad and sets kErrTree.
__global__ void k_check_tree(const Node* __restrict__ nodes, uint32_t node_count, const float4* __restrict__ tris,
                             uint32_t tri_count, unsigned* __restrict__ err, uint32_t* __restrict__ bad) {
  const uint32_t m = node_count > tri_count ? node_count : tri_count;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    if (i < node_count) {
      const Node nd = nodes[i];
      const int first = node_first(nd), cnt = lucent::node_count(nd);
      bool ok = first >= 0 && cnt >= 0 && isfinite(nd.lo.x) && isfinite(nd.lo.y) && isfinite(nd.lo.z) &&
                isfinite(nd.hi.x) && isfinite(nd.hi.y) && isfinite(nd.hi.z);
      if (ok && cnt > 0) ok = (uint64_t)first + (uint64_t)cnt <= tri_count;
      else if (ok) ok = (uint32_t)first > i && (uint64_t)first + 1 < node_count;
      if (!ok) {
        atomicOr(err, kErrTree);
        atomicMin(bad, i);
      }
    }
    if (i < tri_count) {
      const int src = __float_as_int(tris[3 * (size_t)i].w);
      if (src < 0 || (uint32_t)src >= tri_count) {
        atomicOr(err, kErrTree);
        atomicMin(bad, node_count + i);
      }
    }
  }
}

// Outputs of an empty tree: every ray misses (bvh.ts:274), t = +inf, u = v = 0.
__global__ void k_fill_miss(uint32_t n, int32_t* prim, float* t, float* u, float* v) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    prim[i] = -1;
    if (t) t[i] = __int_as_float(0x7f800000);
    if (u) u[i] = 0.f;
    if (v) v[i] = 0.f;
  }
}

}  // namespace lucent

using namespace lucent;

extern "C" lucent_status lucent_bvh_intersect_noalloc(const float* nodes_d, uint32_t node_count, const float* tris_d,
                                                      uint32_t tri_count, const float* rays_d, uint32_t n,
                                                      double t_min, double t_max, int32_t* prim_d, float* t_d,
                                                      float* u_d, float* v_d, void* stream) {
  clear_error();
  if (n == 0) return LUCENT_OK;
  if (!nodes_d || !rays_d || !prim_d || node_count == 0 || (tri_count && !tris_d))
    return fail(LUCENT_ERR_INVALID, "null argument");
  if (n > kNoAllocMaxRays)
    return fail(LUCENT_ERR_UNSUPPORTED, "%u rays in one call; the no-allocation limit is %u", n, kNoAllocMaxRays);
  if (tri_count > (1u << 23)) return fail(LUCENT_ERR_UNSUPPORTED, "%u triangles; the limit is 2^23", tri_count);
  if (!(t_min >= 0) || t_max != t_max) return fail(LUCENT_ERR_INVALID, "t_min must be >= 0 and t_max not NaN");
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e;
  if (tri_count == 0) {
    k_fill_miss<<<grid_for(n, 256), 256, 0, s>>>(n, prim_d, t_d, u_d, v_d);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return e == cudaSuccess ? LUCENT_OK : cuda_fail(e, "no-allocation miss fill");
  }
  void* base = nullptr;
  lucent_status st = noalloc_scratch(&base);
  if (st) return st;
  char* b = (char*)base;
  unsigned* err = (unsigned*)b;
  uint32_t* qlen = (uint32_t*)(b + 4);
  uint32_t* work = (uint32_t*)(b + 8);
  uint32_t* bad = (uint32_t*)(b + 12);
  uint32_t* queue = (uint32_t*)(b + kNoAllocHeader);
  // The array keeps the previous call's contents: the counters must start at
  // zero and the first-bad-record slot at its maximum.
  e = cudaMemsetAsync(b, 0, 12, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(bad, 0xff, 4, s);
  if (e != cudaSuccess) return cuda_fail(e, "clear no-allocation scratch");
  const uint32_t m = node_count > tri_count ? node_count : tri_count;
  k_check_tree<<<grid_for(m, 256), 256, 0, s>>>((const Node*)nodes_d, node_count, (const float4*)tris_d, tri_count,
                                                err, bad);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  unsigned word[4] = {0, 0, 0, 0};
  if (e == cudaSuccess) e = cudaMemcpy(word, b, sizeof word, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "no-allocation tree check");
  if (word[0] & kErrTree) {
    if (word[3] < node_count) return fail(LUCENT_ERR_INVALID, "malformed BVH: node %u", word[3]);
    return fail(LUCENT_ERR_INVALID, "malformed BVH: triangle slot %u has a source index out of range",
                word[3] - node_count);
  }
  launch_closest((const Node*)nodes_d, node_count, (const float4*)tris_d, rays_d, n, t_min, t_max, prim_d, t_d, u_d,
                 v_d, queue, qlen, work, err, false, true, s);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = cudaMemcpy(word, err, sizeof word[0], cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "no-allocation closest hit");
  if (word[0] & kErrIterations) return fail(LUCENT_ERR_DEVICE, "traversal exceeded node_count steps (malformed BVH)");
  if (word[0] & kErrStack) return fail(LUCENT_ERR_DEVICE, "traversal needed more than 64 stack entries");
  if (word[0]) return fail(LUCENT_ERR_DEVICE, "device error word 0x%x", word[0]);
  return LUCENT_OK;
}
