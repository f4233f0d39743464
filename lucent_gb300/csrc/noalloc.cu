// Closest hit for callers that cannot allocate device memory.
//
// Some hosts forbid the library from calling cudaMalloc: a process whose own
// allocator has reserved the device's memory up front, a real-time loop that
// must not take the allocator's implicit synchronisation, or a plugin whose
// host owns every allocation. This entry point runs the same kernels as
// lucent_bvh_intersect_device, but the scratch those kernels need (error
// word, ray counter, slow-path queue) lives in one file-scope __device__
// array that the module carries, so nothing is allocated per call.
#include <mutex>

#include "../../include/lucent.h"
#include "api_util.h"
#include "internal.h"

namespace lucent {

constexpr uint32_t kNoAllocMaxRays = 1u << 20;  // rays per call
constexpr size_t kNoAllocHeader = 256;          // error word, queue length, ray counter

// Every GPU that loads this library keeps this array (4 MiB + 256 B) until the
// process exits. All calls share it.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocHeader + 4 * (size_t)kNoAllocMaxRays];

// Host code cannot use the array's name as a device address; the address is
// fetched once per device, with that device current.
static std::mutex g_noalloc_mu;
static void* g_noalloc_ptr[128];

static lucent_status noalloc_scratch(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= 128) return fail(LUCENT_ERR_UNSUPPORTED, "device ordinal %d", dev);
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-allocation scratch)");
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return LUCENT_OK;
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
  if (!(t_min >= 0) || t_max != t_max) return fail(LUCENT_ERR_INVALID, "t_min must be >= 0 and t_max not NaN");
  cudaStream_t s = (cudaStream_t)stream;
  if (tri_count == 0) {  // bvh.ts:274: an empty BVH never hits
    cudaError_t e = cudaMemsetAsync(prim_d, 0xff, (size_t)n * 4, s);
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
  uint32_t* queue = (uint32_t*)(b + kNoAllocHeader);
  // The array keeps the previous call's contents: the counters must start at zero.
  cudaError_t e = cudaMemsetAsync(b, 0, 12, s);
  if (e != cudaSuccess) return cuda_fail(e, "clear no-allocation scratch");
  launch_closest((const Node*)nodes_d, node_count, (const float4*)tris_d, rays_d, n, t_min, t_max, prim_d, t_d, u_d,
                 v_d, queue, qlen, work, err, false, true, s);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  unsigned word = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&word, err, sizeof word, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "no-allocation closest hit");
  if (word & kErrIterations) return fail(LUCENT_ERR_DEVICE, "traversal exceeded node_count steps (malformed BVH)");
  if (word & kErrStack) return fail(LUCENT_ERR_DEVICE, "traversal needed more than 64 stack entries");
  if (word) return fail(LUCENT_ERR_DEVICE, "device error word 0x%x", word);
  return LUCENT_OK;
}
