// Host-side helpers shared by the C ABI translation units.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#include "../../include/lucent.h"

namespace lucent {

lucent_status fail(lucent_status code, const char* fmt, ...);
lucent_status cuda_fail(cudaError_t e, const char* what);
void clear_error();

// A growable device allocation owned by a handle.
struct DeviceBuffer {
  void* ptr = nullptr;
  size_t cap = 0;
  lucent_status reserve(size_t bytes);
  void release();
};

}  // namespace lucent

extern "C" {
// Reference-layout BVH checks shared by the C-ABI files (defined in api.cu).
uint32_t tree_depth(const float* nodes, uint32_t node_count, uint32_t tri_count);
lucent_status validate_bvh(const float* nodes, uint32_t node_count, const uint32_t* tri, uint32_t tri_count);
}
