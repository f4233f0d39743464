// Internal launcher declarations shared between the kernel files and the C ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "../../include/lucent.h"
#include "common.cuh"

namespace lucent {

int grid_for(uint32_t n, int block);
int persistent_blocks(const void* kernel, int block);
void launch_pack_nodes(const float* ref_d, uint32_t count, Node* out_d, cudaStream_t s);
void launch_gather_tris(const float* pos_d, const uint32_t* idx_d, uint32_t tri_count, float4* out_d,
                        cudaStream_t s);
void launch_unpack(const Node* nodes, uint32_t count, const float4* tris, uint32_t tri_count, float* ref_d,
                   uint32_t* idx_d, cudaStream_t s);
void launch_closest(const Node* nodes, uint32_t node_count, const float4* tris, const float* rays_d, uint32_t n, double tMin,
                    double tMax, int32_t* prim, float* t, float* u, float* v, uint32_t* queue, uint32_t* queue_len,
                    uint32_t* work, unsigned* err, bool exact_only, bool top_levels, cudaStream_t s,
                    const Node* wide = nullptr);
// Four-wide view of a binary node array (traverse_wide.cuh): 4 records per node.
void launch_wide_view(const Node* nodes, uint32_t node_count, Node* wide, cudaStream_t s);
void launch_closest_d(const Node* nodes, uint32_t node_count, const float4* tris, const double* rays_d, uint32_t n, double tMin,
                      double tMax, int32_t* prim, double* t, double* u, double* v, unsigned* err, cudaStream_t s);

struct DeviceBuffer;
// Texture arrays (texture.cu): decode tables (512: sRGB byte -> linear, then
// byte / 255) and sRGB code-value midpoints (255), the shared layer size
// (renderer.ts:316-322), and the resampling of each referenced image into its
// layer of a size x size RGBA8 array.
void texel_tables(float lut[512], float mid[255]);
int texture_array_size(const uint32_t* w, const uint32_t* h, const int32_t* layers, uint32_t n_layers);
lucent_status build_texture_layers(const uint8_t* const* images, const uint32_t* w, const uint32_t* h,
                                   const int32_t* layers, uint32_t n_layers, int size, bool srgb, const float* lut_d,
                                   const float* mid_d, uint8_t* out_d, cudaStream_t s);
// buildEnvSampler on the GPU (env_sampler.cu): the sampler grid of a w x h
// map, and the table (gw * gh float4) built from a device RGB map.
void env_grid(uint32_t w, uint32_t h, uint32_t max_w, uint32_t& gw, uint32_t& gh);
lucent_status gpu_env_sampler(const float* rgb_d, uint32_t w, uint32_t h, uint32_t max_w, uint32_t& gw, uint32_t& gh,
                              float4* table_d, double& total, cudaStream_t s);
lucent_status gpu_build_bvh(const float* pos_d, uint32_t n, int max_leaf, int bins, cudaStream_t s,
                            std::vector<float>& nodes_ref, std::vector<uint32_t>& tri_out, double bounds[6],
                            DeviceBuffer* nodes_dev, DeviceBuffer* tris_dev);

}  // namespace lucent
