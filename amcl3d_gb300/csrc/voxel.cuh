// Scan voxel downsample on the device: pcl::VoxelGrid<pcl::PointXYZ> as the ROS node
// runs it on every accepted scan before the filter update (Node.cpp:130-137).
#pragma once

#include <mutex>

#include "common.cuh"

struct amcl_voxel_s
{
  amcl::StreamHolder st;
  amcl::DevBuf keys[2], vals[2], hist, tiles, starts, meta, in, out;
  amcl::PinnedBuf h_in, h_out, h_meta;
  std::mutex mu;
};

namespace amcl
{
// Device-side summary of one filter call (written by the kernels, read back once).
struct VoxelMeta
{
  uint32_t mm[6];     // order-preserving encodings of min.xyz, max.xyz over the finite points
  uint32_t n_finite;  // finite points
  uint32_t overflow;  // 1: the voxel count overflowed int32, the input is returned unchanged
  uint32_t n_out;     // output points
  uint32_t pad[7];
};

// Enqueues the whole filter on `s`: n float4 points in `in` (device) -> the centroids in
// `out` (device, room for n points).  The output count lands in the handle's VoxelMeta;
// voxel_read_count synchronises `s` and returns it.
int voxel_enqueue(amcl_voxel_s* v, const float4* in, uint32_t n, const float leaf[3], float4* out, cudaStream_t s);
int voxel_read_count(amcl_voxel_s* v, cudaStream_t s, uint32_t* n_out);
// AMCL_EINVAL unless every leaf size is positive and finite with a finite inverse.
int voxel_check_leaf(const float leaf[3], const char* fn);
}  // namespace amcl
