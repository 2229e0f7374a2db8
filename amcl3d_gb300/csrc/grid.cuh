// Host-side grid handle shared by the grid, weighting and filter translation units.
#pragma once
#include "common.cuh"
#include "locate.cuh"

struct amcl_grid_s
{
  amcl::StreamHolder st;
  amcl_grid_info info{};
  bool built = false;
  bool l2_window = false;
  amcl::DevBuf dist;    // float per cell (the reference's Grid3dCell::dist)
  amcl::DevBuf prob;    // float per cell (Grid3dCell::prob)
  amcl::DevBuf prob16;  // __half copy
  amcl::DevBuf prob8;   // uint8 copy
  amcl::DevBuf tabs;    // locate tables: float2 pairs (T[k], T[k+1]) per axis
  std::vector<float> tabs_host;
  amcl::GridView view{};
  uint64_t cells() const
  {
    return static_cast<uint64_t>(info.size[0]) * info.size[1] * info.size[2];
  }
};

namespace amcl
{
// Fills the host tables and the view's scalar fields from grid->info.
int grid_prepare_view(amcl_grid_s* g);
// Applies the grid's L2 persisting window (if enabled) to a stream.
void grid_apply_l2_window(amcl_grid_s* g, cudaStream_t s);
size_t grid_table_floats(const amcl_grid_s* g);

// Launches the per-particle cloud weighting on `s` (see weight.cu).
struct WeightArgs
{
  const float4* pose;  // x, y, z, yaw
  uint32_t P;
  const float4* cloud;  // x, y, z, unused (PCL's PointXYZ layout)
  uint32_t N;
  float sr, cr, sp, cp;
  const float4* ranges;  // (r, ax, ay, az)
  uint32_t nr;
  float k1, k2;
  float* wp;
  float* wr;
  uint8_t* inmap;
  unsigned long long* acc_wp;  // 10 digits, exact sum of wp over in-map particles (may be null)
  unsigned long long* acc_wr;
  int* err;
  int cloud_sum;  // 0 float running sum, 1 Neumaier
  int kernel;     // 1 thread-per-particle, 2 two-phase
  int ignore_map; // weigh every particle (computeCloudWeight itself has no map test)
  int yaw_only;   // set by launch_cloud_weight when roll = pitch = 0
  float* scratch;           // two-phase only: ceil(P/32)*32*N floats
  uint64_t scratch_floats;  // capacity
  int wait_probe;           // two-phase only: make one bounded wait give up (AMCL_OPT_WAIT_PROBE)
};
int launch_cloud_weight(amcl_grid_s* g, const WeightArgs& a, cudaStream_t s);
// Chooses the kernel for AMCL_OPT_WEIGHT_KERNEL = 0.
int choose_weight_kernel(uint32_t P, uint32_t N);
uint64_t two_phase_scratch_floats(uint32_t P, uint32_t N);
// Packs host points (stride floats apart) as float4 (x, y, z, 0).
void pack_cloud(const float* xyz, uint32_t n, uint32_t stride, float4* out);
}  // namespace amcl
