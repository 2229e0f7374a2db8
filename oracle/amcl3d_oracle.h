/*
 * amcl3d_oracle.h - CPU restatement of amcl3d's particle-filter hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the GPU library is checked
 * against: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * may load it, and only as the checker.  It is never a fallback for the GPU path.
 *
 * Each function restates the reference's arithmetic in plain C (ISO C, no FMA
 * contraction), citing amcl3d/src file:line.  Two switches cover the two places
 * where this GPU build's arithmetic differs from the reference by design:
 *   yaw_trig  0: sinf/cosf of the yaw from libm (what the reference calls);
 *             1: sin/cos in double rounded to float (what the GPU computes).
 *   exp_mode  0: expf from libm (reference); 1: exp in double rounded to float (GPU).
 * Sums whose order differs by design (the GPU's exact normalisation sums) are
 * restated in the Python layer with math.fsum.
 */
#ifndef AMCL3D_ORACLE_H
#define AMCL3D_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct
{
  double min[3], max[3], res;
  uint32_t size[3];
  const float* prob; /* size[0]*size[1]*size[2] cells, reference linear order */
} orc_grid;

/* Grid3d::computeCloudWeight (Grid3d.cpp:133-199) for P poses (x, y, z, yaw) at a
 * shared roll/pitch.  cells (optional, P*n) receives each point's cell index or -1. */
void orc_cloud_weights(const orc_grid* g, const float* poses4, uint64_t P, const float* xyz, uint64_t n,
                       uint32_t stride, float roll, float pitch, int yaw_trig, float* out, int64_t* cells);

/* Grid3d::isIntoMap (Grid3d.cpp:201-208). */
int orc_is_into_map(const orc_grid* g, float x, float y, float z);

/* ParticleFilter::computeRangeWeight (ParticleFilter.cpp:224-244); r4 = (r, ax, ay, az). */
float orc_range_weight(float x, float y, float z, const float* r4, uint32_t nr, double sigma, int exp_mode);

/* ParticleFilter::update (ParticleFilter.cpp:121-196) with the reference's float
 * running sums; p7 = P particles of 7 floats, updated in place; mean4 = x, y, z, a. */
void orc_update_f32(float* p7, uint64_t P, const orc_grid* g, const float* xyz, uint64_t n, uint32_t stride,
                    const float* r4, uint32_t nr, double alpha, double sigma, double roll, double pitch,
                    int yaw_trig, int exp_mode, float mean4[4]);

/* ParticleFilter::resample (ParticleFilter.cpp:198-222) with the float running sum
 * and the uniform draw u01; idx[m] = source particle (the reference's overrun,
 * i == P, is reported as P).  Returns 1 if an overrun happened. */
int orc_resample_f32(const float* w, uint64_t P, float u01, int32_t* idx);

/* ParticleFilter::predict (ParticleFilter.cpp:97-119) given the normal draws
 * z (4 per particle, order x, y, z, a) in place of std::normal_distribution. */
void orc_predict(float* p7, uint64_t P, const float* z4, double xm, double ym, double zm, double am, double dx,
                 double dy, double dz, double da, int yaw_trig);

/* Pose part of ParticleFilter::init (ParticleFilter.cpp:58-77) given the draws
 * (particle 0 takes none); writes x, y, z, a and the unnormalised w. */
void orc_init_pose(float* p7, uint64_t P, const float* z4, float x, float y, float z, float a, float xd, float yd,
                   float zd, float ad, int exp_mode);

/* computeGrid (PointCloudTools.cpp:84-149) restricted to the cells
 * [lo, hi) per axis: exact nearest point (float squared distance accumulated as
 * ((0 + dx*dx) + dy*dy) + dz*dz), prob = c1 * expf(-d*d*c2).  dist/prob are the
 * sub-block in x-fastest order.  Runs on `threads` host threads. */
int orc_compute_grid(const float* xyz, uint64_t n, uint32_t stride, const double min[3], const double max[3],
                     double res, double sensor_dev, const uint32_t lo[3], const uint32_t hi[3], int exp_mode,
                     int threads, float* dist, float* prob);

/* pcl::VoxelGrid<PointXYZ>::filter (Node.cpp:130-137; PCL's published algorithm, the
 * points of a voxel summed in input order): out4 (n float4) receives the centroids in
 * voxel-key order, *n_out their count.  Returns 1 if the voxel count overflowed int32 and
 * the input was returned unchanged. */
int orc_voxel_downsample(const float* xyz, uint64_t n, uint32_t stride, const float leaf[3], float* out4,
                         uint64_t* n_out);

/* prob of computeGrid (PointCloudTools.cpp:133-137) for the m listed cells (linear
 * indices ix + iy*size[0] + iz*size[0]*size[1]) only.  A cell whose nearest point lies
 * beyond the distance where c1*expf(-d^2*d^2*c2) underflows to 0 gets 0 without an
 * exact search (the reference's value there is 0 too). */
int orc_grid_cell_probs(const float* xyz, uint64_t n, uint32_t stride, const double min[3], double res,
                        double sensor_dev, const uint32_t size[3], const uint64_t* cells, uint64_t m, int exp_mode,
                        int threads, float* prob);

/* Philox4x32-10 block (Salmon et al., SC'11). */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

#ifdef __cplusplus
}
#endif
#endif
