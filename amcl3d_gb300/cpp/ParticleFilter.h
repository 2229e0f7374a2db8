/*
 * Drop-in amcl3d::ParticleFilter backed by the GB300 library (include/amcl3d_gpu.h).
 *
 * Same public interface as amcl3d/src/ParticleFilter.h:35-172 (Particle, Range,
 * init / predict / update / resample / getMean / isInitialized /
 * buildParticlesPoseMsg), so amcl3d::Node compiles against it unchanged.  The
 * particles stay on the GPU; getMean and buildParticlesPoseMsg read back only what
 * they return.  Adds buildParticlesPool (= init) and defines the range-only update
 * the reference declares (ParticleFilter.h:157) but never implements.
 */
#pragma once

#include "Grid3d.h"

#include <geometry_msgs/Point32.h>
#include <geometry_msgs/PoseArray.h>
#include <geometry_msgs/PoseWithCovarianceStamped.h>
#include <ros/ros.h>

#include <cstdint>
#include <vector>

namespace amcl3d
{
struct Particle
{
  float x; /*!< Position x */
  float y; /*!< Position y */
  float z; /*!< Position z */
  float a; /*!< Yaw angle */

  float w;  /*!< Total weight */
  float wp; /*!< Weight by the 3d point cloud sensor */
  float wr; /*!< Weight by the radio-range sensor*/

  Particle() : x(0), y(0), z(0), a(0), w(0), wp(0), wr(0)
  {
  }
};

struct Range
{
  float r;  /*!< Range measurement */
  float ax; /*!< Position x of the sensor in the environment */
  float ay; /*!< Position y of the sensor in the environment */
  float az; /*!< Position z of the sensor in the environment */

  Range(const float r_, const float ax_, const float ay_, const float az_) : r(r_), ax(ax_), ay(ay_), az(az_)
  {
  }
};

class ParticleFilter
{
public:
  /* seed: the counter-based generator's key (the reference seeds mt19937 from
   * std::random_device; the default here does the same). */
  explicit ParticleFilter();
  explicit ParticleFilter(uint64_t seed);
  virtual ~ParticleFilter();

  bool isInitialized() const
  {
    return initialized_;
  }

  Particle getMean() const;

  void buildParticlesPoseMsg(geometry_msgs::PoseArray& msg) const;

  void init(const int num_particles, const float x_init, const float y_init, const float z_init, const float a_init,
            const float x_dev, const float y_dev, const float z_dev, const float a_dev);
  void buildParticlesPool(const int num_particles, const float x_init, const float y_init, const float z_init,
                          const float a_init, const float x_dev, const float y_dev, const float z_dev,
                          const float a_dev)
  {
    init(num_particles, x_init, y_init, z_init, a_init, x_dev, y_dev, z_dev, a_dev);
  }

  void predict(const double odom_x_mod, const double odom_y_mod, const double odom_z_mod, const double odom_a_mod,
               const double delta_x, const double delta_y, const double delta_z, const double delta_a);

  void update(const Grid3d& grid3d, const pcl::PointCloud<pcl::PointXYZ>::Ptr& cloud,
              const std::vector<Range>& range_data, const double alpha, const double sigma, const double roll,
              const double pitch);
  void update(const std::vector<Range>& range_data, const double alpha, const double sigma);

  void resample();

  /* The particle set (x, y, z, a, w, wp, wr), read back from the device. */
  std::vector<Particle> particles() const;
  amcl_pf_t handle() const
  {
    return pf_;
  }

private:
  void check(int status, const char* what) const;

  bool initialized_{ false };
  amcl_pf_t pf_{ nullptr };
};

}  // namespace amcl3d
