/*
 * Drop-in amcl3d::ParticleFilter over the GB300 library.  Like the reference it
 * throws nothing across its API: a failing device call is logged with ROS_ERROR
 * and leaves the previous state (and mean) in place.
 */
#include "ParticleFilter.h"

#include <cmath>
#include <random>

namespace amcl3d
{
ParticleFilter::ParticleFilter() : ParticleFilter(static_cast<uint64_t>(std::random_device{}()))
{
}

ParticleFilter::ParticleFilter(uint64_t seed)
{
  check(amcl_pf_create(&pf_, seed, nullptr), "amcl_pf_create");
}

ParticleFilter::~ParticleFilter()
{
  amcl_pf_destroy(pf_);
}

void ParticleFilter::check(int status, const char* what) const
{
  if (status != AMCL_OK)
    ROS_ERROR("[%s] %s: %s: %s", ros::this_node::getName().data(), what, amcl_status_string(status),
              amcl_last_error());
}

Particle ParticleFilter::getMean() const
{
  Particle m;
  float m7[7];
  const int rc = amcl_pf_get_mean(pf_, m7, nullptr);
  check(rc, "amcl_pf_get_mean");
  if (rc == AMCL_OK)
  {
    m.x = m7[0];
    m.y = m7[1];
    m.z = m7[2];
    m.a = m7[3];
  }
  return m;
}

std::vector<Particle> ParticleFilter::particles() const
{
  uint32_t n = 0;
  amcl_pf_size(pf_, &n);
  std::vector<Particle> p(n);
  if (n)
    check(amcl_pf_get_particles(pf_, &p[0].x, n), "amcl_pf_get_particles");
  return p;
}

void ParticleFilter::buildParticlesPoseMsg(geometry_msgs::PoseArray& msg) const
{
  /* ParticleFilter.cpp:30-44 */
  const std::vector<Particle> p = particles();
  msg.poses.resize(p.size());
  for (uint32_t i = 0; i < p.size(); ++i)
  {
    msg.poses[i].position.x = static_cast<double>(p[i].x);
    msg.poses[i].position.y = static_cast<double>(p[i].y);
    msg.poses[i].position.z = static_cast<double>(p[i].z);
    msg.poses[i].orientation.x = 0.;
    msg.poses[i].orientation.y = 0.;
    msg.poses[i].orientation.z = std::sin(static_cast<double>(p[i].a * 0.5f));
    msg.poses[i].orientation.w = std::cos(static_cast<double>(p[i].a * 0.5f));
  }
}

void ParticleFilter::init(const int num_particles, const float x_init, const float y_init, const float z_init,
                          const float a_init, const float x_dev, const float y_dev, const float z_dev,
                          const float a_dev)
{
  const int rc = amcl_pf_init(pf_, num_particles, x_init, y_init, z_init, a_init, x_dev, y_dev, z_dev, a_dev);
  check(rc, "amcl_pf_init");
  if (rc == AMCL_OK)
    initialized_ = true;
}

void ParticleFilter::predict(const double odom_x_mod, const double odom_y_mod, const double odom_z_mod,
                             const double odom_a_mod, const double delta_x, const double delta_y,
                             const double delta_z, const double delta_a)
{
  check(amcl_pf_predict(pf_, odom_x_mod, odom_y_mod, odom_z_mod, odom_a_mod, delta_x, delta_y, delta_z, delta_a),
        "amcl_pf_predict");
}

void ParticleFilter::update(const Grid3d& grid3d, const pcl::PointCloud<pcl::PointXYZ>::Ptr& cloud,
                            const std::vector<Range>& range_data, const double alpha, const double sigma,
                            const double roll, const double pitch)
{
  const float* xyz = (cloud && !cloud->empty()) ? &cloud->points[0].x : nullptr;
  const uint32_t n = cloud ? static_cast<uint32_t>(cloud->size()) : 0;
  const float* r4 = range_data.empty() ? nullptr : &range_data[0].r;
  check(amcl_pf_update(pf_, grid3d.handle(), xyz, n, sizeof(pcl::PointXYZ) / sizeof(float), r4,
                       static_cast<uint32_t>(range_data.size()), alpha, sigma, roll, pitch),
        "amcl_pf_update");
}

void ParticleFilter::update(const std::vector<Range>& range_data, const double alpha, const double sigma)
{
  const float* r4 = range_data.empty() ? nullptr : &range_data[0].r;
  check(amcl_pf_update_ranges(pf_, r4, static_cast<uint32_t>(range_data.size()), alpha, sigma),
        "amcl_pf_update_ranges");
}

void ParticleFilter::resample()
{
  check(amcl_pf_resample(pf_), "amcl_pf_resample");
}

}  // namespace amcl3d
