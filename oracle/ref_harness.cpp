// Test infrastructure: extern "C" driver around the UNMODIFIED amcl3d filter core
// (ParticleFilter.cpp, Grid3d.cpp, PointCloudTools.cpp compiled from the reference
// tree against the stand-in headers in tests/stand_in/).  Only the test suite, the smoke
// check and the CPU-baseline leg of the benchmark load the resulting library.
//
// Private members are reached by the test-only `#define private public` below:
// the harness needs to inject particles (ParticleFilter::p_), seed the generator
// (ParticleFilter::generator_) and read the grid cells (Grid3d::grid_info_).
#include <algorithm>
#include <chrono>
#include <cstring>
#include <thread>
#include <vector>

#define private public
#include "ParticleFilter.h"
#undef private

using namespace amcl3d;

typedef pcl::PointCloud<pcl::PointXYZ> Cloud;

extern "C" {

/* ---- Grid3d ---------------------------------------------------------------- */

void* ref_grid_new(void) { return new Grid3d(); }
void ref_grid_free(void* g) { delete static_cast<Grid3d*>(g); }

/* Grid3d::open (Grid3d.cpp:25-78): map file -> point cloud -> (.grid cache | computeGrid). */
int ref_grid_open(void* g, const char* map_path, double sensor_dev)
{
  return static_cast<Grid3d*>(g)->open(map_path, sensor_dev) ? 1 : 0;
}

int ref_grid_info(void* g, uint32_t size[3], double mn[3], double mx[3], double* res)
{
  Grid3d* G = static_cast<Grid3d*>(g);
  if (!G->grid_info_ || !G->pc_info_)
    return 0;
  size[0] = G->grid_info_->size_x;
  size[1] = G->grid_info_->size_y;
  size[2] = G->grid_info_->size_z;
  mn[0] = G->pc_info_->octo_min_x;
  mn[1] = G->pc_info_->octo_min_y;
  mn[2] = G->pc_info_->octo_min_z;
  mx[0] = G->pc_info_->octo_max_x;
  mx[1] = G->pc_info_->octo_max_y;
  mx[2] = G->pc_info_->octo_max_z;
  *res = G->pc_info_->octo_resol;
  return 1;
}

/* Copies grid cells [first, first+count) as separate dist / prob arrays. */
int ref_grid_cells(void* g, uint64_t first, uint64_t count, float* dist, float* prob)
{
  Grid3d* G = static_cast<Grid3d*>(g);
  if (!G->grid_info_ || first + count > G->grid_info_->grid.size())
    return 0;
  for (uint64_t i = 0; i < count; ++i)
  {
    if (dist)
      dist[i] = G->grid_info_->grid[first + i].dist;
    if (prob)
      prob[i] = G->grid_info_->grid[first + i].prob;
  }
  return 1;
}

/* Grid3d::buildGridSliceMsg (Grid3d.cpp:80-121). */
int ref_grid_slice(void* g, double z, int8_t* out, uint64_t cap, uint64_t* len, uint32_t* width, uint32_t* height)
{
  nav_msgs::OccupancyGrid msg;
  if (!static_cast<Grid3d*>(g)->buildGridSliceMsg(z, msg))
    return 0;
  *len = msg.data.size();
  *width = msg.info.width;
  *height = msg.info.height;
  if (out)
    std::memcpy(out, msg.data.data(), std::min<uint64_t>(cap, msg.data.size()));
  return 1;
}

int ref_grid_is_into_map(void* g, float x, float y, float z)
{
  return static_cast<Grid3d*>(g)->isIntoMap(x, y, z) ? 1 : 0;
}

/* ---- point clouds ---------------------------------------------------------- */

void* ref_cloud_new(const float* xyz, uint64_t n, uint64_t stride_floats)
{
  Cloud::Ptr* c = new Cloud::Ptr(new Cloud());
  (*c)->points.reserve(n);
  for (uint64_t i = 0; i < n; ++i)
    (*c)->push_back(pcl::PointXYZ(xyz[i * stride_floats], xyz[i * stride_floats + 1], xyz[i * stride_floats + 2]));
  return c;
}
void ref_cloud_free(void* c) { delete static_cast<Cloud::Ptr*>(c); }

/* Grid3d::computeCloudWeight (Grid3d.cpp:133-199). */
float ref_cloud_weight(void* g, void* c, float tx, float ty, float tz, float roll, float pitch, float yaw)
{
  return static_cast<Grid3d*>(g)->computeCloudWeight(*static_cast<Cloud::Ptr*>(c), tx, ty, tz, roll, pitch, yaw);
}

/* ---- ParticleFilter -------------------------------------------------------- */

void* ref_pf_new(uint32_t seed)
{
  ParticleFilter* pf = new ParticleFilter();
  pf->generator_.seed(seed);
  return pf;
}
void ref_pf_free(void* pf) { delete static_cast<ParticleFilter*>(pf); }
void ref_pf_seed(void* pf, uint32_t seed) { static_cast<ParticleFilter*>(pf)->generator_.seed(seed); }

uint64_t ref_pf_size(void* pf) { return static_cast<ParticleFilter*>(pf)->p_.size(); }

/* Particles as 7 floats each (x, y, z, a, w, wp, wr), the layout of amcl3d::Particle. */
void ref_pf_set_particles(void* pf, const float* p7, uint64_t n)
{
  ParticleFilter* P = static_cast<ParticleFilter*>(pf);
  P->p_.resize(n);
  std::memcpy(P->p_.data(), p7, n * sizeof(Particle));
  P->initialized_ = true;
}
void ref_pf_get_particles(void* pf, float* p7)
{
  ParticleFilter* P = static_cast<ParticleFilter*>(pf);
  std::memcpy(p7, P->p_.data(), P->p_.size() * sizeof(Particle));
}
void ref_pf_get_mean(void* pf, float out7[7])
{
  Particle m = static_cast<ParticleFilter*>(pf)->getMean();
  std::memcpy(out7, &m, sizeof(Particle));
}

void ref_pf_init(void* pf, int n, float x, float y, float z, float a, float xd, float yd, float zd, float ad)
{
  static_cast<ParticleFilter*>(pf)->init(n, x, y, z, a, xd, yd, zd, ad);
}

void ref_pf_predict(void* pf, double xm, double ym, double zm, double am, double dx, double dy, double dz, double da)
{
  static_cast<ParticleFilter*>(pf)->predict(xm, ym, zm, am, dx, dy, dz, da);
}

static std::vector<Range> make_ranges(const float* r4, uint64_t nr)
{
  std::vector<Range> rd;
  for (uint64_t i = 0; i < nr; ++i)
    rd.push_back(Range(r4[4 * i], r4[4 * i + 1], r4[4 * i + 2], r4[4 * i + 3]));
  return rd;
}

/* ParticleFilter::update (ParticleFilter.cpp:121-196); ranges are (r, ax, ay, az). */
void ref_pf_update(void* pf, void* g, void* c, const float* r4, uint64_t nr, double alpha, double sigma, double roll,
                   double pitch)
{
  static_cast<ParticleFilter*>(pf)->update(*static_cast<Grid3d*>(g), *static_cast<Cloud::Ptr*>(c),
                                           make_ranges(r4, nr), alpha, sigma, roll, pitch);
}

/* The uniform draw resample() will take next, without consuming it. */
float ref_pf_peek_uniform(void* pf)
{
  std::mt19937 copy = static_cast<ParticleFilter*>(pf)->generator_;
  std::uniform_real_distribution<float> d(0, 1);
  return d(copy);
}

/* ParticleFilter::resample (ParticleFilter.cpp:198-222).  The reference reads
 * p_[N] when the cumulative sum never reaches u; the harness pads p_ with one
 * zero particle while resampling so that read stays inside the allocation, and
 * reports through *overrun whether it happened. */
void ref_pf_resample(void* pf, int* overrun)
{
  ParticleFilter* P = static_cast<ParticleFilter*>(pf);
  const size_t n = P->p_.size();
  // Detect the overrun by replaying the reference's loop on a copy of the weights.
  std::mt19937 copy = P->generator_;
  std::uniform_real_distribution<float> d(0, 1);
  const float factor = 1.f / n;
  const float r = factor * d(copy);
  float cum = P->p_[0].w;
  int over = 0;
  for (uint32_t m = 0, i = 0; m < n; ++m)
  {
    const float u = r + factor * m;
    while (u > cum)
    {
      if (++i >= n)
        break;
      cum += P->p_[i].w;
    }
    if (i >= n)
      over = 1;
  }
  if (overrun)
    *overrun = over;
  // Every overrunning m reads one slot further (i keeps incrementing), so up to
  // n extra slots can be read: back them with zero particles.
  P->p_.reserve(2 * n);
  for (size_t k = n; k < 2 * n; ++k)
    P->p_.data()[k] = Particle();
  P->resample();
}

/* The computeRangeWeight restatement is private; expose it for per-particle checks. */
float ref_pf_range_weight(void* pf, float x, float y, float z, const float* r4, uint64_t nr, double sigma)
{
  return static_cast<ParticleFilter*>(pf)->computeRangeWeight(x, y, z, make_ranges(r4, nr), sigma);
}

/* ---- CPU baseline timing ----------------------------------------------------- */

/* Times ParticleFilter::update + resample on `nthreads` host threads.  The
 * reference is single-threaded, so each thread runs its own ParticleFilter over
 * an equal slice of the particles against the shared (read-only) Grid3d and
 * cloud.  Returns wall seconds for `reps` rounds; particles are restored before
 * every round so each round does the same work. */
double ref_time_update(void* g, void* c, const float* p7, uint64_t n, const float* r4, uint64_t nr, double alpha,
                       double sigma, double roll, double pitch, int nthreads, int reps, int do_resample)
{
  if (nthreads < 1)
    nthreads = 1;
  std::vector<ParticleFilter*> pfs(nthreads);
  std::vector<std::vector<Particle> > slices(nthreads);
  for (int t = 0; t < nthreads; ++t)
  {
    const uint64_t b = n * t / nthreads, e = n * (t + 1) / nthreads;
    slices[t].assign(reinterpret_cast<const Particle*>(p7) + b, reinterpret_cast<const Particle*>(p7) + e);
    pfs[t] = new ParticleFilter();
    pfs[t]->generator_.seed(1234u + t);
  }
  const std::vector<Range> rd = make_ranges(r4, nr);
  Grid3d& G = *static_cast<Grid3d*>(g);
  const Cloud::Ptr& C = *static_cast<Cloud::Ptr*>(c);
  double total = 0;
  for (int rep = 0; rep < reps; ++rep)
  {
    for (int t = 0; t < nthreads; ++t)
    {
      pfs[t]->p_ = slices[t];
      pfs[t]->p_.reserve(2 * pfs[t]->p_.size());
    }
    auto t0 = std::chrono::steady_clock::now();
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; ++t)
      th.emplace_back([&, t]() {
        if (pfs[t]->p_.empty())
          return;
        pfs[t]->update(G, C, rd, alpha, sigma, roll, pitch);
        if (do_resample)
        {
          const size_t m = pfs[t]->p_.size();
          for (size_t k = m; k < 2 * m; ++k)
            pfs[t]->p_.data()[k] = Particle();
          pfs[t]->resample();
        }
      });
    for (auto& x : th)
      x.join();
    total += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
  for (auto p : pfs)
    delete p;
  return total;
}

}  // extern "C"
