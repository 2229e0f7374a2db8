/*
 * amcl3d_oracle.c - CPU restatement of amcl3d's particle-filter hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see amcl3d_oracle.h): the checker for the GPU
 * library, never part of its data path.  Built as ISO C with FP contraction off,
 * so every a*b+c below rounds twice, exactly as the reference's C++ does.
 */
#define _GNU_SOURCE
#include "amcl3d_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

static void yaw_sincos(float yaw, int mode, float* s, float* c)
{
  if (mode == 0)
  {
    *s = sinf(yaw);
    *c = cosf(yaw);
  }
  else
  {
    *s = (float)sin((double)yaw);
    *c = (float)cos((double)yaw);
  }
}

static float exp_f(float x, int mode) { return mode == 0 ? expf(x) : (float)exp((double)x); }

/* Grid3d::computeCloudWeight, Grid3d.cpp:133-199. */
static float cloud_weight_one(const orc_grid* g, const float* xyz, uint64_t n, uint32_t stride, float tx, float ty,
                              float tz, float sr, float cr, float sp, float cp, float sy, float cy, int64_t* cells)
{
  /* Grid3d.cpp:146-149 (float products, left to right) */
  const float r00 = cy * cp, r01 = cy * sp * sr - sy * cr, r02 = cy * sp * cr + sy * sr;
  const float r10 = sy * cp, r11 = sy * sp * sr + cy * cr, r12 = sy * sp * cr - cy * sr;
  const float r20 = -sp, r21 = cp * sr, r22 = cp * cr;
  /* Grid3d.cpp:151-157 */
  const double sxd = g->max[0] - g->min[0], syd = g->max[1] - g->min[1], szd = g->max[2] - g->min[2];
  const double ox = tx - g->min[0], oy = ty - g->min[1], oz = tz - g->min[2];
  const uint32_t step_y = g->size[0], step_z = g->size[0] * g->size[1];
  const uint64_t grid_size = (uint64_t)g->size[0] * g->size[1] * g->size[2];
  const float error_z = 0;
  float weight = 0.;
  int nn = 0;
  for (uint64_t i = 0; i < n; ++i)
  {
    const float px = xyz[i * stride], py = xyz[i * stride + 1], pz = xyz[i * stride + 2];
    float nx, ny, nz;
    /* Grid3d.cpp:174-176: float sum of products, then + double offset, to float */
    nx = px * r00 + py * r01 + (pz + error_z) * r02 + ox;
    ny = px * r10 + py * r11 + (pz + error_z) * r12 + oy;
    nz = px * r20 + py * r21 + (pz + error_z) * r22 + oz;
    int64_t cell = -1;
    if (nx >= 0 && nx < sxd && ny >= 0 && ny < syd && nz >= 0 && nz < szd) /* Grid3d.cpp:178-179 */
    {
      const uint32_t ix = (uint32_t)floor(nx / g->res); /* Grid3d.cpp:181-183 */
      const uint32_t iy = (uint32_t)floor(ny / g->res);
      const uint32_t iz = (uint32_t)floor(nz / g->res);
      if (ix < g->size[0] && iy < g->size[1] && iz < g->size[2]) /* Grid3d.cpp:185 */
      {
        const uint32_t gi = ix + iy * step_y + iz * step_z; /* Grid3d.cpp:187 */
        if (gi < grid_size)
        {
          weight += g->prob[gi]; /* Grid3d.cpp:191 */
          nn += 1;
          cell = gi;
        }
      }
    }
    if (cells)
      cells[i] = cell;
  }
  return (nn <= 10) ? 0 : weight / nn; /* Grid3d.cpp:198 */
}

void orc_cloud_weights(const orc_grid* g, const float* poses4, uint64_t P, const float* xyz, uint64_t n,
                       uint32_t stride, float roll, float pitch, int yaw_trig, float* out, int64_t* cells)
{
  /* Grid3d.cpp:139-144 with the float overloads */
  const float sr = sinf(roll), cr = cosf(roll), sp = sinf(pitch), cp = cosf(pitch);
  for (uint64_t p = 0; p < P; ++p)
  {
    float sy, cy;
    yaw_sincos(poses4[4 * p + 3], yaw_trig, &sy, &cy);
    out[p] = cloud_weight_one(g, xyz, n, stride, poses4[4 * p], poses4[4 * p + 1], poses4[4 * p + 2], sr, cr, sp, cp,
                              sy, cy, cells ? cells + p * n : NULL);
  }
}

int orc_is_into_map(const orc_grid* g, float x, float y, float z)
{
  /* Grid3d.cpp:207 */
  return x >= g->min[0] && x < g->max[0] && y >= g->min[1] && y < g->max[1] && z >= g->min[2] && z < g->max[2];
}

float orc_range_weight(float x, float y, float z, const float* r4, uint32_t nr, double sigma, int exp_mode)
{
  if (nr == 0) /* ParticleFilter.cpp:227-228 */
    return 0;
  float w = 1;
  const float k1 = 1.f / (sigma * sqrt(2 * M_PI)); /* ParticleFilter.cpp:231 */
  const float k2 = 0.5f / (sigma * sigma);          /* ParticleFilter.cpp:232 */
  for (uint32_t i = 0; i < nr; ++i)
  {
    const float ax = r4[4 * i + 1], ay = r4[4 * i + 2], az = r4[4 * i + 3], rr = r4[4 * i];
    const float r = sqrtf((x - ax) * (x - ax) + (y - ay) * (y - ay) + (z - az) * (z - az)); /* :239 */
    w *= k1 * exp_f(-k2 * (r - rr) * (r - rr), exp_mode);                                   /* :240 */
  }
  return w;
}

void orc_update_f32(float* p7, uint64_t P, const orc_grid* g, const float* xyz, uint64_t n, uint32_t stride,
                    const float* r4, uint32_t nr, double alpha, double sigma, double roll, double pitch,
                    int yaw_trig, int exp_mode, float mean4[4])
{
  /* ParticleFilter.cpp:126-153 */
  float wtp = 0, wtr = 0;
  const float rollf = (float)roll, pitchf = (float)pitch;
  const float sr = sinf(rollf), cr = cosf(rollf), sp = sinf(pitchf), cp = cosf(pitchf);
  for (uint64_t i = 0; i < P; ++i)
  {
    float* q = p7 + 7 * i;
    const float tx = q[0], ty = q[1], tz = q[2];
    if (!orc_is_into_map(g, tx, ty, tz))
    {
      q[4] = 0;
      continue;
    }
    float sy, cy;
    yaw_sincos(q[3], yaw_trig, &sy, &cy);
    q[5] = cloud_weight_one(g, xyz, n, stride, tx, ty, tz, sr, cr, sp, cp, sy, cy, NULL);
    q[6] = orc_range_weight(tx, ty, tz, r4, nr, sigma, exp_mode);
    wtp += q[5];
    wtr += q[6];
  }
  /* ParticleFilter.cpp:159-180 */
  float wt = 0;
  for (uint64_t i = 0; i < P; ++i)
  {
    float* q = p7 + 7 * i;
    if (wtp > 0)
      q[5] /= wtp;
    else
      q[5] = 0;
    if (wtr > 0)
      q[6] /= wtr;
    else
      q[6] = 0;
    if (!orc_is_into_map(g, q[0], q[1], q[2]))
      q[4] = 0;
    else
      q[4] = q[5] * alpha + q[6] * (1 - alpha);
    wt += q[4];
  }
  /* ParticleFilter.cpp:182-195 */
  float mx = 0, my = 0, mz = 0, ma = 0;
  for (uint64_t i = 0; i < P; ++i)
  {
    float* q = p7 + 7 * i;
    if (wt > 0)
      q[4] /= wt;
    else
      q[4] = 0;
    mx += q[4] * q[0];
    my += q[4] * q[1];
    mz += q[4] * q[2];
    ma += q[4] * q[3];
  }
  mean4[0] = mx;
  mean4[1] = my;
  mean4[2] = mz;
  mean4[3] = ma;
}

int orc_resample_f32(const float* w, uint64_t P, float u01, int32_t* idx)
{
  /* ParticleFilter.cpp:198-222 */
  const float factor = 1.f / P;
  const float r = factor * u01;
  float c = w[0];
  float u;
  int over = 0;
  uint64_t i = 0;
  for (uint32_t m = 0; m < P; ++m)
  {
    u = r + factor * m;
    while (u > c)
    {
      if (++i >= P)
        break;
      c += w[i];
    }
    if (i >= P)
      over = 1;
    idx[m] = (int32_t)(i < P ? i : P);
  }
  return over;
}

void orc_predict(float* p7, uint64_t P, const float* z4, double xm, double ym, double zm, double am, double dx,
                 double dy, double dz, double da, int yaw_trig)
{
  /* ParticleFilter.cpp:101-104 */
  const double x_dev = fabs(dx * xm), y_dev = fabs(dy * ym), z_dev = fabs(dz * zm), a_dev = fabs(da * am);
  const float sxf = (float)x_dev, syf = (float)y_dev, szf = (float)z_dev, saf = (float)a_dev;
  for (uint64_t i = 0; i < P; ++i)
  {
    float* q = p7 + 7 * i;
    /* ranGaussian(0, dev): normal_distribution<float> returns z * stddev + mean */
    const float gx = z4[4 * i] * sxf + 0.0f, gy = z4[4 * i + 1] * syf + 0.0f;
    const float gz = z4[4 * i + 2] * szf + 0.0f, ga = z4[4 * i + 3] * saf + 0.0f;
    float sa, ca;
    yaw_sincos(q[3], yaw_trig, &sa, &ca); /* :110-111 */
    const float rand_x = dx + gx;          /* :112 */
    const float rand_y = dy + gy;          /* :113 */
    q[0] += ca * rand_x - sa * rand_y;     /* :114 */
    q[1] += sa * rand_x + ca * rand_y;     /* :115 */
    q[2] += dz + gz;                       /* :116 */
    q[3] += da + ga;                       /* :117 */
  }
}

void orc_init_pose(float* p7, uint64_t P, const float* z4, float x, float y, float z, float a, float xd, float yd,
                   float zd, float ad, int exp_mode)
{
  /* ParticleFilter.cpp:54-77 */
  const float dev = fmaxf(fmaxf(xd, yd), zd);
  const float gc1 = 1. / (dev * sqrt(2 * M_PI));
  const float gc2 = 1. / (2 * dev * dev);
  if (P == 0)
    return;
  p7[0] = x;
  p7[1] = y;
  p7[2] = z;
  p7[3] = a;
  p7[4] = gc1;
  p7[5] = p7[6] = 0;
  for (uint64_t i = 1; i < P; ++i)
  {
    float* q = p7 + 7 * i;
    q[0] = x + (z4[4 * i] * xd + 0.0f);
    q[1] = y + (z4[4 * i + 1] * yd + 0.0f);
    q[2] = z + (z4[4 * i + 2] * zd + 0.0f);
    q[3] = a + (z4[4 * i + 3] * ad + 0.0f);
    const float dist = sqrtf((q[0] - x) * (q[0] - x) + (q[1] - y) * (q[1] - y) + (q[2] - z) * (q[2] - z));
    q[4] = gc1 * exp_f(-dist * dist * gc2, exp_mode);
    q[5] = q[6] = 0;
  }
}

/* ---- computeGrid: exact nearest point over a bucket grid -------------------------------- */

typedef struct
{
  const float* xyz;
  uint64_t n;
  uint32_t stride;
  double lo[3];
  double h;
  int nb[3];
  uint32_t* start;
  uint32_t* order;
  /* query */
  double min[3], res;
  uint32_t qlo[3], qhi[3];
  float c1, c2;
  int exp_mode;
  float* dist;
  float* prob;
  int nthreads;
  int tid;
} grid_job;

/* Exact nearest squared distance; with max_d2 finite the search may stop once no
 * point within sqrt(max_d2) remains possible (the result is then >= max_d2, possibly
 * INFINITY). */
static float nn_sqdist(const grid_job* J, float qx, float qy, float qz, double max_d2)
{
  float best = INFINITY;
  const double qc[3] = { qx, qy, qz };
  int c[3];
  for (int a = 0; a < 3; ++a)
  {
    long v = (long)floor((qc[a] - J->lo[a]) / J->h);
    if (v < 0)
      v = 0;
    if (v > J->nb[a] - 1)
      v = J->nb[a] - 1;
    c[a] = (int)v;
  }
  int rmax = J->nb[0];
  if (J->nb[1] > rmax)
    rmax = J->nb[1];
  if (J->nb[2] > rmax)
    rmax = J->nb[2];
  for (int r = 0; r <= rmax; ++r)
  {
    for (int bz = c[2] - r; bz <= c[2] + r; ++bz)
      for (int by = c[1] - r; by <= c[1] + r; ++by)
        for (int bx = c[0] - r; bx <= c[0] + r; ++bx)
        {
          int ch = abs(bx - c[0]);
          if (abs(by - c[1]) > ch)
            ch = abs(by - c[1]);
          if (abs(bz - c[2]) > ch)
            ch = abs(bz - c[2]);
          if (ch != r || bx < 0 || by < 0 || bz < 0 || bx >= J->nb[0] || by >= J->nb[1] || bz >= J->nb[2])
            continue;
          const uint64_t b = ((uint64_t)bz * J->nb[1] + by) * J->nb[0] + bx;
          for (uint32_t j = J->start[b]; j < J->start[b + 1]; ++j)
          {
            const float* p = J->xyz + (uint64_t)J->order[j] * J->stride;
            /* flann::L2_Simple<float>: result += diff*diff, in float */
            float d = 0;
            float t = qx - p[0];
            d += t * t;
            t = qy - p[1];
            d += t * t;
            t = qz - p[2];
            d += t * t;
            if (d < best)
              best = d;
          }
        }
    double bound = INFINITY;
    for (int a = 0; a < 3; ++a)
    {
      if (c[a] - r > 0)
      {
        double v = qc[a] - (J->lo[a] + (c[a] - r) * J->h);
        if (v < 0)
          v = 0;
        if (v < bound)
          bound = v;
      }
      if (c[a] + r < J->nb[a] - 1)
      {
        double v = (J->lo[a] + (c[a] + r + 1) * J->h) - qc[a];
        if (v < 0)
          v = 0;
        if (v < bound)
          bound = v;
      }
    }
    if (bound == INFINITY)
      break;
    if (best < INFINITY && (double)best < bound * bound * (1.0 - 1e-6))
      break;
    if (bound * bound * (1.0 - 1e-6) > max_d2)
      break;
  }
  return best;
}

static void* grid_worker(void* arg)
{
  const grid_job* J = (const grid_job*)arg;
  const uint32_t wx = J->qhi[0] - J->qlo[0], wy = J->qhi[1] - J->qlo[1], wz = J->qhi[2] - J->qlo[2];
  const uint64_t total = (uint64_t)wx * wy * wz;
  for (uint64_t k = J->tid; k < total; k += J->nthreads)
  {
    const uint32_t ix = J->qlo[0] + (uint32_t)(k % wx);
    const uint32_t iy = J->qlo[1] + (uint32_t)((k / wx) % wy);
    const uint32_t iz = J->qlo[2] + (uint32_t)(k / ((uint64_t)wx * wy));
    /* PointCloudTools.cpp:127-129 */
    const float qx = J->min[0] + (ix * J->res);
    const float qy = J->min[1] + (iy * J->res);
    const float qz = J->min[2] + (iz * J->res);
    if (J->n == 0)
    {
      J->dist[k] = -1.0f; /* PointCloudTools.cpp:142-143 */
      J->prob[k] = 0.0f;
      continue;
    }
    const float dist = nn_sqdist(J, qx, qy, qz, INFINITY);
    J->dist[k] = dist;                                            /* PointCloudTools.cpp:136 */
    J->prob[k] = J->c1 * exp_f(-dist * dist * J->c2, J->exp_mode); /* PointCloudTools.cpp:137 */
  }
  return NULL;
}

/* The point buckets of the exact search (cube side h: twice the mean point spacing). */
static int build_buckets(grid_job* J, const float* xyz, uint64_t n, uint32_t stride)
{
  grid_job base = *J;
  uint32_t* cell = NULL;
  if (n)
  {
    double hi_b[3];
    for (int a = 0; a < 3; ++a)
    {
      base.lo[a] = INFINITY;
      hi_b[a] = -INFINITY;
    }
    for (uint64_t i = 0; i < n; ++i)
      for (int a = 0; a < 3; ++a)
      {
        const double v = xyz[i * stride + a];
        if (v < base.lo[a])
          base.lo[a] = v;
        if (v > hi_b[a])
          hi_b[a] = v;
      }
    double vol = 1.0;
    for (int a = 0; a < 3; ++a)
      vol *= fmax(hi_b[a] - base.lo[a], 1e-3);
    base.h = fmax(cbrt(vol / (double)n) * 2.0, 1e-3);
    uint64_t total = 1;
    for (int a = 0; a < 3; ++a)
    {
      base.nb[a] = (int)floor((hi_b[a] - base.lo[a]) / base.h) + 1;
      total *= (uint64_t)base.nb[a];
    }
    base.start = (uint32_t*)calloc(total + 1, sizeof(uint32_t));
    base.order = (uint32_t*)malloc(n * sizeof(uint32_t));
    cell = (uint32_t*)malloc(n * sizeof(uint32_t));
    uint32_t* fill = (uint32_t*)malloc((total + 1) * sizeof(uint32_t));
    if (!base.start || !base.order || !cell || !fill)
    {
      free(base.start);
      free(base.order);
      free(cell);
      free(fill);
      return -2;
    }
    for (uint64_t i = 0; i < n; ++i)
    {
      int c[3];
      for (int a = 0; a < 3; ++a)
      {
        int v = (int)floor((xyz[i * stride + a] - base.lo[a]) / base.h);
        if (v > base.nb[a] - 1)
          v = base.nb[a] - 1;
        if (v < 0)
          v = 0;
        c[a] = v;
      }
      cell[i] = (uint32_t)(((uint64_t)c[2] * base.nb[1] + c[1]) * base.nb[0] + c[0]);
      base.start[cell[i] + 1]++;
    }
    for (uint64_t b = 0; b < total; ++b)
      base.start[b + 1] += base.start[b];
    memcpy(fill, base.start, (total + 1) * sizeof(uint32_t));
    for (uint64_t i = 0; i < n; ++i)
      base.order[fill[cell[i]]++] = (uint32_t)i;
    free(fill);
  }
  free(cell);
  *J = base;
  return 0;
}

int orc_compute_grid(const float* xyz, uint64_t n, uint32_t stride, const double min[3], const double max[3],
                     double res, double sensor_dev, const uint32_t lo[3], const uint32_t hi[3], int exp_mode,
                     int threads, float* dist, float* prob)
{
  grid_job base;
  memset(&base, 0, sizeof(base));
  base.xyz = xyz;
  base.n = n;
  base.stride = stride;
  base.res = res;
  base.c1 = (float)(1. / (sensor_dev * sqrt(2 * M_PI))); /* PointCloudTools.cpp:114 */
  base.c2 = (float)(1. / (2. * sensor_dev * sensor_dev)); /* PointCloudTools.cpp:115 */
  base.exp_mode = exp_mode;
  base.dist = dist;
  base.prob = prob;
  for (int a = 0; a < 3; ++a)
  {
    base.min[a] = min[a];
    base.qlo[a] = lo[a];
    base.qhi[a] = hi[a];
    if (hi[a] < lo[a])
      return -1;
  }
  (void)max;
  if (build_buckets(&base, xyz, n, stride))
    return -2;
  if (threads < 1)
    threads = 1;
  grid_job* jobs = (grid_job*)malloc(sizeof(grid_job) * threads);
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * threads);
  for (int t = 0; t < threads; ++t)
  {
    jobs[t] = base;
    jobs[t].nthreads = threads;
    jobs[t].tid = t;
    pthread_create(&th[t], NULL, grid_worker, &jobs[t]);
  }
  for (int t = 0; t < threads; ++t)
    pthread_join(th[t], NULL);
  free(jobs);
  free(th);
  free(base.start);
  free(base.order);
  return 0;
}

/* ---- prob of chosen cells --------------------------------------------------------------- */

typedef struct
{
  grid_job J;
  const uint64_t* cells;
  uint64_t m;
  uint32_t size[3];
  double max_d2;
} cells_job;

static void* cells_worker(void* arg)
{
  const cells_job* C = (const cells_job*)arg;
  const grid_job* J = &C->J;
  const uint64_t sxy = (uint64_t)C->size[0] * C->size[1];
  for (uint64_t k = J->tid; k < C->m; k += J->nthreads)
  {
    const uint64_t idx = C->cells[k];
    const uint32_t ix = (uint32_t)(idx % C->size[0]);
    const uint32_t iy = (uint32_t)((idx / C->size[0]) % C->size[1]);
    const uint32_t iz = (uint32_t)(idx / sxy);
    const float qx = J->min[0] + (ix * J->res); /* PointCloudTools.cpp:127-129 */
    const float qy = J->min[1] + (iy * J->res);
    const float qz = J->min[2] + (iz * J->res);
    if (J->n == 0)
    {
      J->prob[k] = 0.0f;
      continue;
    }
    const float dist = nn_sqdist(J, qx, qy, qz, C->max_d2);
    J->prob[k] = (double)dist >= C->max_d2 ? 0.0f : J->c1 * exp_f(-dist * dist * J->c2, J->exp_mode);
  }
  return NULL;
}

int orc_grid_cell_probs(const float* xyz, uint64_t n, uint32_t stride, const double min[3], double res,
                        double sensor_dev, const uint32_t size[3], const uint64_t* cells, uint64_t m, int exp_mode,
                        int threads, float* prob)
{
  cells_job base;
  memset(&base, 0, sizeof(base));
  base.J.xyz = xyz;
  base.J.n = n;
  base.J.stride = stride;
  base.J.res = res;
  base.J.c1 = (float)(1. / (sensor_dev * sqrt(2 * M_PI))); /* PointCloudTools.cpp:114 */
  base.J.c2 = (float)(1. / (2. * sensor_dev * sensor_dev)); /* PointCloudTools.cpp:115 */
  base.J.exp_mode = exp_mode;
  base.J.prob = prob;
  for (int a = 0; a < 3; ++a)
  {
    base.J.min[a] = min[a];
    base.size[a] = size[a];
  }
  base.cells = cells;
  base.m = m;
  /* beyond d^2 = sqrt(120 / c2) the float product d^2*d^2*c2 exceeds 120 and expf
   * underflows to 0 (it is 0 above 103.98): the cell's prob is 0 without the exact d */
  base.max_d2 = sqrt(120.0 / (double)base.J.c2);
  if (build_buckets(&base.J, xyz, n, stride))
    return -2;
  if (threads < 1)
    threads = 1;
  cells_job* jobs = (cells_job*)malloc(sizeof(cells_job) * threads);
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * threads);
  for (int t = 0; t < threads; ++t)
  {
    jobs[t] = base;
    jobs[t].J.nthreads = threads;
    jobs[t].J.tid = t;
    pthread_create(&th[t], NULL, cells_worker, &jobs[t]);
  }
  for (int t = 0; t < threads; ++t)
    pthread_join(th[t], NULL);
  free(jobs);
  free(th);
  free(base.J.start);
  free(base.J.order);
  return 0;
}

/* ---- Philox4x32-10 ------------------------------------------------------------------------ */

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r)
  {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    const uint32_t n1 = (uint32_t)p1;
    const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    const uint32_t n3 = (uint32_t)p0;
    c0 = n0;
    c1 = n1;
    c2 = n2;
    c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

/* ---- scan voxel downsample (pcl::VoxelGrid<PointXYZ>, Node.cpp:130-137) ------------------- */

/* PCL's VoxelGrid is a third-party dependency whose source is not in the reference tree
 * (package.xml lists pcl_ros without a version; the README targets ROS Kinetic, whose
 * PCL is 1.7.x).  This restates its published algorithm (VoxelGrid::applyFilter):
 *   inverse leaf = 1.0f / leaf (float);  min/max over the finite points (float);
 *   voxel counts d = (int64)((max - min) * inv) + 1 per axis; if dx*dy*dz > INT32_MAX the
 *     filter warns and returns its input unchanged;
 *   min_b = (int)floor(min * inv);  div_b = (int)floor(max * inv) - min_b + 1;
 *   per finite point: ijk = (int)(floor(p * inv) - (float)min_b), key = i + j*div_b.x +
 *     k*div_b.x*div_b.y;  sort the (key, point) pairs by key;
 *   per run of equal keys: centroid = first point, += each further point (float), then
 *     /= (float)count; output points in key order, w component 1.
 * The reference sorts with std::sort, whose order among equal keys is unspecified; here
 * the points of a voxel are summed in input order (a stable sort).  With two points per
 * voxel the order cannot matter (float addition commutes).  Returns 1 when the overflow
 * rule returned the input, 0 otherwise; *n_out receives the output count (out must hold
 * n float4 points). */
static int cmp_u64(const void* a, const void* b)
{
  const uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
  return (x > y) - (x < y);
}

int orc_voxel_downsample(const float* xyz, uint64_t n, uint32_t stride, const float leaf[3], float* out4,
                         uint64_t* n_out)
{
  float inv[3], mn[3] = { FLT_MAX, FLT_MAX, FLT_MAX }, mx[3] = { -FLT_MAX, -FLT_MAX, -FLT_MAX };
  uint64_t n_fin = 0;
  for (int a = 0; a < 3; ++a)
    inv[a] = 1.0f / leaf[a];
  for (uint64_t i = 0; i < n; ++i)
  {
    const float* p = xyz + i * stride;
    if (!(isfinite(p[0]) && isfinite(p[1]) && isfinite(p[2])))
      continue;
    ++n_fin;
    for (int a = 0; a < 3; ++a)
    {
      if (p[a] < mn[a])
        mn[a] = p[a];
      if (p[a] > mx[a])
        mx[a] = p[a];
    }
  }
  *n_out = 0;
  if (n_fin == 0)
    return 0;
  /* voxel counts (int64)span + 1 and their product; the product in double, since PCL's
   * int64 product wraps (undefined) beyond 2^63 and a span of 2^31 or more overflows on
   * its own.  The key space div_b.x*div_b.y*div_b.z must also fit 32 bits (PCL's int
   * key would wrap); both count as the overflow that returns the input. */
  double dprod = 1.0, bprod = 1.0;
  int32_t min_b[3], div_b[3];
  for (int a = 0; a < 3; ++a)
  {
    const float span = (mx[a] - mn[a]) * inv[a];
    dprod *= span < 2147483648.0f ? (double)((int64_t)span + 1) : 4294967296.0;
    const float lo = mn[a] * inv[a], hi = mx[a] * inv[a];
    min_b[a] = (int32_t)floorf(lo);
    div_b[a] = (int32_t)floorf(hi) - min_b[a] + 1;
    bprod *= (double)div_b[a];
  }
  if (dprod > (double)INT32_MAX || bprod > 4294967295.0)
  {
    for (uint64_t i = 0; i < n; ++i)
    {
      const float* p = xyz + i * stride;
      out4[4 * i + 0] = p[0];
      out4[4 * i + 1] = p[1];
      out4[4 * i + 2] = p[2];
      out4[4 * i + 3] = 1.0f;
    }
    *n_out = n;
    return 1;
  }
  const uint32_t mul1 = (uint32_t)div_b[0], mul2 = (uint32_t)div_b[0] * (uint32_t)div_b[1];
  uint64_t* kv = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)n_fin);
  uint64_t m = 0;
  for (uint64_t i = 0; i < n; ++i)
  {
    const float* p = xyz + i * stride;
    if (!(isfinite(p[0]) && isfinite(p[1]) && isfinite(p[2])))
      continue;
    uint32_t ijk[3];
    for (int a = 0; a < 3; ++a)
    {
      const float q = p[a] * inv[a];
      ijk[a] = (uint32_t)(int32_t)(floorf(q) - (float)min_b[a]);
    }
    const uint32_t key = ijk[0] + ijk[1] * mul1 + ijk[2] * mul2;
    kv[m++] = ((uint64_t)key << 32) | (uint64_t)(uint32_t)i;
  }
  qsort(kv, (size_t)m, sizeof(uint64_t), cmp_u64);
  uint64_t v = 0;
  for (uint64_t j = 0; j < m;)
  {
    const uint32_t key = (uint32_t)(kv[j] >> 32);
    const float* p = xyz + (kv[j] & 0xFFFFFFFFu) * stride;
    float c[3] = { p[0], p[1], p[2] };
    uint64_t e = j + 1;
    for (; e < m && (uint32_t)(kv[e] >> 32) == key; ++e)
    {
      const float* q = xyz + (kv[e] & 0xFFFFFFFFu) * stride;
      c[0] = c[0] + q[0];
      c[1] = c[1] + q[1];
      c[2] = c[2] + q[2];
    }
    const float cnt = (float)(e - j);
    out4[4 * v + 0] = c[0] / cnt;
    out4[4 * v + 1] = c[1] / cnt;
    out4[4 * v + 2] = c[2] / cnt;
    out4[4 * v + 3] = 1.0f;
    ++v;
    j = e;
  }
  free(kv);
  *n_out = v;
  return 0;
}
