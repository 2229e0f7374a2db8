/*
 * amcl3d_gpu.h - C ABI of the GB300 particle-filter hot path of amcl3d.
 *
 * Two opaque handles mirror the two classes of the amcl3d filter core:
 *   amcl_grid_t  <->  amcl3d::Grid3d         (amcl3d/src/Grid3d.h:34-159)
 *   amcl_pf_t    <->  amcl3d::ParticleFilter (amcl3d/src/ParticleFilter.h:67-213)
 * Every entry point returns an int status (AMCL_OK on success); amcl_last_error()
 * gives the detail of the last failure on the calling thread.  Plain pointers and
 * sizes only: no C++ or CUDA types cross this boundary (streams are passed as
 * void*, a cudaStream_t or NULL for a stream the library creates).
 *
 * Host arrays are copied to the device inside the call; *_dev variants take
 * device pointers for callers whose inputs are already resident in HBM.
 * Calls on one handle are ordered on that handle's stream; entry points that
 * return values to the host synchronise that stream.  A handle must not be used
 * from two threads at once.
 */
#ifndef AMCL3D_GPU_H
#define AMCL3D_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------ */
enum
{
  AMCL_OK = 0,
  AMCL_EINVAL = 1,    /* bad argument (null handle, size out of range, ...)        */
  AMCL_ENOMEM = 2,    /* device or pinned-host allocation failed                   */
  AMCL_ECUDA = 3,     /* a CUDA runtime call failed                                */
  AMCL_ETIMEDOUT = 4, /* a bounded device-side wait gave up                        */
  AMCL_ESTATE = 5,    /* call not valid in the handle's state (e.g. no grid yet)   */
  AMCL_EIO = 6,       /* file could not be read or written                         */
  AMCL_ERANGE = 7,    /* input exceeds a documented limit                          */
  AMCL_ENOTSUP = 8    /* option not supported for this handle                      */
};

const char* amcl_status_string(int status);
const char* amcl_last_error(void);
int amcl_version(int* major, int* minor);

/* ---- grid storage of the gathered per-cell probability -------------------------- */
enum
{
  AMCL_GRID_F32 = 0, /* float, what the reference stores in Grid3dCell::prob          */
  AMCL_GRID_F16 = 1, /* IEEE half                                                     */
  AMCL_GRID_U8 = 2   /* uint8 code q, prob = q * scale, scale = max(prob) / 255        */
};

typedef struct amcl_grid_s* amcl_grid_t;
typedef struct amcl_pf_s* amcl_pf_t;
typedef struct amcl_voxel_s* amcl_voxel_t;

/* Mirrors PointCloudInfo's bounds/resolution (PointCloudTools.h:54-68) and
 * Grid3dInfo's sizes (PointCloudTools.h:37-50). */
typedef struct
{
  double min[3];     /* octo_min_x/y/z                                               */
  double max[3];     /* octo_max_x/y/z                                               */
  double resolution; /* octo_resol                                                   */
  double sensor_dev; /* Grid3dInfo::sensor_dev                                       */
  uint32_t size[3];  /* size_x, size_y, size_z = ceil((max - min) / resolution)      */
  uint32_t storage;  /* AMCL_GRID_* currently used by the weighting kernels          */
  float u8_scale;    /* scale of the uint8 storage (0 if not built)                  */
  uint32_t reserved;
} amcl_grid_info;

/* ---- Grid3d --------------------------------------------------------------------- */

/* Creates an empty grid bound to `stream` (NULL: the library creates one). */
int amcl_grid_create(amcl_grid_t* out, void* stream);
int amcl_grid_destroy(amcl_grid_t g);

/* computeGrid (PointCloudTools.cpp:84-149), reached through Grid3d::open
 * (Grid3d.cpp:25-78), also named buildGridMap: builds the nearest-occupied
 * squared-distance field and its probability c1*expf(-d2*d2*c2) on the device from
 * the occupied-leaf centres `xyz` (n points, `stride_floats` floats apart) and the
 * octomap bounds.  The reference refuses more than 250e6 cells
 * (PointCloudTools.cpp:103-105); this build accepts up to 2^32-1 cells (the limit of
 * the reference's uint32 cell index, Grid3d.cpp:187) and returns AMCL_ERANGE above. */
int amcl_grid_build(amcl_grid_t g, const float* xyz, uint64_t n, uint32_t stride_floats, const double min[3],
                    const double max[3], double resolution, double sensor_dev);

/* Loads cells computed elsewhere (host arrays of size_x*size_y*size_z floats; dist
 * may be NULL).  The sizes in `info` must equal ceil((max-min)/res) per axis. */
int amcl_grid_load_cells(amcl_grid_t g, const amcl_grid_info* info, const float* dist, const float* prob);

/* The reference's .grid cache (Grid3d::saveGrid/loadGrid, Grid3d.cpp:210-275):
 * uint32 size_x,size_y,size_z; double sensor_dev; {float dist, float prob}[cells].
 * load rejects a sensor_dev that differs by >= DBL_EPSILON (Grid3d.cpp:256-260,
 * returns AMCL_ESTATE) and a file whose sizes do not match the bounds. */
int amcl_grid_save(amcl_grid_t g, const char* path);
int amcl_grid_load(amcl_grid_t g, const char* path, const double min[3], const double max[3], double resolution,
                   double sensor_dev);

int amcl_grid_info_get(amcl_grid_t g, amcl_grid_info* out);
/* Copies cells [first, first+count) to host arrays (either may be NULL). */
int amcl_grid_read_cells(amcl_grid_t g, uint64_t first, uint64_t count, float* dist, float* prob);

/* Selects the storage the weighting kernels gather (building F16/U8 copies from the
 * F32 probabilities on first use). */
int amcl_grid_set_storage(amcl_grid_t g, int storage);

/* The yaw-only cloud-weighting loop this grid selects (no reference counterpart; the
 * cells are the same on every loop): 0 = the general loop (a float-float estimate with a
 * margin test per point), 1 = the zero-minimum loop (every offset double(t) - min is a
 * float: the cell index read off the floor bits), 2 = the general yaw loop for a minimum
 * that makes the offsets non-floats (a real map's).  AMCL_ESTATE if not built. */
int amcl_grid_weight_loop(amcl_grid_t g, int* loop);

/* Keeps the gathered probability array in an L2 persisting access-policy window on
 * this grid's stream and on the streams of filters that use it (0 = off, default). */
int amcl_grid_set_l2_window(amcl_grid_t g, int enable);

/* Grid3d::isIntoMap (Grid3d.cpp:201-208): min <= p < max per axis, 0 if not built. */
int amcl_grid_is_into_map(amcl_grid_t g, float x, float y, float z, int* inside);

/* Grid3d::computeCloudWeight (Grid3d.cpp:133-199) for P poses (x, y, z, yaw as 4
 * floats each) and one host cloud (n points, stride_floats apart) at shared roll and
 * pitch.  out[p] is the mean probability of the in-grid points, 0 if 10 or fewer
 * points fall inside the grid (and 0 for every pose when no grid is built). */
int amcl_grid_cloud_weights(amcl_grid_t g, const float* poses4, uint32_t P, const float* xyz, uint32_t n,
                            uint32_t stride_floats, float roll, float pitch, float* out);

/* No counterpart in the reference.  The same weights as amcl_grid_cloud_weights
 * for callers that must not allocate device memory (a real-time loop that may not
 * enter the CUDA allocator, memory handed out only by a host framework's pool):
 * nothing is allocated; the two-phase kernel's scratch is a fixed 16 MiB
 * file-scope device array that every GPU loading the library holds until exit.
 * poses (P x float4 x, y, z, yaw) and cloud (n x float4 x, y, z, unused) are
 * 16-byte aligned device buffers, out is P device floats (all 0 when no grid is
 * built, as amcl_grid_cloud_weights gives); the call runs on `stream` (NULL: the
 * default stream) and waits for that stream to finish before it returns.  Limits: P <= 65536 and
 * ceil(P/32)*32*n <= 4194304, else AMCL_ERANGE.  All calls share the array, so calls
 * that overlap on the GPU race.  The first call on a device looks the array's
 * address up; make it before any stream capture. */
int amcl_grid_cloud_weights_noalloc(amcl_grid_t g, const void* poses_f4_dev, uint32_t P, const void* cloud_f4_dev,
                                    uint32_t n, float roll, float pitch, float* out_dev, void* stream);

/* openOcTree + computePointCloud (PointCloudTools.cpp:26-82) without the octomap
 * library, from octomap's file formats (.bt binary, .ot full): the centres of the
 * occupied leaves as float4 (x, y, z, 1) in the leaf iterator's order (at most cap;
 * xyz4 may be NULL to ask for the count), the metric bounds over every leaf and the
 * resolution.  AMCL_EIO when the file cannot be read; AMCL_EINVAL for another
 * extension, a malformed file, a tree that is not an OcTree or an empty tree (the
 * cases where openOcTree / computePointCloud throw). */
int amcl_octomap_read(const char* path, float* xyz4, uint64_t cap, uint64_t* n_points, double min[3], double max[3],
                      double* resolution, uint64_t* tree_nodes);

/* Grid3d::open (Grid3d.cpp:25-78): reads the map as amcl_octomap_read does, loads
 * the .grid file beside it when that matches (amcl_grid_load), else builds the
 * distance field on the GPU and writes that file (a failed write is not an error).
 * *n_points (may be NULL) receives the occupied leaf count. */
int amcl_grid_open(amcl_grid_t g, const char* map_path, double sensor_dev, uint64_t* n_points);

/* Grid3d::buildGridSliceMsg (Grid3d.cpp:80-121): int8 occupancy of the z slice,
 * prob scaled to 0..100 by the slice maximum.  Writes min(cap, len) values; *len,
 * *width, *height receive the message sizes.  AMCL_EINVAL when z is outside the map. */
int amcl_grid_slice(amcl_grid_t g, double z, int8_t* out, uint64_t cap, uint64_t* len, uint32_t* width,
                    uint32_t* height);

/* ---- ParticleFilter ----------------------------------------------------------------
 * Particles are exchanged as amcl3d::Particle, 7 floats each in this order:
 * x, y, z, a (yaw), w, wp, wr (ParticleFilter.h:35-49). */

int amcl_pf_create(amcl_pf_t* out, uint64_t seed, void* stream);
int amcl_pf_destroy(amcl_pf_t pf);

/* ParticleFilter::init (ParticleFilter.cpp:46-95), also named
 * buildParticlesPool: |num_particles| particles, particle 0 at the given pose, the
 * rest drawn from N(pose, dev) per axis; weights c1*exp(-d^2*c2) with
 * dev = max(x_dev, y_dev, z_dev), normalised; the mean is computed. */
int amcl_pf_init(amcl_pf_t pf, int num_particles, float x, float y, float z, float a, float x_dev, float y_dev,
                 float z_dev, float a_dev);

/* ParticleFilter::predict (ParticleFilter.cpp:97-119). */
int amcl_pf_predict(amcl_pf_t pf, double odom_x_mod, double odom_y_mod, double odom_z_mod, double odom_a_mod,
                    double delta_x, double delta_y, double delta_z, double delta_a);

/* ParticleFilter::update (ParticleFilter.cpp:121-196) with a host cloud (n points,
 * stride_floats apart; PCL's PointXYZ is 4 floats) and nr ranges given as
 * (r, ax, ay, az) float quadruples (ParticleFilter.h:53-63). */
int amcl_pf_update(amcl_pf_t pf, amcl_grid_t g, const float* xyz, uint32_t n, uint32_t stride_floats,
                   const float* ranges4, uint32_t nr, double alpha, double sigma, double roll, double pitch);

/* Same, with the cloud already on the device as n float4 (x, y, z, unused),
 * 16-byte aligned, and the ranges on the host.  The cloud must stay valid until the
 * next call that synchronises this filter's stream. */
int amcl_pf_update_dev(amcl_pf_t pf, amcl_grid_t g, const void* cloud_f4_dev, uint32_t n, const float* ranges4,
                       uint32_t nr, double alpha, double sigma, double roll, double pitch);

/* Range-only update declared at ParticleFilter.h:157 but never defined by the
 * reference: wr from the beacons only, wp = 0, w = (1 - alpha) * wr normalised. */
int amcl_pf_update_ranges(amcl_pf_t pf, const float* ranges4, uint32_t nr, double alpha, double sigma);

/* ParticleFilter::resample (ParticleFilter.cpp:198-222), systematic: the uniform
 * draw comes from this filter's counter-based generator. */
int amcl_pf_resample(amcl_pf_t pf);
/* Same with the uniform draw u01 in [0, 1) given by the caller (r = u01 / N). */
int amcl_pf_resample_with(amcl_pf_t pf, float u01);

/* ParticleFilter::getMean (ParticleFilter.h:94-97): the mean stored by the last
 * init/update as a Particle (7 floats; w, wp, wr are 0).  If mean_var is not NULL it
 * receives the double mean x, y, z, a then the weighted variance x, y, z, a. */
int amcl_pf_get_mean(amcl_pf_t pf, float mean7[7], double mean_var[8]);

int amcl_pf_is_initialized(amcl_pf_t pf, int* initialized);
int amcl_pf_size(amcl_pf_t pf, uint32_t* n);
/* Copies min(cap, size) particles out / replaces the particle set (parity injection). */
int amcl_pf_get_particles(amcl_pf_t pf, float* p7, uint32_t cap);
int amcl_pf_set_particles(amcl_pf_t pf, const float* p7, uint32_t n);

/* Options (amcl_pf_set_option). */
enum
{
  /* Sum of the per-point probabilities inside a particle's weight:
   * 0 = float running sum in cloud order (the reference's arithmetic, bit-exact),
   * 1 = compensated (Neumaier) float sum in cloud order. */
  AMCL_OPT_CLOUD_SUM = 1,
  /* Cumulative weights driving resample:
   * 0 = exact (fixed-point, equal to the correctly rounded real prefix),
   * 1 = float running sum in particle order (the reference's arithmetic). */
  AMCL_OPT_RESAMPLE_PREFIX = 2,
  /* Weighting kernel: 0 = automatic, 1 = one thread per particle over the whole
   * cloud, 2 = two-phase (point tiles across the GPU, then ordered per-particle
   * sums from a device scratch buffer). */
  AMCL_OPT_WEIGHT_KERNEL = 3,
  /* Seed of the counter-based generator (resets its counter). */
  AMCL_OPT_SEED = 4,
  /* Test of the bounded device-side waits: 1 = the next update's two-phase weighting
   * waits on a barrier that nothing completes, gives up after a short budget (before
   * it issues any copy) and weighs nothing; the update's result is then reported as
   * AMCL_ETIMEDOUT by the next call that reads the filter back.  One use, then 0. */
  AMCL_OPT_WAIT_PROBE = 5
};
int amcl_pf_set_option(amcl_pf_t pf, int option, int64_t value);

/* Debug/parity: the four normal draws (x, y, z, a order) of the last predict or
 * init, 4*size floats.  Recorded only while enabled. */
int amcl_pf_record_draws(amcl_pf_t pf, int enable);
int amcl_pf_get_draws(amcl_pf_t pf, float* out, uint32_t cap_floats);
/* Debug/parity: the last resample's source index per output particle. */
int amcl_pf_get_resample_index(amcl_pf_t pf, int32_t* out, uint32_t cap);

/* ---- scan voxel downsample ---------------------------------------------------------
 * pcl::VoxelGrid<pcl::PointXYZ> as Node.cpp:130-137 runs it on every accepted scan
 * (setLeafSize(voxel_size, voxel_size, voxel_size); filter): one centroid per occupied
 * leaf, in voxel-key order, w component 1; the points of a leaf are summed in input
 * order; non-finite points are skipped; when the leaf count overflows int32 the input
 * is returned unchanged.  A handle owns the device scratch and a stream; calls on one
 * handle are serialised. */
int amcl_voxel_create(amcl_voxel_t* out, void* stream);
int amcl_voxel_destroy(amcl_voxel_t v);
int amcl_voxel_stream(amcl_voxel_t v, void** stream);

/* Host cloud in (n points, stride_floats apart), host centroids out (float4 each, at
 * most cap); *n_out receives the centroid count (AMCL_ERANGE if it exceeds cap).
 * Leaf sizes must be positive and finite; n <= 2^30. */
int amcl_voxel_filter(amcl_voxel_t v, const float* xyz, uint64_t n, uint32_t stride_floats, float leaf_x,
                      float leaf_y, float leaf_z, float* out4, uint64_t cap, uint64_t* n_out);

/* Device cloud in (n float4, 16-byte aligned), device centroids out (room for n
 * float4); runs on the handle's stream and synchronises it to return *n_out. */
int amcl_voxel_filter_dev(amcl_voxel_t v, const void* in_f4_dev, uint64_t n, float leaf_x, float leaf_y, float leaf_z,
                          void* out_f4_dev, uint64_t* n_out);

/* Node.cpp:130-162 on the device: the raw host scan is copied in once, downsampled
 * by the voxel filter on this filter's stream and weighed from device memory by
 * ParticleFilter::update (as amcl_pf_update).  The downsampled cloud (the node
 * publishes it) is copied to down4 when down4 is not NULL (at most down_cap points,
 * AMCL_ERANGE beyond); *n_down receives its size. */
int amcl_pf_update_voxel(amcl_pf_t pf, amcl_grid_t g, amcl_voxel_t v, const float* xyz, uint32_t n,
                         uint32_t stride_floats, float leaf_x, float leaf_y, float leaf_z, const float* ranges4,
                         uint32_t nr, double alpha, double sigma, double roll, double pitch, float* down4,
                         uint64_t down_cap, uint64_t* n_down);

/* ---- batches: many filters stepped together ------------------------------------------------
 * No counterpart in the reference (one filter per node there).  A batch owns fixed
 * device arenas sized at creation: `max_particles` particles in total over at most
 * `max_filters` filters, and `max_points_per_step` scan points over all filters of one
 * step.  Adding a filter that does not fit fails with AMCL_ENOMEM (admission against
 * the memory budget).  Each filter in a batch computes exactly what a single
 * amcl_pf_t with the same seed computes (same arithmetic, exact sums), whatever the
 * other filters in the step.  All calls on one batch must come from one thread at a
 * time. */
typedef struct amcl_batch_s* amcl_batch_t;

int amcl_batch_create(amcl_batch_t* out, uint32_t max_filters, uint64_t max_particles, uint64_t max_points_per_step,
                      void* stream);
int amcl_batch_destroy(amcl_batch_t b);
/* A filter slot with room for `capacity` particles on `grid` (may be changed later). */
int amcl_batch_add(amcl_batch_t b, amcl_grid_t grid, uint32_t capacity, uint64_t seed, int* slot);
int amcl_batch_remove(amcl_batch_t b, int slot);
int amcl_batch_set_grid(amcl_batch_t b, int slot, amcl_grid_t grid);
/* ParticleFilter::init for one slot (as amcl_pf_init). */
int amcl_batch_init(amcl_batch_t b, int slot, int num_particles, float x, float y, float z, float a, float x_dev,
                    float y_dev, float z_dev, float a_dev);
int amcl_batch_set_particles(amcl_batch_t b, int slot, const float* p7, uint32_t n);
int amcl_batch_get_particles(amcl_batch_t b, int slot, float* p7, uint32_t cap);
/* Stages one filter step for the next amcl_batch_step: predict with odom8 =
 * (x_mod, y_mod, z_mod, a_mod, delta_x, delta_y, delta_z, delta_a) unless NULL, then
 * update with the cloud and ranges (as amcl_pf_update), then resample if `resample`. */
int amcl_batch_stage(amcl_batch_t b, int slot, const float* xyz, uint32_t n, uint32_t stride_floats,
                     const float* ranges4, uint32_t nr, const double* odom8, double alpha, double sigma, double roll,
                     double pitch, int resample);
/* amcl_batch_stage for `count` filters whose clouds are packed one after another in
 * one host array: filter k (slot slots[k], each slot at most once) takes the next n[k]
 * points of xyz (stride_floats apart) and the next nr[k] ranges of ranges4 (nr NULL:
 * none), odometry odom8[8k..8k+7] (NULL: no predict).  Every argument is checked
 * before anything is staged; the copies run on several host threads when large. */
int amcl_batch_stage_packed(amcl_batch_t b, uint32_t count, const int* slots, const float* xyz, const uint32_t* n,
                            uint32_t stride_floats, const float* ranges4, const uint32_t* nr, const double* odom8,
                            double alpha, double sigma, double roll, double pitch, int resample);
/* amcl_batch_stage for `count` filters in one call: slots[k] gets clouds[k] (n[k]
 * points, stride_floats apart), nr[k] ranges at ranges4[k] (nr and ranges4 may be
 * NULL: no ranges), odometry odom8[8k..8k+7] (odom8 NULL: no predict); the other
 * parameters are shared.  Stops at the first failing filter. */
int amcl_batch_stage_many(amcl_batch_t b, uint32_t count, const int* slots, const float* const* clouds,
                          const uint32_t* n, uint32_t stride_floats, const float* const* ranges4, const uint32_t* nr,
                          const double* odom8, double alpha, double sigma, double roll, double pitch, int resample);
/* Launches the staged steps of every filter (one CUDA graph launch); returns before
 * they finish.  Staging for the next step may proceed meanwhile. */
int amcl_batch_step(amcl_batch_t b);
int amcl_batch_wait(amcl_batch_t b);
/* Mean (and double mean + variance) of a slot's last completed update (waits). */
int amcl_batch_get_mean(amcl_batch_t b, int slot, float mean7[7], double mean_var[8]);
/* Shape of the weighting kernel: particle tile (threads per block: 64, 128, 256, 512)
 * and point tile (scan points staged in shared memory per iteration). */
int amcl_batch_set_tuning(amcl_batch_t b, int threads, int chunk);

/* Point-parallel weighting of small steps: mode 0 (default) splits every filter's
 * scan over the SMs when the step's particle tiles cannot fill the GPU, 1 never
 * splits, 2 always splits (when the probability slabs fit).  scratch_bytes (0: keep;
 * default 4 GiB) bounds the slab memory a split step may allocate.  Results are the
 * same either way. */
int amcl_batch_set_split(amcl_batch_t b, int mode, uint64_t scratch_bytes);
int amcl_batch_get_tuning(amcl_batch_t b, int* threads, int* chunk);
/* Times the weighting phase of the last step under each candidate (particle tile x
 * point tile) shape, `reps` runs each, keeps the fastest and reports it.  The state of
 * every filter is restored afterwards. */
int amcl_batch_autotune(amcl_batch_t b, int reps, int* best_threads, int* best_chunk, double* best_ms);
/* Largest contiguous free particle range and free slots (admission headroom). */
int amcl_batch_capacity(amcl_batch_t b, uint64_t* free_particles, uint32_t* free_slots);
/* Steps launched, CUDA graphs captured and work buffers regrown since creation (each
 * capture and regrowth is a pause of that batch's stream; any may be NULL). */
int amcl_batch_counters(amcl_batch_t b, uint64_t* steps, uint64_t* graphs_built, uint64_t* reallocs);
int amcl_batch_stream(amcl_batch_t b, void** stream);

/* ---- server: many localisation sessions, continuous batching ------------------------------
 * No counterpart in the reference.  Sessions are filter slots of internal batches
 * (lanes; state resident on the device); submitted update requests are served by one
 * scheduler thread per lane that steps every session of the lane with a pending
 * request together, staging requests that arrive during a step for the next one.  Results come back through
 * amcl_server_poll in completion order; times are seconds of a monotonic clock. */
typedef struct amcl_server_s* amcl_server_t;
typedef struct
{
  uint64_t ticket;
  int64_t session;
  int32_t status; /* AMCL_OK or the failure of this request's step */
  int32_t reserved;
  double t_submit, t_done;
  float mean[4]; /* x, y, z, yaw after the update */
  double var[4];
} amcl_server_result;

int amcl_server_create(amcl_server_t* out, uint32_t max_sessions, uint64_t max_particles, uint64_t max_points_per_step,
                       void* stream);
/* The same with `lanes` (1-16) concurrent batches, each with its own stream and
 * scheduler thread (amcl_server_create: 4 lanes, or 1 on a caller's stream).  Every
 * lane's arena can hold max_particles; max_particles bounds the sessions' total. */
int amcl_server_create_lanes(amcl_server_t* out, uint32_t max_sessions, uint64_t max_particles,
                             uint64_t max_points_per_step, uint32_t lanes, void* stream);
int amcl_server_destroy(amcl_server_t s);
/* Admission: AMCL_ENOMEM when the session does not fit in the remaining budget.
 * init8 = (x, y, z, yaw, x_dev, y_dev, z_dev, yaw_dev) of ParticleFilter::init. */
int amcl_server_open_session(amcl_server_t s, amcl_grid_t grid, uint32_t capacity, uint64_t seed, int num_particles,
                             const float init8[8], int64_t* session);
/* Waits for the session's pending requests, then frees its slot. */
int amcl_server_close_session(amcl_server_t s, int64_t session);
/* One update request (predict with odom8 unless NULL, update, resample if asked). */
int amcl_server_submit(amcl_server_t s, int64_t session, const float* xyz, uint32_t n, uint32_t stride_floats,
                       const float* ranges4, uint32_t nr, const double* odom8, double alpha, double sigma,
                       double roll, double pitch, int resample, uint64_t* ticket);
int amcl_server_poll(amcl_server_t s, amcl_server_result* out, uint32_t cap, uint32_t* n);
int amcl_server_stats(amcl_server_t s, uint64_t* steps, uint64_t* requests, double* busy_s, uint32_t* max_batch,
                      uint32_t* sessions);
/* amcl_batch_counters summed over the lanes. */
int amcl_server_counters(amcl_server_t s, uint64_t* graphs_built, uint64_t* reallocs);
/* The batch of the first lane. */
int amcl_server_batch(amcl_server_t s, amcl_batch_t* batch);

/* Raw stream of the handle (cudaStream_t), for callers that time it with events. */
int amcl_pf_stream(amcl_pf_t pf, void** stream);
int amcl_grid_stream(amcl_grid_t g, void** stream);

/* ---- profiling: device time per kernel family, measured with CUDA events ---------- */
enum
{
  AMCL_PROF_CLOUD_WEIGHT = 0, /* the per-particle cloud weighting kernel(s)      */
  AMCL_PROF_NORMALIZE = 1,    /* blend + normalisation + mean                     */
  AMCL_PROF_RESAMPLE = 2,
  AMCL_PROF_PREDICT = 3,
  AMCL_PROF_DISTANCE_FIELD = 4,
  AMCL_PROF_COUNT = 5
};
/* Enables event pairs around each kernel family on the filter's stream. */
int amcl_pf_profile(amcl_pf_t pf, int enable);
/* Synchronises and returns the accumulated milliseconds and launch counts. */
int amcl_pf_profile_read(amcl_pf_t pf, double ms[AMCL_PROF_COUNT], uint64_t launches[AMCL_PROF_COUNT],
                         int reset);
/* Kernel launches issued so far by this process (all handles). */
uint64_t amcl_kernel_launches(void);

#ifdef __cplusplus
}
#endif

#endif /* AMCL3D_GPU_H */
