// Multi-session localisation server over filter batches (amcl_batch_*).
//
// Each session is one filter slot of one of the server's lanes: a lane is a batch
// (its own stream, arenas and captured step graphs) with its own scheduler thread,
// so the lanes' steps run concurrently on the GPU.  A session's particles and
// generator state stay on the device between requests.  Clients submit update
// requests (scan, odometry increment, beacon ranges) from any thread; each lane's
// scheduler forms its batch steps: every session of the lane with a pending request
// contributes its oldest one.  Continuous batching: while step k runs on the GPU,
// requests that arrive are staged for step k + 1, which launches as soon as step k's
// results have been read back.  A session's requests complete in submission order
// (one per step).  New sessions go to the lane carrying the fewest particles.
//
// Admission: the server's particle budget bounds the capacity of all open sessions
// together (each lane's arena can hold the whole budget, so a session fits in any
// lane); beyond it amcl_server_open_session fails with AMCL_ENOMEM and the caller
// retries once sessions close.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "common.cuh"

namespace
{
double now_s()
{
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Request
{
  uint64_t ticket;
  double t_submit;
  std::vector<float> xyz;  // n x 4
  std::vector<float> ranges;
  uint32_t n, nr;
  bool has_odom;
  double odom[8];
  double alpha, sigma, roll, pitch;
  int resample;
};

struct Session
{
  int lane = 0;
  int slot = -1;
  uint64_t capacity = 0;
  std::deque<Request> pending;
  int in_flight = 0;  // staged or running requests
};
}  // namespace

struct amcl_server_s
{
  struct Lane
  {
    amcl_batch_t batch = nullptr;
    std::thread worker;
    uint32_t sessions = 0;
    uint64_t particles = 0;       // particle capacity of the lane's sessions (its share of the load)
    std::vector<int64_t> ids;     // the lane's sessions
    uint64_t pending = 0;         // requests queued on the lane's sessions
    // signalled when one of them gets a request (held by pointer: lanes live in a vector)
    std::unique_ptr<std::condition_variable> cv = std::make_unique<std::condition_variable>();
  };
  std::vector<Lane> lanes;
  uint64_t budget = 0, admitted = 0;  // particle capacity of the open sessions
  std::mutex mu;
  std::map<int64_t, Session> sessions;
  int64_t next_session = 1;
  uint64_t next_ticket = 1;
  std::vector<amcl_server_result> done;
  bool stop = false;
  int last_error = AMCL_OK;
  // statistics
  uint64_t steps = 0, requests_done = 0, weights_done = 0;
  double busy_s = 0;
  uint32_t max_batch = 0;
};

namespace
{
void worker_loop(amcl_server_s* S, int lane)
{
  amcl_batch_t batch = S->lanes[lane].batch;
  struct InFlight
  {
    int64_t session;
    int slot;
    uint64_t ticket;
    double t_submit;
    uint64_t weights;
  };
  std::vector<InFlight> flight, next;
  struct Taken
  {
    int64_t session;
    int slot;
    Request r;
  };
  std::vector<Taken> taken;
  std::vector<amcl_server_result> failed;
  amcl_server_s::Lane& L = S->lanes[lane];
  double t_launch = 0;
  while (true)
  {
    // Take the next step's requests (the oldest of each of the lane's sessions) under
    // the server lock, then stage them (copying the clouds) without it, so submits
    // and the other lanes are not held up by the copies.
    next.clear();
    taken.clear();
    failed.clear();
    {
      std::unique_lock<std::mutex> lock(S->mu);
      if (flight.empty())
        L.cv->wait(lock, [&] { return S->stop || L.pending > 0; });
      if (S->stop && flight.empty())
        return;
      for (int64_t id : L.ids)
      {
        auto it = S->sessions.find(id);
        if (it == S->sessions.end() || it->second.pending.empty())
          continue;
        Session& ss = it->second;
        taken.push_back(Taken{ id, ss.slot, std::move(ss.pending.front()) });
        ss.pending.pop_front();
        ss.in_flight += 1;
        L.pending -= 1;
      }
    }
    for (Taken& t : taken)
    {
      const Request& r = t.r;
      const int rc = amcl_batch_stage(batch, t.slot, r.n ? r.xyz.data() : nullptr, r.n, 4,
                                      r.nr ? r.ranges.data() : nullptr, r.nr, r.has_odom ? r.odom : nullptr,
                                      r.alpha, r.sigma, r.roll, r.pitch, r.resample);
      if (rc != AMCL_OK)
      {
        amcl_server_result res{};
        res.ticket = r.ticket;
        res.session = t.session;
        res.status = rc;
        res.t_submit = r.t_submit;
        res.t_done = now_s();
        failed.push_back(res);
        continue;
      }
      next.push_back(InFlight{ t.session, t.slot, r.ticket, r.t_submit, 0 });
    }
    if (!failed.empty())
    {
      std::lock_guard<std::mutex> lock(S->mu);
      for (auto& res : failed)
      {
        S->done.push_back(res);
        auto it = S->sessions.find(res.session);
        if (it != S->sessions.end())
          it->second.in_flight -= 1;
      }
    }
    // Wait for the step in flight, read its results, then launch the next one.
    if (!flight.empty())
    {
      const int rc = amcl_batch_wait(batch);
      const double t = now_s();
      std::lock_guard<std::mutex> lock(S->mu);
      S->busy_s += t - t_launch;
      for (auto& f : flight)
      {
        amcl_server_result res{};
        res.ticket = f.ticket;
        res.session = f.session;
        res.status = rc;
        res.t_submit = f.t_submit;
        res.t_done = t;
        float m7[7];
        double mv[8];
        if (rc == AMCL_OK && amcl_batch_get_mean(batch, f.slot, m7, mv) == AMCL_OK)
        {
          for (int k = 0; k < 4; ++k)
          {
            res.mean[k] = m7[k];
            res.var[k] = mv[4 + k];
          }
        }
        S->done.push_back(res);
        S->requests_done += 1;
        auto it = S->sessions.find(f.session);
        if (it != S->sessions.end())
          it->second.in_flight -= 1;
      }
      S->steps += 1;
      flight.clear();
    }
    if (!next.empty())
    {
      t_launch = now_s();
      const int rc = amcl_batch_step(batch);
      std::lock_guard<std::mutex> lock(S->mu);
      if (rc != AMCL_OK)
      {
        S->last_error = rc;
        for (auto& f : next)
        {
          amcl_server_result res{};
          res.ticket = f.ticket;
          res.session = f.session;
          res.status = rc;
          res.t_submit = f.t_submit;
          res.t_done = now_s();
          S->done.push_back(res);
          auto it = S->sessions.find(f.session);
          if (it != S->sessions.end())
            it->second.in_flight -= 1;
        }
        next.clear();
      }
      S->max_batch = std::max<uint32_t>(S->max_batch, static_cast<uint32_t>(next.size()));
      flight.swap(next);
    }
  }
}
}  // namespace

extern "C" int amcl_server_create_lanes(amcl_server_t* out, uint32_t max_sessions, uint64_t max_particles,
                                        uint64_t max_points_per_step, uint32_t lanes, void* stream)
{
  if (!out || !lanes || lanes > 16 || (stream && lanes != 1))
    return amcl::fail(AMCL_EINVAL, "amcl_server_create_lanes: bad arguments (1-16 lanes; a caller's stream: 1 lane)");
  amcl_server_s* S = new amcl_server_s();
  S->budget = max_particles;
  S->lanes.resize(lanes);
  for (auto& L : S->lanes)
  {
    const int rc = amcl_batch_create(&L.batch, max_sessions, max_particles, max_points_per_step, stream);
    if (rc)
    {
      for (auto& M : S->lanes)
        amcl_batch_destroy(M.batch);
      delete S;
      return rc;
    }
  }
  for (uint32_t k = 0; k < lanes; ++k)
    S->lanes[k].worker = std::thread(worker_loop, S, static_cast<int>(k));
  *out = S;
  return AMCL_OK;
}

extern "C" int amcl_server_create(amcl_server_t* out, uint32_t max_sessions, uint64_t max_particles,
                                  uint64_t max_points_per_step, void* stream)
{
  return amcl_server_create_lanes(out, max_sessions, max_particles, max_points_per_step, stream ? 1u : 4u, stream);
}

extern "C" int amcl_server_destroy(amcl_server_t S)
{
  if (!S)
    return AMCL_OK;
  {
    std::lock_guard<std::mutex> lock(S->mu);
    S->stop = true;
    for (auto& kv : S->sessions)
      kv.second.pending.clear();
  }
  for (auto& L : S->lanes)
    L.cv->notify_all();
  for (auto& L : S->lanes)
    if (L.worker.joinable())
      L.worker.join();
  for (auto& L : S->lanes)
    amcl_batch_destroy(L.batch);
  delete S;
  return AMCL_OK;
}

extern "C" int amcl_server_open_session(amcl_server_t S, amcl_grid_t grid, uint32_t capacity, uint64_t seed,
                                        int num_particles, const float init8[8], int64_t* session)
{
  if (!S || !grid || !init8 || !session || !capacity)
    return amcl::fail(AMCL_EINVAL, "amcl_server_open_session: bad arguments");
  const uint64_t need = (static_cast<uint64_t>(capacity) + 255) & ~255ull;
  int lane = 0;
  {
    std::lock_guard<std::mutex> lock(S->mu);
    if (S->admitted + need > S->budget)
      return amcl::fail(AMCL_ENOMEM, "amcl_server_open_session: the particle budget is taken (admission refused)");
    // the lane carrying the fewest particles: requests scale with them
    for (int k = 1; k < static_cast<int>(S->lanes.size()); ++k)
      if (S->lanes[k].particles < S->lanes[lane].particles)
        lane = k;
    S->admitted += need;  // reserved while the slot is set up (without the server lock)
    S->lanes[lane].sessions += 1;
    S->lanes[lane].particles += need;
  }
  amcl_batch_t batch = S->lanes[lane].batch;
  int slot = -1;
  int rc = amcl_batch_add(batch, grid, capacity, seed, &slot);
  if (!rc)
  {
    rc = amcl_batch_init(batch, slot, num_particles, init8[0], init8[1], init8[2], init8[3], init8[4], init8[5],
                         init8[6], init8[7]);
    if (rc)
      amcl_batch_remove(batch, slot);
  }
  std::lock_guard<std::mutex> lock(S->mu);
  if (rc)
  {
    S->admitted -= need;
    S->lanes[lane].sessions -= 1;
    S->lanes[lane].particles -= need;
    return rc;
  }
  const int64_t id = S->next_session++;
  Session& ss = S->sessions[id];
  ss.lane = lane;
  ss.slot = slot;
  ss.capacity = need;
  S->lanes[lane].ids.push_back(id);
  *session = id;
  return AMCL_OK;
}

extern "C" int amcl_server_close_session(amcl_server_t S, int64_t session)
{
  if (!S)
    return amcl::fail(AMCL_EINVAL, "amcl_server_close_session: null server");
  // Wait until the session has nothing pending or in flight, then take it out of the
  // schedule and free its slot (waiting for the lane's current step, not under the
  // server lock).
  Session ss;
  for (int spins = 0;; ++spins)
  {
    {
      std::lock_guard<std::mutex> lock(S->mu);
      auto it = S->sessions.find(session);
      if (it == S->sessions.end())
        return amcl::fail(AMCL_EINVAL, "amcl_server_close_session: no such session");
      if (it->second.pending.empty() && it->second.in_flight == 0)
      {
        ss = it->second;
        S->sessions.erase(it);
        auto& ids = S->lanes[ss.lane].ids;
        ids.erase(std::remove(ids.begin(), ids.end(), session), ids.end());
        break;
      }
    }
    if (spins > 200000)
      return amcl::fail(AMCL_ETIMEDOUT, "amcl_server_close_session: requests still pending");
    std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
  const int rc = amcl_batch_remove(S->lanes[ss.lane].batch, ss.slot);
  std::lock_guard<std::mutex> lock(S->mu);
  S->admitted -= ss.capacity;
  S->lanes[ss.lane].sessions -= 1;
  S->lanes[ss.lane].particles -= ss.capacity;
  return rc;
}

extern "C" int amcl_server_submit(amcl_server_t S, int64_t session, const float* xyz, uint32_t n,
                                  uint32_t stride_floats, const float* ranges4, uint32_t nr, const double* odom8,
                                  double alpha, double sigma, double roll, double pitch, int resample,
                                  uint64_t* ticket)
{
  if (!S || (n && !xyz) || (nr && !ranges4) || stride_floats < 3)
    return amcl::fail(AMCL_EINVAL, "amcl_server_submit: bad arguments");
  Request r;
  r.t_submit = now_s();
  r.n = n;
  r.nr = nr;
  r.xyz.resize(4ull * n);
  for (uint32_t i = 0; i < n; ++i)
  {
    r.xyz[4ull * i] = xyz[static_cast<uint64_t>(i) * stride_floats];
    r.xyz[4ull * i + 1] = xyz[static_cast<uint64_t>(i) * stride_floats + 1];
    r.xyz[4ull * i + 2] = xyz[static_cast<uint64_t>(i) * stride_floats + 2];
    r.xyz[4ull * i + 3] = 0.0f;
  }
  r.ranges.assign(ranges4, ranges4 + 4ull * nr);
  r.has_odom = odom8 != nullptr;
  if (odom8)
    std::memcpy(r.odom, odom8, sizeof(r.odom));
  r.alpha = alpha;
  r.sigma = sigma;
  r.roll = roll;
  r.pitch = pitch;
  r.resample = resample;
  int lane = 0;
  {
    std::lock_guard<std::mutex> lock(S->mu);
    auto it = S->sessions.find(session);
    if (it == S->sessions.end())
      return amcl::fail(AMCL_EINVAL, "amcl_server_submit: no such session");
    r.ticket = S->next_ticket++;
    if (ticket)
      *ticket = r.ticket;
    lane = it->second.lane;
    it->second.pending.push_back(std::move(r));
    S->lanes[lane].pending += 1;
  }
  S->lanes[lane].cv->notify_one();  // the session's lane picks it up
  return AMCL_OK;
}

extern "C" int amcl_server_poll(amcl_server_t S, amcl_server_result* out, uint32_t cap, uint32_t* n)
{
  if (!S || !n || (cap && !out))
    return amcl::fail(AMCL_EINVAL, "amcl_server_poll: bad arguments");
  std::lock_guard<std::mutex> lock(S->mu);
  const uint32_t m = std::min<uint32_t>(cap, static_cast<uint32_t>(S->done.size()));
  for (uint32_t i = 0; i < m; ++i)
    out[i] = S->done[i];
  S->done.erase(S->done.begin(), S->done.begin() + m);
  *n = m;
  return AMCL_OK;
}

extern "C" int amcl_server_stats(amcl_server_t S, uint64_t* steps, uint64_t* requests, double* busy_s,
                                 uint32_t* max_batch, uint32_t* sessions)
{
  if (!S)
    return amcl::fail(AMCL_EINVAL, "amcl_server_stats: null server");
  std::lock_guard<std::mutex> lock(S->mu);
  if (steps)
    *steps = S->steps;
  if (requests)
    *requests = S->requests_done;
  if (busy_s)
    *busy_s = S->busy_s;
  if (max_batch)
    *max_batch = S->max_batch;
  if (sessions)
    *sessions = static_cast<uint32_t>(S->sessions.size());
  return AMCL_OK;
}

extern "C" int amcl_server_counters(amcl_server_t S, uint64_t* graphs_built, uint64_t* reallocs)
{
  if (!S)
    return amcl::fail(AMCL_EINVAL, "amcl_server_counters: null server");
  uint64_t g = 0, r = 0;
  for (auto& L : S->lanes)
  {
    uint64_t lg = 0, lr = 0;
    const int rc = amcl_batch_counters(L.batch, nullptr, &lg, &lr);
    if (rc)
      return rc;
    g += lg;
    r += lr;
  }
  if (graphs_built)
    *graphs_built = g;
  if (reallocs)
    *reallocs = r;
  return AMCL_OK;
}

extern "C" int amcl_server_batch(amcl_server_t S, amcl_batch_t* batch)
{
  if (!S || !batch)
    return amcl::fail(AMCL_EINVAL, "amcl_server_batch: bad arguments");
  *batch = S->lanes[0].batch;
  return AMCL_OK;
}
