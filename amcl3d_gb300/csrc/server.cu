// Multi-session localisation server over a filter batch (amcl_batch_*).
//
// Each session is one filter slot of the batch: its particles and generator state
// stay on the device between requests.  Clients submit update requests (scan,
// odometry increment, beacon ranges) from any thread; a scheduler thread forms the
// batch steps: every session with a pending request contributes its oldest one.
// Continuous batching: while step k runs on the GPU, requests that arrive are
// staged for step k + 1, which launches as soon as step k's results have been read
// back.  A session's requests complete in submission order (one per step).
//
// Admission: opening a session takes a slot and a particle range of the batch's
// fixed arenas; when they are exhausted amcl_server_open_session fails with
// AMCL_ENOMEM and the caller retries once sessions close.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
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
  int slot = -1;
  std::deque<Request> pending;
  int in_flight = 0;  // staged or running requests
};
}  // namespace

struct amcl_server_s
{
  amcl_batch_t batch = nullptr;
  std::mutex mu;
  std::condition_variable cv;
  std::map<int64_t, Session> sessions;
  int64_t next_session = 1;
  uint64_t next_ticket = 1;
  std::vector<amcl_server_result> done;
  std::thread worker;
  bool stop = false;
  int last_error = AMCL_OK;
  // statistics
  uint64_t steps = 0, requests_done = 0, weights_done = 0;
  double busy_s = 0;
  uint32_t max_batch = 0;
};

namespace
{
void worker_loop(amcl_server_s* S)
{
  struct InFlight
  {
    int64_t session;
    int slot;
    uint64_t ticket;
    double t_submit;
    uint64_t weights;
  };
  std::vector<InFlight> flight, next;
  double t_launch = 0;
  while (true)
  {
    // Stage the next step from the pending requests (one per session).
    next.clear();
    {
      std::unique_lock<std::mutex> lock(S->mu);
      if (flight.empty())
        S->cv.wait(lock, [&] {
          if (S->stop)
            return true;
          for (auto& kv : S->sessions)
            if (!kv.second.pending.empty())
              return true;
          return false;
        });
      if (S->stop && flight.empty())
        return;
      for (auto& kv : S->sessions)
      {
        Session& ss = kv.second;
        if (ss.pending.empty())
          continue;
        Request& r = ss.pending.front();
        const int rc = amcl_batch_stage(S->batch, ss.slot, r.n ? r.xyz.data() : nullptr, r.n, 4,
                                        r.nr ? r.ranges.data() : nullptr, r.nr, r.has_odom ? r.odom : nullptr,
                                        r.alpha, r.sigma, r.roll, r.pitch, r.resample);
        InFlight f{ kv.first, ss.slot, r.ticket, r.t_submit, 0 };
        if (rc != AMCL_OK)
        {
          amcl_server_result res{};
          res.ticket = r.ticket;
          res.session = kv.first;
          res.status = rc;
          res.t_submit = r.t_submit;
          res.t_done = now_s();
          S->done.push_back(res);
          ss.pending.pop_front();
          continue;
        }
        f.weights = 0;
        next.push_back(f);
        ss.pending.pop_front();
        ss.in_flight += 1;
      }
    }
    // Wait for the step in flight, read its results, then launch the next one.
    if (!flight.empty())
    {
      const int rc = amcl_batch_wait(S->batch);
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
        if (rc == AMCL_OK && amcl_batch_get_mean(S->batch, f.slot, m7, mv) == AMCL_OK)
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
      const int rc = amcl_batch_step(S->batch);
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

extern "C" int amcl_server_create(amcl_server_t* out, uint32_t max_sessions, uint64_t max_particles,
                                  uint64_t max_points_per_step, void* stream)
{
  if (!out)
    return amcl::fail(AMCL_EINVAL, "amcl_server_create: null out");
  amcl_server_s* S = new amcl_server_s();
  const int rc = amcl_batch_create(&S->batch, max_sessions, max_particles, max_points_per_step, stream);
  if (rc)
  {
    delete S;
    return rc;
  }
  S->worker = std::thread(worker_loop, S);
  *out = S;
  return AMCL_OK;
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
  S->cv.notify_all();
  if (S->worker.joinable())
    S->worker.join();
  amcl_batch_destroy(S->batch);
  delete S;
  return AMCL_OK;
}

extern "C" int amcl_server_open_session(amcl_server_t S, amcl_grid_t grid, uint32_t capacity, uint64_t seed,
                                        int num_particles, const float init8[8], int64_t* session)
{
  if (!S || !grid || !init8 || !session)
    return amcl::fail(AMCL_EINVAL, "amcl_server_open_session: bad arguments");
  std::lock_guard<std::mutex> lock(S->mu);
  int slot = -1;
  int rc = amcl_batch_add(S->batch, grid, capacity, seed, &slot);
  if (rc)
    return rc;  // AMCL_ENOMEM: no room in the arenas (admission refused)
  rc = amcl_batch_init(S->batch, slot, num_particles, init8[0], init8[1], init8[2], init8[3], init8[4], init8[5],
                       init8[6], init8[7]);
  if (rc)
  {
    amcl_batch_remove(S->batch, slot);
    return rc;
  }
  const int64_t id = S->next_session++;
  S->sessions[id].slot = slot;
  *session = id;
  return AMCL_OK;
}

extern "C" int amcl_server_close_session(amcl_server_t S, int64_t session)
{
  if (!S)
    return amcl::fail(AMCL_EINVAL, "amcl_server_close_session: null server");
  // Wait until the session has nothing pending or in flight.
  for (int spins = 0;; ++spins)
  {
    {
      std::lock_guard<std::mutex> lock(S->mu);
      auto it = S->sessions.find(session);
      if (it == S->sessions.end())
        return amcl::fail(AMCL_EINVAL, "amcl_server_close_session: no such session");
      if (it->second.pending.empty() && it->second.in_flight == 0)
      {
        const int rc = amcl_batch_remove(S->batch, it->second.slot);
        S->sessions.erase(it);
        return rc;
      }
    }
    if (spins > 200000)
      return amcl::fail(AMCL_ETIMEDOUT, "amcl_server_close_session: requests still pending");
    std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
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
  {
    std::lock_guard<std::mutex> lock(S->mu);
    auto it = S->sessions.find(session);
    if (it == S->sessions.end())
      return amcl::fail(AMCL_EINVAL, "amcl_server_submit: no such session");
    r.ticket = S->next_ticket++;
    if (ticket)
      *ticket = r.ticket;
    it->second.pending.push_back(std::move(r));
  }
  S->cv.notify_one();
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

extern "C" int amcl_server_batch(amcl_server_t S, amcl_batch_t* batch)
{
  if (!S || !batch)
    return amcl::fail(AMCL_EINVAL, "amcl_server_batch: bad arguments");
  *batch = S->batch;
  return AMCL_OK;
}
