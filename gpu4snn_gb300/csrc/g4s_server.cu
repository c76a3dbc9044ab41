// g4s_server.cu — a simulation server with continuous batching, built on the public C ABI.
//
// Requests (network size, fan-out, steps, seed, drive) are submitted from any thread.  An
// admission thread turns queued requests into device-resident networks (tables generated
// on the GPU, on the network's own stream) while their estimated device bytes fit the
// memory budget; a round thread advances every resident request together in one
// persistent launch of the SKL team kernel (g4s_nets_run): `quantum` steps in its first
// round, then as many as the median resident request runs in `quantum` steps (from the
// measured per-step times), so that the round's teams finish together.  A
// request that has run all its steps leaves at the end of its round: its raster, counts,
// final state and statistics are copied to the host, its device memory is freed, and
// requests admitted meanwhile join the next round.  So arrivals overlap on the GPU with
// the work already there, and a request's results are those of the same network run
// alone (the arithmetic is per network and order independent).  The networks' device
// memory comes from the server's own stream-ordered pool, which keeps what a finished
// request frees for the next ones until the server stops: cudaFree of a network's ~20
// buffers took ~1.3 ms of the round thread's time per finished request (the driver
// unmapping them), a stream-ordered free into the pool a few microseconds.  (Retiring
// finished requests on a thread of their own was measured slower: its copies and frees
// slowed the admission thread's network creation 2-3x, so fewer requests were resident.)
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/gpu4snn.h"
#include "g4s_internal.h"

using namespace g4s;
using Clock = std::chrono::steady_clock;

namespace {

struct Request {
  int64_t id = 0;
  g4s_request req{};
  g4s_net *net = nullptr;
  int64_t est_bytes = 0;
  int32_t remaining = 0;
  double step_ms = 0.0;  // measured per-step time in the last round (0: not yet run)
  // accounting of the request's device use: creation, device time of its steps in the
  // rounds and the same times the CTAs of its team, rounds, last team size
  double create_ms = 0.0, device_ms = 0.0, sm_ms = 0.0;
  int32_t rounds = 0, team = 0;
  Clock::time_point t_submit, t_admit, t_done;
  // results, on the host once the request is done
  int status = 0;
  std::vector<int32_t> rt, rid, counts;
  std::vector<float> v, u;
  std::vector<int32_t> nospks;
  int64_t spikes = 0;
  double rate_hz = 0, isi_cv = 0;
};

// most steps a request without a recorded raster advances in one round (its chunk length)
constexpr int64_t kRoundMaxSteps = 16384;

int64_t estimate_bytes(const g4s_request &r, int32_t quantum) {
  const int64_t stride = ((int64_t)r.nsyn + 3) / 4 * 4;
  const int64_t raster = r.record_raster ? 4 * r.n * (int64_t)quantum : ((int64_t)64 << 20);
  // tables (and their interleaved copy), neuron state and statistics, spike lists, the
  // segment table at the largest team (a small batch spreads a network over the GPU),
  // raster, per-step arrays
  return r.n * stride * 16 + r.n * (8 + 16 + 4 + 8 + 4 + 32 + 32 + 4) + r.n * (kMaxTeam + 1) * 2 + raster +
         16384 * 28 + ((int64_t)1 << 20);
}

}  // namespace

struct g4s_server {
  int device = 0;
  cudaMemPool_t pool = nullptr;  // device memory of the requests' networks
  int64_t budget = 0;
  int32_t quantum = 0;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<std::unique_ptr<Request>> queued;    // submitted, not admitted
  std::deque<std::unique_ptr<Request>> admitted;  // on the device, not yet in a round
  std::map<int64_t, std::unique_ptr<Request>> done;
  std::vector<int64_t> done_unpolled;
  int64_t next_id = 1;
  int64_t bytes_in_use = 0, peak_bytes = 0;
  bool stopping = false;
  std::thread admit_thread, round_thread;
  // statistics
  std::atomic<int64_t> rounds{0}, completed{0}, events{0}, launches{0};
  double busy_ms = 0.0;
  Clock::time_point t_start;
};

static void finish_request(g4s_server *s, Request *r) {
  g4s_net *n = r->net;
  int64_t sz = 0;
  if (r->status == 0 && g4s_net_raster(n, nullptr, nullptr, 0, &sz) == 0) {
    r->rt.resize((size_t)sz);
    r->rid.resize((size_t)sz);
    if (sz) g4s_net_raster(n, r->rt.data(), r->rid.data(), sz, &sz);
  }
  int64_t nc = 0;
  if (r->status == 0 && g4s_net_counts(n, nullptr, 0, &nc) == 0) {
    r->counts.resize((size_t)nc);
    if (nc) g4s_net_counts(n, r->counts.data(), nc, &nc);
  }
  if (r->status == 0) {
    r->v.resize((size_t)r->req.n);
    r->u.resize((size_t)r->req.n);
    r->nospks.resize((size_t)r->req.n);
    g4s_net_state(n, r->v.data(), r->u.data(), nullptr, nullptr, nullptr, nullptr, nullptr, r->nospks.data());
    g4s_net_stats(n, &r->rate_hz, &r->isi_cv, &r->spikes);
  }
  g4s_net_destroy(n);
  r->net = nullptr;
  r->t_done = Clock::now();
}

// Admission: queued requests become device-resident networks while they fit the budget.
static void admit_loop(g4s_server *s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    s->cv.wait(lk, [&] {
      return s->stopping || (!s->queued.empty() && s->bytes_in_use + s->queued.front()->est_bytes <= s->budget);
    });
    if (s->stopping) return;
    std::unique_ptr<Request> r = std::move(s->queued.front());
    s->queued.pop_front();
    s->bytes_in_use += r->est_bytes;
    s->peak_bytes = std::max(s->peak_bytes, s->bytes_in_use);
    lk.unlock();
    g4s_net_desc d{};
    d.n = r->req.n;
    d.nsyn = r->req.nsyn;
    d.exc_permille = 800;
    d.self_loops = 0;
    d.conn_law = G4S_CONN_PHILOX;
    d.seed = r->req.seed;
    d.drive_scale = r->req.drive_scale;
    d.record_raster = r->req.record_raster;
    d.raster_budget_bytes = r->req.record_raster ? 4 * r->req.n * (int64_t)s->quantum : 0;
    const Clock::time_point t_create = Clock::now();
    int rc = net_create_pooled(&d, s->pool, &r->net);
    // (the team kernel's rows and lists here, off the round thread)
    if (rc == 0 && (rc = net_prepare_rows(r->net)) != 0) {
      g4s_net_destroy(r->net);
      r->net = nullptr;
    }
    r->t_admit = Clock::now();
    r->create_ms = std::chrono::duration<double, std::milli>(r->t_admit - t_create).count();
    lk.lock();
    if (rc != 0) {
      r->status = rc;
      r->net = nullptr;
      r->t_done = r->t_admit;
      s->bytes_in_use -= r->est_bytes;
      s->done_unpolled.push_back(r->id);
      s->done[r->id] = std::move(r);
      s->completed++;
    } else {
      s->admitted.push_back(std::move(r));
    }
    s->cv.notify_all();
  }
}

// Rounds: every resident request advances by up to `quantum` steps in one launch.
static void round_loop(g4s_server *s) {
  cudaSetDevice(s->device);
  std::vector<std::unique_ptr<Request>> active;
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv.wait(lk, [&] { return s->stopping || !s->admitted.empty() || !active.empty(); });
      if (s->stopping && active.empty()) return;
      while (!s->admitted.empty()) {
        active.push_back(std::move(s->admitted.front()));
        s->admitted.pop_front();
      }
    }
    // Time-balanced rounds: a request that has run before advances by as many steps as
    // the median measured request does in `quantum` steps, so that the teams of a round
    // finish together instead of the fast ones idling while the slowest runs its quantum
    // (capped by the request's chunk: the quantum when its raster is recorded).
    std::vector<double> seen;
    for (auto &r : active)
      if (r->step_ms > 0.0) seen.push_back(r->step_ms);
    double target_ms = 0.0;
    if (!seen.empty()) {
      std::nth_element(seen.begin(), seen.begin() + seen.size() / 2, seen.end());
      target_ms = seen[seen.size() / 2] * s->quantum;
    }
    std::vector<g4s_net *> nets;
    std::vector<int32_t> steps;
    for (auto &r : active) {
      nets.push_back(r->net);
      int64_t st = s->quantum;
      if (r->step_ms > 0.0 && target_ms > 0.0) {
        const int64_t cap = r->req.record_raster ? s->quantum : kRoundMaxSteps;
        st = std::max<int64_t>(1, std::min<int64_t>(cap, (int64_t)(target_ms / r->step_ms)));
      }
      steps.push_back((int32_t)std::min<int64_t>(r->remaining, st));
    }
    double ms = 0.0;
    int64_t nl = 0;
    const int rc = g4s_nets_run(nets.data(), steps.data(), (int32_t)nets.size(), &ms, &nl);
    s->rounds++;
    s->launches += nl;
    std::vector<std::unique_ptr<Request>> still;
    int64_t ev = 0;
    for (size_t i = 0; i < active.size(); ++i) {
      Request *r = active[i].get();
      if (rc != 0) r->status = rc;
      g4s_net_info inf{};
      if (rc == 0 && g4s_net_get_info(r->net, &inf) == 0) ev += inf.last_run_spikes * (int64_t)r->req.nsyn;
      if (rc == 0 && steps[i] > 0) {
        r->step_ms = net_recent_step_ms(r->net, steps[i]);
        r->team = net_team_size(r->net);  // (the batch's team, read without re-planning)
        r->device_ms += r->step_ms * steps[i];
        r->sm_ms += r->step_ms * steps[i] * r->team;
        r->rounds += 1;
      }
      r->remaining -= steps[i];
      if (r->remaining <= 0 || rc != 0) {
        finish_request(s, r);
        std::lock_guard<std::mutex> lk(s->mu);
        s->bytes_in_use -= r->est_bytes;
        s->done_unpolled.push_back(r->id);
        s->done[r->id] = std::move(active[i]);
        s->completed++;
        s->cv.notify_all();
      } else {
        still.push_back(std::move(active[i]));
      }
    }
    s->events += ev;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->busy_ms += ms;
    }
    active.swap(still);
  }
}

extern "C" {

int g4s_server_start(int64_t hbm_budget_bytes, int32_t quantum_steps, g4s_server **out) {
  if (!out) return set_error(G4S_ERR_INVALID, "null output handle");
  *out = nullptr;
  if (hbm_budget_bytes <= 0 || quantum_steps < 1) return set_error(G4S_ERR_INVALID, "budget and quantum must be > 0");
  g4s_server *s = new (std::nothrow) g4s_server;
  if (!s) return set_error(G4S_ERR_NOMEM, "host allocation");
  cudaError_t e = cudaGetDevice(&s->device);
  if (e != cudaSuccess) {
    delete s;
    return cuda_error(e, "cudaGetDevice");
  }
  cudaMemPoolProps props{};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = s->device;
  e = cudaMemPoolCreate(&s->pool, &props);
  uint64_t keep = UINT64_MAX;  // never return freed memory to the driver while the server runs
  if (e == cudaSuccess) e = cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
  if (e != cudaSuccess) {
    if (s->pool) cudaMemPoolDestroy(s->pool);
    delete s;
    return cuda_error(e, "server memory pool");
  }
  s->budget = hbm_budget_bytes;
  s->quantum = quantum_steps;
  s->t_start = Clock::now();
  s->admit_thread = std::thread(admit_loop, s);
  s->round_thread = std::thread(round_loop, s);
  *out = s;
  return G4S_OK;
}

int g4s_server_submit(g4s_server *s, const g4s_request *req, int64_t *id_out) {
  if (!s || !req) return set_error(G4S_ERR_INVALID, "null argument");
  const int64_t maxsyn = req->n - 1;
  if (req->n < 2 || req->n > (int64_t)INT32_MAX || req->nsyn < 1 || req->nsyn > maxsyn || req->nsyn > kMaxSortedNsyn ||
      req->steps < 0 || !(req->drive_scale >= 0.0f))
    return set_error(G4S_ERR_INVALID, "malformed request");
  auto r = std::make_unique<Request>();
  r->req = *req;
  r->remaining = req->steps;
  r->est_bytes = estimate_bytes(*req, s->quantum);
  r->t_submit = Clock::now();
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stopping) return set_error(G4S_ERR_STATE, "server is stopping");
  if (r->est_bytes > s->budget)
    return set_error(G4S_ERR_BUDGET, "request needs " + std::to_string(r->est_bytes) + " bytes, budget is " +
                                         std::to_string(s->budget));
  r->id = s->next_id++;
  if (id_out) *id_out = r->id;
  s->queued.push_back(std::move(r));
  s->cv.notify_all();
  return G4S_OK;
}

int g4s_server_poll(g4s_server *s, g4s_request_result *out, int32_t cap, int32_t *n_out) {
  if (!s || !n_out || (cap > 0 && !out)) return set_error(G4S_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  int32_t k = 0;
  while (k < cap && !s->done_unpolled.empty()) {
    const int64_t id = s->done_unpolled.front();
    s->done_unpolled.erase(s->done_unpolled.begin());
    const Request *r = s->done[id].get();
    g4s_request_result &o = out[k++];
    o.id = r->id;
    o.status = r->status;
    o.steps_done = r->req.steps - std::max(r->remaining, 0);
    o.total_spikes = (int64_t)r->rt.size() > 0 ? (int64_t)r->rt.size() : r->spikes;
    o.latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
    o.queue_ms = std::chrono::duration<double, std::milli>(r->t_admit - r->t_submit).count();
    o.rate_hz = r->rate_hz;
    o.isi_cv = r->isi_cv;
    o.create_ms = r->create_ms;
    o.device_ms = r->device_ms;
    o.sm_ms = r->sm_ms;
    o.rounds = r->rounds;
    o.team = r->team;
  }
  *n_out = k;
  return G4S_OK;
}

int g4s_server_result(g4s_server *s, int64_t id, int32_t *t, int32_t *ids, int64_t cap, int64_t *n, float *v, float *u,
                      int32_t *nospks) {
  if (!s) return set_error(G4S_ERR_INVALID, "null handle");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->done.find(id);
  if (it == s->done.end()) return set_error(G4S_ERR_STATE, "request " + std::to_string(id) + " is not done");
  const Request *r = it->second.get();
  if (r->status != 0) return set_error(r->status, "request failed");
  const int64_t sz = (int64_t)r->rt.size();
  if (n) *n = sz;
  const int64_t m = std::min(sz, cap);
  if (m > 0) {
    if (!t || !ids) return set_error(G4S_ERR_INVALID, "null raster buffer");
    memcpy(t, r->rt.data(), (size_t)m * 4);
    memcpy(ids, r->rid.data(), (size_t)m * 4);
  }
  if (v) memcpy(v, r->v.data(), r->v.size() * 4);
  if (u) memcpy(u, r->u.data(), r->u.size() * 4);
  if (nospks) memcpy(nospks, r->nospks.data(), r->nospks.size() * 4);
  return G4S_OK;
}

int g4s_server_release(g4s_server *s, int64_t id) {
  if (!s) return set_error(G4S_ERR_INVALID, "null handle");
  std::lock_guard<std::mutex> lk(s->mu);
  if (!s->done.erase(id)) return set_error(G4S_ERR_STATE, "request " + std::to_string(id) + " is not done");
  return G4S_OK;
}

int g4s_server_get_stats(g4s_server *s, g4s_server_stats *out) {
  if (!s || !out) return set_error(G4S_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  out->rounds = s->rounds;
  out->launches = s->launches;
  out->completed = s->completed;
  out->queued = (int64_t)s->queued.size();
  out->resident = (int64_t)s->admitted.size();
  out->events = s->events;
  out->busy_ms = s->busy_ms;
  out->wall_ms = std::chrono::duration<double, std::milli>(Clock::now() - s->t_start).count();
  out->bytes_in_use = s->bytes_in_use;
  out->peak_bytes = s->peak_bytes;
  return G4S_OK;
}

int g4s_server_stop(g4s_server *s, int32_t drain) {
  if (!s) return set_error(G4S_ERR_INVALID, "null handle");
  if (drain) {
    // wait until every submitted request is done
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv.wait(lk, [&] { return s->completed >= s->next_id - 1; });
  }
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stopping = true;
    s->cv.notify_all();
  }
  s->admit_thread.join();
  s->round_thread.join();
  for (auto &r : s->admitted)
    if (r->net) g4s_net_destroy(r->net);
  // (every network of the pool is destroyed: its memory goes back to the driver)
  cudaMemPoolDestroy(s->pool);
  delete s;
  return G4S_OK;
}

}  // extern "C"
