// g4s_api.cu — the C ABI (include/gpu4snn.h): network handles, the chunked step loop, the
// reference's result files and its experiment sweep.
//
// A run is executed in chunks of at most `chunk_steps` steps; a chunk's spike ids go to a
// device raster buffer sized so that every neuron could fire at every step of the chunk,
// so it can never overflow.  After each chunk the per-step counts, raster offsets and
// globaltimer stamps come back to the host (and the raster, when it is recorded).
#include <cuda_runtime.h>
#include <sys/stat.h>

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <cmath>
#include <map>
#include <memory>
#include <mutex>
#include <tuple>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/gpu4snn.h"
#include "g4s_internal.h"

using namespace g4s;

// ---------------------------------------------------------------------------------------
// Errors.
// ---------------------------------------------------------------------------------------
static thread_local std::string g_last_error;

namespace g4s {
int set_error(int code, const std::string &msg) {
  g_last_error = msg;
  return code;
}
int cuda_error(cudaError_t e, const char *what) {
  return set_error(e == cudaErrorMemoryAllocation ? G4S_ERR_NOMEM : G4S_ERR_CUDA,
                   std::string(what) + ": " + cudaGetErrorString(e));
}
}  // namespace g4s

#define G4S_CUDA(call)                                  \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cuda_error(e_, #call); \
  } while (0)

struct TeamLaunch {
  TeamItem *d_items = nullptr, *h_items = nullptr;
  int2 *d_slots = nullptr, *h_slots = nullptr;
  int *d_ctl = nullptr, *h_ctl = nullptr;  // [0] slot count, [1] queue head
  int *h_status = nullptr;                 // per item: status word, team error word
  int64_t *d_off = nullptr, *h_off = nullptr;  // per item: its share of the pack (many networks)
  unsigned char *d_pack = nullptr, *h_pack = nullptr;
  size_t cap_pack = 0;
  int cap_items = 0, cap_slots = 0;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  // the round as a CUDA graph, replayed while its shape (networks, teams, buffers) holds
  cudaGraphExec_t exec = nullptr;
  std::vector<uint64_t> sig;
  std::vector<int> order;  // networks of the round in flight (team_round_start .. finish)
  // a round of many networks, launched directly: its networks and steps, read back by pack
  bool direct = false;
  std::vector<g4s_net *> nets;
  std::vector<int> steps;
  TeamLaunch() = default;
  TeamLaunch(const TeamLaunch &) = delete;
  TeamLaunch &operator=(const TeamLaunch &) = delete;
  ~TeamLaunch() { release(); }  // (a thread's own launch buffers go when the thread ends)
  void drop_graph() {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
    sig.clear();
  }
  void release() {
    drop_graph();
    cudaFree(d_items);
    cudaFree(d_slots);
    cudaFree(d_ctl);
    cudaFreeHost(h_items);
    cudaFreeHost(h_slots);
    cudaFreeHost(h_ctl);
    cudaFreeHost(h_status);
    cudaFree(d_off);
    cudaFreeHost(h_off);
    cudaFree(d_pack);
    cudaFreeHost(h_pack);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    d_items = h_items = nullptr;
    d_slots = h_slots = nullptr;
    d_ctl = h_ctl = nullptr;
    h_status = nullptr;
    d_off = h_off = nullptr;
    d_pack = h_pack = nullptr;
    cap_pack = 0;
    cap_items = cap_slots = 0;
    e0 = e1 = nullptr;
    order.clear();
    direct = false;
  }
  int reserve(int items, int slots) {
    if (!e0 && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess))
      return set_error(G4S_ERR_CUDA, "team launch events");
    if (!d_ctl && (cudaMalloc((void **)&d_ctl, 16) != cudaSuccess || cudaMallocHost((void **)&h_ctl, 16) != cudaSuccess))
      return set_error(G4S_ERR_NOMEM, "team launch control words");
    if (items > cap_items) {
      drop_graph();
      cudaFree(d_items);
      cudaFreeHost(h_items);
      cudaFreeHost(h_status);
      cudaFree(d_off);
      cudaFreeHost(h_off);
      d_items = h_items = nullptr;
      h_status = nullptr;
      d_off = h_off = nullptr;
      cap_items = 0;  // (until the new buffers exist)
      if (cudaMalloc((void **)&d_items, sizeof(TeamItem) * items) != cudaSuccess ||
          cudaMallocHost((void **)&h_items, sizeof(TeamItem) * items) != cudaSuccess ||
          cudaMallocHost((void **)&h_status, sizeof(int) * 2 * items) != cudaSuccess ||
          cudaMalloc((void **)&d_off, sizeof(int64_t) * items) != cudaSuccess ||
          cudaMallocHost((void **)&h_off, sizeof(int64_t) * items) != cudaSuccess)
        return set_error(G4S_ERR_NOMEM, "team items");
      cap_items = items;
    }
    if (slots > cap_slots) {
      drop_graph();
      cudaFree(d_slots);
      cudaFreeHost(h_slots);
      d_slots = h_slots = nullptr;
      cap_slots = 0;
      if (cudaMalloc((void **)&d_slots, sizeof(int2) * slots) != cudaSuccess ||
          cudaMallocHost((void **)&h_slots, sizeof(int2) * slots) != cudaSuccess)
        return set_error(G4S_ERR_NOMEM, "team slots");
      cap_slots = slots;
    }
    return G4S_OK;
  }
  int reserve_pack(size_t bytes) {
    if (bytes <= cap_pack) return G4S_OK;
    bytes = std::max(bytes, 2 * cap_pack);
    cudaFree(d_pack);
    cudaFreeHost(h_pack);
    d_pack = h_pack = nullptr;
    cap_pack = 0;
    if (cudaMalloc((void **)&d_pack, bytes) != cudaSuccess || cudaMallocHost((void **)&h_pack, bytes) != cudaSuccess)
      return set_error(G4S_ERR_NOMEM, "team round read-back buffer");
    cap_pack = bytes;
    return G4S_OK;
  }
};

// A scheme and, for SKL, a team size chosen by the autotuner (0 = the default team).
struct TuneChoice {
  int alg = kAlgSKL;
  int team = 0;
  int mode = kDeliverAuto;
  int nt = 0;  // threads per CTA of the team kernel (0: chosen from the step size)
};

// ---------------------------------------------------------------------------------------
// Handle.
// ---------------------------------------------------------------------------------------
struct g4s_net {
  g4s_net_desc desc{};
  NetView v{};
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, ek0 = nullptr, ek1 = nullptr;
  double last_kernel_ms = 0;
  int64_t last_launches = 0;
  GridSync *gs = nullptr;
  double *d_stats = nullptr;
  int64_t chunk_steps = 0;   // steps per chunk of the team kernel
  int64_t chunk_legacy = 0;  // steps per chunk of the other kernels (raster = spike list)
  // chunks of the host-driven schemes as CUDA graphs: the chunk's first step (device word,
  // set from pinned memory at each replay) and up to kStepGraphs captured chunks, keyed by
  // scheme, length, last-chunk flag and launch shape
  long long *d_t0 = nullptr, *h_t0 = nullptr;
  struct StepGraph {
    std::vector<uint64_t> key;
    cudaGraphExec_t exec = nullptr;
  };
  std::vector<StepGraph> step_graphs;
  int64_t t_abs = 0;
  uint32_t tag_next = 0;  // record tags of the team kernel: never repeated for this handle's lists
  uint64_t serial = 0;    // creation number, unique in the process (keys the captured rounds)
  unsigned long long barrier_ns = 2000000000ull;
  size_t device_bytes = 0;
  // pinned staging of one chunk
  int *h_counts = nullptr;
  long long *h_base = nullptr;
  unsigned long long *h_stamps = nullptr;
  int *h_raster = nullptr;
  // host results since the last reset
  std::vector<int32_t> rt, rid, counts;
  std::vector<float> upd_ms, step_ms;
  int64_t total_spikes = 0;
  double last_ms = 0, last_wall_ms = 0;
  int64_t last_spikes = 0;
  int last_alg = -1;
  DeliverShape shape;
  int barrier_stall = 0;  // injected: extra arrivals the next SKL launch waits for
  // SKL team kernel: team size and slice, per-step spike lists, per-row segment table,
  // requested team size (0 = auto), whether the tables satisfy the exactness bound of the
  // split accumulation, and the launch buffers of the handle's own runs
  int team_p = 0;
  int64_t team_rc = 0;
  bool team_ready = false;
  bool team_batch = false;  // geometry planned for a multi-network batch
  int64_t team_slice = 0;   // ... with this many neurons per CTA
  bool team_ok = true;
  bool pair_ready = false;  // the interleaved rows match the tables
  unsigned long long *list = nullptr;
  uint16_t *seg = nullptr;
  size_t seg_bytes = 0;
  // device memory from this stream-ordered pool (a server's, which keeps freed memory for
  // the next requests' networks), allocated and freed on the handle's stream; null: cudaMalloc
  cudaMemPool_t pool = nullptr;
  int want_p = 0;
  int deliver_mode = kDeliverAuto;
  int team_nt = 0;            // threads per CTA asked for: kTeamNT, kTeamNTSmall, 0 = automatic
  int team_nt_eff = kTeamNT;  // ... in use (set when the team is planned)
  bool tables_fit = false;
  unsigned long long max_in = 0, max_mag = 0;
  TeamLaunch launch;
  // autotuner: this handle's measured choice
  bool tuned = false;
  TuneChoice tune;
  // raster streamed to a binary file (while set, the raster is not kept in host memory)
  RasterFile *rstream = nullptr;
};

static std::atomic<int> g_fail_next_alloc{0};

static cudaError_t net_malloc(g4s_net *n, void **p, size_t bytes) {
  if (n->pool) return cudaMallocFromPoolAsync(p, bytes, n->pool, n->stream);
  return cudaMalloc(p, bytes);
}
static void net_free(g4s_net *n, const void *p) {
  if (!p) return;
  if (n->pool)
    cudaFreeAsync(const_cast<void *>(p), n->stream);
  else
    cudaFree(const_cast<void *>(p));
}

static void free_net(g4s_net *n) {
  if (!n) return;
  NetView &v = n->v;
  if (n->rstream) {
    raster_close(n->rstream);
    n->rstream = nullptr;
  }
  n->launch.release();  // its captured round refers to the buffers below
  for (auto &gr : n->step_graphs)  // (and so do the captured chunks)
    if (gr.exec) cudaGraphExecDestroy(gr.exec);
  n->step_graphs.clear();
  net_free(n, n->d_t0);
  cudaFreeHost(n->h_t0);
  net_free(n, const_cast<int2 *>(v.pair));
  net_free(n, v.vu);
  net_free(n, v.abcd);
  net_free(n, v.rpar);
  net_free(n, v.acc);
  net_free(n, v.ilast);
  net_free(n, v.sstat);
  net_free(n, const_cast<int *>(v.idx));
  net_free(n, const_cast<float *>(v.w));
  net_free(n, v.raster);
  net_free(n, v.counts);
  net_free(n, v.base);
  net_free(n, v.stamps);
  net_free(n, v.status);
  net_free(n, n->gs);
  net_free(n, n->d_stats);
  net_free(n, n->seg);
  net_free(n, n->list);
  cudaFreeHost(n->h_counts);
  cudaFreeHost(n->h_base);
  cudaFreeHost(n->h_stamps);
  cudaFreeHost(n->h_raster);
  if (n->ev0) cudaEventDestroy(n->ev0);
  if (n->ev1) cudaEventDestroy(n->ev1);
  if (n->ek0) cudaEventDestroy(n->ek0);
  if (n->ek1) cudaEventDestroy(n->ek1);
  if (n->stream) cudaStreamDestroy(n->stream);
  delete n;
}

static int64_t row_stride(int32_t nsyn) { return ((int64_t)nsyn + 3) / 4 * 4; }

static int validate(const g4s_net_desc *d) {
  if (!d) return set_error(G4S_ERR_INVALID, "null descriptor");
  if (d->n < 2 || d->n > (int64_t)INT32_MAX) return set_error(G4S_ERR_INVALID, "n must be in [2, 2^31)");
  if (d->nsyn < 1) return set_error(G4S_ERR_INVALID, "nsyn must be >= 1");
  if (d->nsyn > kMaxSortedNsyn) return set_error(G4S_ERR_INVALID, "nsyn must be <= 16384");
  const int64_t maxsyn = d->self_loops ? d->n : d->n - 1;
  if (d->nsyn > maxsyn) return set_error(G4S_ERR_INVALID, "nsyn exceeds the number of possible targets");
  if (d->exc_permille < 0 || d->exc_permille > 1000) return set_error(G4S_ERR_INVALID, "exc_permille must be in [0, 1000]");
  if (d->conn_law != G4S_CONN_PHILOX && d->conn_law != G4S_CONN_GLIBC)
    return set_error(G4S_ERR_INVALID, "unknown connectivity law");
  if (d->conn_law == G4S_CONN_GLIBC && d->n > (int64_t)INT32_MAX / 2)
    return set_error(G4S_ERR_INVALID, "glibc law limited to n < 2^30");
  if (!(d->drive_scale >= 0.0f) || d->drive_scale > 1e6f) return set_error(G4S_ERR_INVALID, "bad drive_scale");
  return G4S_OK;
}

template <class T>
static int dalloc(g4s_net *n, T **p, size_t count, const char *what) {
  const size_t bytes = count * sizeof(T);
  cudaError_t e = g_fail_next_alloc.exchange(0) ? cudaErrorMemoryAllocation : net_malloc(n, (void **)p, bytes ? bytes : 16);
  if (e != cudaSuccess) {
    *p = nullptr;
    return set_error(G4S_ERR_NOMEM, std::string("cudaMalloc of ") + what + " (" + std::to_string(bytes) +
                                        " bytes): " + cudaGetErrorString(e));
  }
  n->device_bytes += bytes;
  return G4S_OK;
}

static void set_drive(g4s_net *n) {
  n->v.ge = 5.0f * n->desc.drive_scale;
  n->v.gi = 2.0f * n->desc.drive_scale;
}

static int alloc_net(const g4s_net_desc *d, g4s_net **out, cudaMemPool_t pool = nullptr) {
  int rc = validate(d);
  if (rc) return rc;
  g4s_net *n = new (std::nothrow) g4s_net;
  if (!n) return set_error(G4S_ERR_NOMEM, "host allocation");
  n->pool = pool;
  static std::atomic<uint64_t> next_serial{1};
  n->serial = next_serial++;
  n->desc = *d;
  NetView &v = n->v;
  v.n = d->n;
  v.nexc = (d->n * (int64_t)d->exc_permille) / 1000;
  v.nsyn = d->nsyn;
  v.stride = (int32_t)row_stride(d->nsyn);
  v.seed = d->seed;
  set_drive(n);
  const size_t N = (size_t)d->n, S = (size_t)v.stride;
  // chunk: a raster buffer that holds every neuron firing at every step of the chunk (the
  // host-driven schemes and the fallback kernel use it as the spike list).  The team
  // kernel keeps its spike lists elsewhere, so when the raster is not recorded its chunk
  // is bounded only by the per-step arrays.
  const int64_t dflt = d->record_raster ? ((int64_t)1 << 30) : ((int64_t)64 << 20);
  int64_t budget = d->raster_budget_bytes > 0 ? d->raster_budget_bytes : dflt;
  int64_t cs = budget / (int64_t)(4 * N);
  if (cs < 1) cs = 1;
  if (cs > 100000) cs = 100000;
  n->chunk_legacy = cs;
  n->chunk_steps = d->record_raster ? cs : 16384;
  v.raster_cap = cs * (int64_t)N;
  cs = std::max<int64_t>(cs, n->chunk_steps);
  size_t free_b = 0, total_b = 0;
  cudaError_t e = cudaMemGetInfo(&free_b, &total_b);
  if (e != cudaSuccess) {
    free_net(n);
    return cuda_error(e, "cudaMemGetInfo");
  }
  if (pool) {  // memory the pool holds for reuse counts as free
    uint64_t reserved = 0, used = 0;
    if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved) == cudaSuccess &&
        cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used) == cudaSuccess && reserved > used)
      free_b += (size_t)(reserved - used);
    (void)cudaGetLastError();
    // (a pool allocates on the handle's stream)
    if ((e = cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking)) != cudaSuccess) {
      free_net(n);
      return cuda_error(e, "stream");
    }
  }
  const size_t need = N * S * 8 + N * (8 + 16 + 4 + 8 + 4 + 32) + (size_t)v.raster_cap * 4 + (size_t)cs * 32;
  if (need + ((size_t)256 << 20) > free_b) {
    free_net(n);
    return set_error(G4S_ERR_NOMEM, "network needs " + std::to_string(need) + " bytes of device memory, " +
                                        std::to_string(free_b) + " free");
  }
  if ((rc = dalloc(n, &v.vu, N, "v,u")) || (rc = dalloc(n, &v.abcd, N, "a,b,c,d")) ||
      (rc = dalloc(n, &v.rpar, N, "parameter r")) ||
      (rc = dalloc(n, &v.acc, N, "currents")) || (rc = dalloc(n, &v.ilast, N, "input current")) ||
      (rc = dalloc(n, &v.sstat, N, "spike statistics")) ||
      (rc = dalloc(n, const_cast<int **>(&v.idx), N * S, "targets")) ||
      (rc = dalloc(n, const_cast<float **>(&v.w), N * S, "weights")) ||
      (rc = dalloc(n, &v.raster, (size_t)v.raster_cap, "raster")) ||
      (rc = dalloc(n, &v.counts, (size_t)cs, "counts")) || (rc = dalloc(n, &v.base, (size_t)cs, "offsets")) ||
      (rc = dalloc(n, &v.stamps, (size_t)cs * 2 + 2, "stamps")) || (rc = dalloc(n, &v.status, 1, "status")) ||
      (rc = dalloc(n, &n->gs, 1 + 2 * (size_t)kMaxTeam * kRecLines, "barrier and spike records")) ||
      (rc = dalloc(n, &n->d_stats, 2, "stats")) || (rc = dalloc(n, &n->d_t0, 1, "chunk start"))) {
    free_net(n);
    return rc;
  }
  if ((!n->stream && (e = cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking)) != cudaSuccess) ||
      (e = cudaEventCreate(&n->ev0)) != cudaSuccess || (e = cudaEventCreate(&n->ev1)) != cudaSuccess ||
      (e = cudaEventCreate(&n->ek0)) != cudaSuccess || (e = cudaEventCreate(&n->ek1)) != cudaSuccess ||
      (e = cudaMallocHost((void **)&n->h_counts, (size_t)cs * 4)) != cudaSuccess ||
      (e = cudaMallocHost((void **)&n->h_base, (size_t)cs * 8)) != cudaSuccess ||
      (e = cudaMallocHost((void **)&n->h_stamps, ((size_t)cs * 2 + 2) * 8)) != cudaSuccess ||
      (e = cudaMallocHost((void **)&n->h_t0, sizeof(long long))) != cudaSuccess) {
    free_net(n);
    return cuda_error(e, "stream/event/pinned allocation");
  }
  if (d->record_raster) {
    e = cudaMallocHost((void **)&n->h_raster, (size_t)v.raster_cap * 4);
    if (e != cudaSuccess) {
      free_net(n);
      return cuda_error(e, "pinned raster staging");
    }
  }
  if ((e = cudaMemsetAsync(v.status, 0, sizeof(int), n->stream)) != cudaSuccess ||
      (e = cudaMemsetAsync(n->gs, 0, sizeof(GridSync), n->stream)) != cudaSuccess) {
    free_net(n);
    return cuda_error(e, "clearing status words");
  }
  *out = n;
  return G4S_OK;
}

static int status_rc(int st, int bar, const char *what);

static int check_status(g4s_net *n, const char *what) {
  int st = 0, bar = 0;
  G4S_CUDA(cudaMemcpyAsync(&st, n->v.status, sizeof(int), cudaMemcpyDeviceToHost, n->stream));
  G4S_CUDA(cudaMemcpyAsync(&bar, &n->gs->error, sizeof(int), cudaMemcpyDeviceToHost, n->stream));
  G4S_CUDA(cudaStreamSynchronize(n->stream));
  return status_rc(st, bar, what);
}

// The device's status word and a team's error word as a G4S status.
static int status_rc(int st, int bar, const char *what) {
  if (bar == kErrTimeoutCode) return set_error(G4S_ERR_TIMEOUT, std::string(what) + ": grid barrier timed out");
  if (st == kErrOverflowCode) return set_error(G4S_ERR_OVERFLOW, std::string(what) + ": raster overflow");
  if (st == kErrConnCode) return set_error(G4S_ERR_INVALID, std::string(what) + ": connectivity draws exhausted");
  if (st != 0 || bar != 0) return set_error(G4S_ERR_CUDA, std::string(what) + ": device error " + std::to_string(st));
  return G4S_OK;
}

static int reset_net(g4s_net *n) {
  NetView &v = n->v;
  if (n->rstream) {  // the step numbering restarts: a streamed raster ends here
    RasterFile *f = n->rstream;
    n->rstream = nullptr;
    int rc = raster_close(f);
    if (rc) return rc;
  }
  set_drive(n);
  G4S_CUDA(cudaMemsetAsync(v.status, 0, sizeof(int), n->stream));
  G4S_CUDA(cudaMemsetAsync(n->gs, 0, sizeof(GridSync), n->stream));
  G4S_CUDA(launch_init(v, n->stream));
  G4S_CUDA(cudaStreamSynchronize(n->stream));
  n->t_abs = 0;
  n->rt.clear();
  n->rid.clear();
  n->counts.clear();
  n->upd_ms.clear();
  n->step_ms.clear();
  n->total_spikes = 0;
  return G4S_OK;
}

static int prepare_rows(g4s_net *n);  // (defined with the team set-up below)

// ---------------------------------------------------------------------------------------
// Host generator of the reference's tables (glibc rand).  The k-th remaining target of a
// row is found by a binary search over the sorted list of targets already taken, which
// gives the reference's list-and-memmove result (gpu4snn.cu:880-898) in O(nsyn log nsyn)
// per synapse instead of O(n).
// ---------------------------------------------------------------------------------------
namespace g4s {
int conn_glibc_host(unsigned seed, int32_t n, int32_t nsyn, int32_t stride, int32_t *idx, float *w) {
  if (n < 1 || nsyn < 0 || nsyn > n || stride < nsyn) return set_error(G4S_ERR_INVALID, "bad glibc table request");
  const int32_t nexc = (int32_t)(((int64_t)n * 4) / 5);
  const float wscale = 1000.0f / (float)nsyn;
  std::vector<int32_t> taken;
  taken.reserve((size_t)nsyn);
  srand(seed);
  for (int32_t i = 0; i < n; ++i) {
    taken.clear();
    int32_t *ri = idx + (int64_t)i * stride;
    float *rw = w + (int64_t)i * stride;
    for (int32_t j = 0; j < nsyn; ++j) {
      const int32_t size = n - j;
      const int32_t k = (int32_t)((size_t)rand() % (size_t)size);
      float x = i < nexc ? wscale * 0.5f : wscale * -1.0f;
      x = x * (float)rand();
      x = x / (float)RAND_MAX;
      int32_t lo = k, hi = k + (int32_t)taken.size();
      while (lo < hi) {
        const int32_t mid = lo + (hi - lo) / 2;
        const int32_t le = (int32_t)(std::upper_bound(taken.begin(), taken.end(), mid) - taken.begin());
        if (mid + 1 - le >= k + 1)
          hi = mid;
        else
          lo = mid + 1;
      }
      taken.insert(std::upper_bound(taken.begin(), taken.end(), lo), lo);
      ri[j] = lo;
      rw[j] = x;
    }
    for (int32_t j = nsyn; j < stride; ++j) {
      ri[j] = -1;
      rw[j] = 0.0f;
    }
  }
  return G4S_OK;
}

int net_prepare_rows(g4s_net *n) { return n && n->tables_fit ? prepare_rows(n) : G4S_OK; }

double net_recent_step_ms(const g4s_net *n, int64_t k) {
  double sum = 0.0;
  int64_t used = 0;
  for (int64_t i = (int64_t)n->step_ms.size() - 1; i >= 0 && k > 0; --i, --k)
    if (n->step_ms[(size_t)i] > 0.0f) {  // (the last step of a launch has no successor stamp)
      sum += n->step_ms[(size_t)i];
      ++used;
    }
  return used ? sum / (double)used : 0.0;
}

const NetView &net_view(const g4s_net *n) { return n->v; }
cudaStream_t net_stream(const g4s_net *n) { return n->stream; }
int64_t net_steps_done(const g4s_net *n) { return n->t_abs; }
int net_team_size(const g4s_net *n) { return n->team_ready && n->team_ok && n->team_p > 0 ? n->team_p : 1; }

}  // namespace g4s

// ---------------------------------------------------------------------------------------
// Step loop.
// ---------------------------------------------------------------------------------------
// ---------------------------------------------------------------------------------------
// Autotuner.  Choices are cached process-wide by (log2 N, log2 Nsyn, log2 firing rate):
// a scheme and, for SKL, the team size.  g4s_net_autotune measures the candidates on the
// handle itself from a device snapshot of its state, restored afterwards, so tuning does
// not change the simulation.  ALG_AUTO uses the handle's own choice, else the cached one
// for its key (with the rate of its last run), else SKL with the default team.
// ---------------------------------------------------------------------------------------
static std::mutex g_tune_mu;
static std::map<std::tuple<int, int, int>, TuneChoice> g_tune_cache;

static int ilog2(double x) { return x < 1.0 ? 0 : (int)std::floor(std::log2(x)); }

static std::tuple<int, int, int> tune_key(const g4s_net *n, double rate_hz) {
  return std::make_tuple(ilog2((double)n->v.n), ilog2((double)n->v.nsyn), ilog2(rate_hz + 1.0));
}

static double recent_rate(const g4s_net *n) {
  const size_t k = std::min<size_t>(n->counts.size(), 200);
  if (!k) return 8.0;  // no history: assume the balanced regime
  double s = 0;
  for (size_t i = n->counts.size() - k; i < n->counts.size(); ++i) s += n->counts[i];
  return s / (double)k / (double)n->v.n * 1000.0;
}

static int resolve_alg(g4s_net *n, int alg) {
  if (alg != kAlgAuto) return alg;
  n->shape = DeliverShape{};
  n->shape.group = 0;
  TuneChoice c;
  if (n->tuned) {
    c = n->tune;
  } else {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_cache.find(tune_key(n, recent_rate(n)));
    if (it != g_tune_cache.end()) c = it->second;
  }
  if (c.alg == kAlgSKL && c.team != n->want_p && n->want_p == 0 && c.team > 0) {
    n->want_p = c.team;
    n->team_ready = false;
    n->team_ok = true;
  }
  if (c.alg == kAlgSKL) {
    n->deliver_mode = c.mode;
    if (n->team_nt != c.nt) {
      n->team_nt = c.nt;
      n->team_ready = false;
    }
  }
  return c.alg;
}

// ---------------------------------------------------------------------------------------
// Team geometry of one network for the SKL team kernel: p CTAs (at most the co-resident
// count, one per SM), by default one per 128 neurons alone and one per 8192 in a batch,
// and the currents plus the spike buffer of a slice within the shared-memory limit.
// Returns false if the network does not fit or its tables break the exactness bound of
// the split accumulation (the global-atomic persistent kernel is used instead).
// ---------------------------------------------------------------------------------------
static bool plan_team(g4s_net *n, int want, bool batch, int64_t slice, int *p_out, int64_t *rc_out) {
  const NetView &v = n->v;
  if (!n->tables_fit) return false;
  int pmax = 0;
  // (both CTA sizes fit one CTA per SM: planned with the default)
  if (team_max_blocks(kTeamSmemLimit, &pmax) != cudaSuccess || pmax < 1) {
    (void)cudaGetLastError();
    return false;
  }
  pmax = std::min(pmax, kMaxTeam);
  // alone, a network spreads over the GPU (one CTA per 128 neurons, up to one per SM); in a
  // batch it takes one CTA per `slice` neurons (8192 unless the batch is small), so that more
  // networks run at once
  int64_t p = want > 0 ? want : (batch ? (v.n + slice - 1) / slice : (v.n + kSoloSlice - 1) / kSoloSlice);
  if (p < 1) p = 1;
  if (p > pmax) p = pmax;
  int64_t rc = (v.n + p - 1) / p;
  if (team_smem(rc, (int)p) == 0) {
    rc = (v.n + pmax - 1) / pmax;
    p = (v.n + rc - 1) / rc;
    if (team_smem(rc, (int)p) == 0) return false;
  }
  int pfit = 0;
  if (team_max_blocks(team_smem(rc, (int)p), &pfit) != cudaSuccess || pfit < p) {
    (void)cudaGetLastError();
    return false;
  }
  *p_out = (int)p;
  *rc_out = rc;
  return true;
}

// The team kernel's buffers that do not depend on the team: the interleaved rows of its
// segment reads (optional: without them, as when the device has no room left for them, the
// kernel reads the separate arrays) and the tagged spike lists.  Both are ready on return
// (a batch may launch on another handle's stream).
static int prepare_rows(g4s_net *n) {
  if (!n->v.pair) {
    const size_t bytes = (size_t)n->v.n * (size_t)n->v.stride * sizeof(int2);
    if (!g_fail_next_alloc.exchange(0) && net_malloc(n, (void **)&n->v.pair, bytes) == cudaSuccess) {
      n->device_bytes += bytes;
      n->pair_ready = false;
    } else {
      (void)cudaGetLastError();
      n->v.pair = nullptr;
    }
  }
  if (n->v.pair && !n->pair_ready) {
    G4S_CUDA(launch_pairs(n->v, n->stream));
    G4S_CUDA(cudaStreamSynchronize(n->stream));
    n->pair_ready = true;
  }
  if (!n->list) {
    cudaError_t e = net_malloc(n, (void **)&n->list, (size_t)n->v.n * 4 * sizeof(unsigned long long));
    if (e != cudaSuccess) return cuda_error(e, "spike lists");
    G4S_CUDA(cudaMemsetAsync(n->list, 0, (size_t)n->v.n * 4 * sizeof(unsigned long long), n->stream));
    G4S_CUDA(cudaStreamSynchronize(n->stream));
    n->tag_next = 0;
    n->device_bytes += (size_t)n->v.n * 4 * sizeof(unsigned long long);
  }
  return G4S_OK;
}

// Team geometry, the per-step spike lists and, for teams of more than one CTA, the
// per-row segment table.
static int prepare_team(g4s_net *n, bool batch = false, int64_t slice = kBatchSlice) {
  if (n->team_ready && n->team_batch == batch && (!batch || n->team_slice == slice)) return G4S_OK;
  int p = 0;
  int64_t rc = 0;
  n->team_batch = batch;
  n->team_slice = slice;
  if (!plan_team(n, n->want_p, batch, slice, &p, &rc)) {
    n->team_ok = false;
    return G4S_OK;
  }
  // CTA size: the one asked for; automatically 768 threads when a rank's expected share of
  // a step is small (fewer than 32768 synapses, from the recent firing rate), where the
  // spill-free kernel's shorter chain wins, else 1024 (more reads in flight); a batch takes
  // 1024 (measured faster for ensembles of small networks)
  if (n->team_nt) {
    n->team_nt_eff = n->team_nt;
  } else {
    const double syn = (double)n->v.n * recent_rate(n) / 1000.0 * (double)n->v.nsyn / (double)p;
    n->team_nt_eff = !batch && syn < 32768.0 ? kTeamNTSmall : kTeamNT;
  }
  int rc0 = prepare_rows(n);
  if (rc0) return rc0;
  if (p > 1) {
    const size_t bytes = (size_t)n->v.n * (size_t)(p + 1) * sizeof(uint16_t);
    if (bytes > n->seg_bytes) {
      net_free(n, n->seg);
      n->seg = nullptr;
      n->device_bytes -= n->seg_bytes;
      n->seg_bytes = 0;
      cudaError_t e = net_malloc(n, (void **)&n->seg, bytes);
      if (e != cudaSuccess) return cuda_error(e, "segment table");
      n->seg_bytes = bytes;
      n->device_bytes += bytes;
    }
    G4S_CUDA(launch_segoff(n->v, p, rc, n->seg, n->stream));
    G4S_CUDA(cudaStreamSynchronize(n->stream));
  }
  n->team_p = p;
  n->team_rc = rc;
  n->team_ready = true;
  n->team_ok = true;
  return G4S_OK;
}

// Tables are kept with every row sorted by target (the pairs stay together); the
// segment table of the team kernel is rebuilt on the next SKL run.  The exactness bound
// of the split shared-memory accumulation is measured here: fewer than 65536 synapses
// into any neuron and sum(|q| >> 16) + 1 over them below 2^31 - 2^20.
// Largest in-degree (h[0]) of the tables and, with with_mag, the largest sum(|q| >> 16) + 1
// over a neuron's inputs (h[1]), else the largest (|q| >> 16) + 1 of any synapse (h[2]); on
// the network's stream (stream-ordered scratch).
static int bound_pass(g4s_net *n, bool with_mag, unsigned long long h[3]) {
  cudaStream_t st = n->stream;
  unsigned *cnt = nullptr;
  unsigned long long *mag = nullptr, *out = nullptr;
  cudaError_t e = cudaMallocAsync((void **)&cnt, (size_t)n->v.n * 4, st);
  if (e == cudaSuccess && with_mag) e = cudaMallocAsync((void **)&mag, (size_t)n->v.n * 8, st);
  if (e == cudaSuccess) e = cudaMallocAsync((void **)&out, 24, st);
  if (e == cudaSuccess) e = launch_inbound(n->v, cnt, mag, out, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, out, 24, cudaMemcpyDeviceToHost, st);
  if (cnt) cudaFreeAsync(cnt, st);
  if (mag) cudaFreeAsync(mag, st);
  if (out) cudaFreeAsync(out, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? G4S_OK : cuda_error(e, "table bound pass");
}

static int finish_tables(g4s_net *n, bool may_be_sorted) {
  // (rows that arrive sorted, as tables read back from a network do, skip the sort)
  // Scratch is stream-ordered (cudaMallocAsync / cudaFreeAsync on the network's stream):
  // a plain cudaFree waits for the whole device, i.e. for whatever other networks are
  // running, where a server creates networks while its rounds run.
  cudaStream_t st = n->stream;
  int *flag = nullptr, h_unsorted = 1;
  cudaError_t ef = may_be_sorted ? cudaMallocAsync((void **)&flag, sizeof(int), st) : cudaSuccess;
  if (ef == cudaSuccess && flag) ef = launch_rows_sorted(n->v, flag, st);
  if (ef == cudaSuccess && flag) ef = cudaMemcpyAsync(&h_unsorted, flag, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (flag) cudaFreeAsync(flag, st);
  if (ef == cudaSuccess && flag) ef = cudaStreamSynchronize(st);
  if (ef != cudaSuccess) return cuda_error(ef, "row order check");
  if (h_unsorted) G4S_CUDA(launch_sort_rows(n->v, !may_be_sorted, st));
  n->team_ready = false;
  n->pair_ready = false;
  // The bound.  One pass counts the in-degrees and finds the largest term (|q| >> 16) + 1
  // of any synapse: sum(|q| >> 16) + 1 over a neuron's inputs is at most its in-degree x
  // that term, which settles the bound unless some neuron has many large inputs (for the
  // generated law, an in-degree of about 32 x nsyn); only then are the sums formed exactly,
  // by a second pass with one more atomic per synapse.
  unsigned long long h[3] = {~0ull, ~0ull, ~0ull};
  int rc = bound_pass(n, false, h);
  if (rc) return rc;
  const unsigned long long limit = (1ull << 31) - (1ull << 20);
  if (h[0] < 65536ull && h[2] < limit && h[0] * h[2] < limit)
    h[1] = h[0] * h[2];  // (an upper bound of the sum)
  else if ((rc = bound_pass(n, true, h)))
    return rc;
  n->max_in = h[0];
  n->max_mag = h[1];
  n->tables_fit = h[0] < 65536ull && h[1] < (1ull << 31) - (1ull << 20);
  return check_status(n, "row sort");
}

// Results of one chunk of `cs` steps: per-step counts, raster offsets and stamps, and the
// raster itself when recorded; each step's ids sorted (the device order is by CTA).
// The three steps of absorbing a chunk, so that a batch can enqueue every network's
// copies on one stream and synchronise once: per-step metadata, then the raster of the
// networks that record it, then the host-side bookkeeping.
static int chunk_copy_meta(g4s_net *n, int cs, cudaStream_t s) {
  NetView &v = n->v;
  G4S_CUDA(cudaMemcpyAsync(n->h_counts, v.counts, (size_t)cs * 4, cudaMemcpyDeviceToHost, s));
  G4S_CUDA(cudaMemcpyAsync(n->h_base, v.base, (size_t)cs * 8, cudaMemcpyDeviceToHost, s));
  G4S_CUDA(cudaMemcpyAsync(n->h_stamps, v.stamps, (size_t)cs * 16, cudaMemcpyDeviceToHost, s));
  return G4S_OK;
}

static int64_t chunk_total(const g4s_net *n, int cs) { return (int64_t)n->h_base[cs - 1] + n->h_counts[cs - 1]; }

static int chunk_copy_raster(g4s_net *n, int cs, cudaStream_t s) {
  const int64_t total = chunk_total(n, cs);
  if (n->desc.record_raster && total > 0)
    G4S_CUDA(cudaMemcpyAsync(n->h_raster, n->v.raster, (size_t)total * 4, cudaMemcpyDeviceToHost, s));
  return G4S_OK;
}

// One step's ids in ascending order.  The team kernel writes them rank by rank (ranks own
// ascending ranges), each rank's few ids in arrival order, so an insertion sort finishes in
// a few shifts per id; an order far from sorted (a one-CTA team's ids) goes to std::sort
// once the shifts exceed a small multiple of the count.
static void sort_step_ids(int *b, int cnt) {
  int64_t budget = 4 * (int64_t)cnt + 64;
  for (int i = 1; i < cnt; ++i) {
    const int x = b[i];
    int j = i;
    while (j > 0 && b[j - 1] > x) {
      b[j] = b[j - 1];
      --j;
      if (--budget < 0) {
        b[j] = x;
        std::sort(b, b + cnt);
        return;
      }
    }
    b[j] = x;
  }
}

// The host side of a finished chunk that began at step t0, from its per-step counts, raster
// offsets and stamps and the raster in the pinned staging buffer: the sorted raster (kept
// or streamed to its file), the counts and the per-step times.
static void chunk_finish_from(g4s_net *n, int cs, const int *counts, const long long *base,
                              const unsigned long long *stamps, int64_t t0, int64_t *spikes) {
  const int64_t total = (int64_t)base[cs - 1] + counts[cs - 1];
  if (n->desc.record_raster && n->rstream) {
    for (int lt = 0; lt < cs; ++lt) sort_step_ids(n->h_raster + base[lt], counts[lt]);
    raster_push(n->rstream, counts, cs, n->h_raster, total);
  } else if (n->desc.record_raster && total > 0) {
    const size_t off = n->rt.size();
    n->rt.resize(off + (size_t)total);
    n->rid.resize(off + (size_t)total);
    auto steps = [&](int l0, int l1) {
      for (int lt = l0; lt < l1; ++lt) {
        int *b = n->h_raster + base[lt];
        sort_step_ids(b, counts[lt]);
        const int32_t t = (int32_t)(t0 + lt);
        int32_t *rt = n->rt.data() + off + (size_t)base[lt], *rid = n->rid.data() + off + (size_t)base[lt];
        for (int q = 0; q < counts[lt]; ++q) {
          rt[q] = t;
          rid[q] = b[q];
        }
      }
    };
    // a large chunk on several host threads, each a run of whole steps (steps are independent)
    const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    const int parts = total >= ((int64_t)1 << 20) ? (int)std::min<int64_t>(hw, cs) : 1;
    if (parts <= 1) {
      steps(0, cs);
    } else {
      std::vector<std::thread> pool;
      int l0 = 0;
      for (int p = 0; p < parts; ++p) {
        // the steps up to the p+1-th share of the chunk's ids
        const int64_t goal = total * (p + 1) / parts;
        int l1 = l0;
        while (l1 < cs && (p == parts - 1 || (int64_t)base[l1] < goal)) ++l1;
        if (p == parts - 1) {
          steps(l0, l1);
        } else if (l1 > l0) {
          pool.emplace_back(steps, l0, l1);
        }
        l0 = l1;
      }
      for (auto &th : pool) th.join();
    }
  }
  for (int lt = 0; lt < cs; ++lt) {
    n->counts.push_back(counts[lt]);
    const unsigned long long s0 = stamps[2 * lt], s1 = stamps[2 * lt + 1];
    const unsigned long long s2 = lt + 1 < cs ? stamps[2 * lt + 2] : 0ull;
    n->upd_ms.push_back(s1 > s0 ? (float)((s1 - s0) * 1e-6) : 0.0f);
    n->step_ms.push_back(s2 > s0 ? (float)((s2 - s0) * 1e-6) : 0.0f);
  }
  *spikes = total;
}

static void chunk_finish(g4s_net *n, int cs, int64_t *spikes) {
  chunk_finish_from(n, cs, n->h_counts, n->h_base, n->h_stamps, n->t_abs, spikes);
  n->t_abs += cs;
}

// Results of one chunk of `cs` steps of one network: per-step counts, raster offsets and
// stamps, and the raster itself when recorded; each step's ids sorted (the device order
// is by CTA).
static int absorb_chunk(g4s_net *n, int cs, int64_t *spikes) {
  int rc = chunk_copy_meta(n, cs, n->stream);
  if (rc) return rc;
  G4S_CUDA(cudaStreamSynchronize(n->stream));
  if ((rc = chunk_copy_raster(n, cs, n->stream))) return rc;
  G4S_CUDA(cudaStreamSynchronize(n->stream));
  chunk_finish(n, cs, spikes);
  return G4S_OK;
}

// Delivery mapping of a network's multi-CTA team: the one set or tuned, else eight-lane
// groups when a rank's segment of a row holds kGroupMinSegment synapses or more on average.
static int deliver_mode_of(const g4s_net *n) {
  if (n->deliver_mode != kDeliverAuto) return n->deliver_mode;
  return n->team_p > 1 && (int64_t)n->v.nsyn >= (int64_t)kGroupMinSegment * n->team_p ? kDeliverGroup : kDeliverRun;
}

// ---------------------------------------------------------------------------------------
// One launch of the team kernel over several networks (a "round"): network i advances
// steps[i] steps (at most its chunk length).  Multi-CTA teams are queued first, then the
// one-CTA teams by decreasing work, so that long networks start early.
// ---------------------------------------------------------------------------------------
// team_round_start enqueues the round on stream s and returns; team_round_finish waits for
// it and checks every network's status words.  Between the two, the host may work on the
// previous round's results, but must not touch the pinned per-step buffers (the round's
// graph writes them at its end) nor the networks' device arrays.
static int team_round_start(g4s_net *const *nets, const int *steps, const bool *last, int count, TeamLaunch &L,
                            cudaStream_t s, unsigned long long limit_ns, int stall) {
  std::vector<int> order;
  L.order.clear();
  int nslots = 0, maxteam = 1;
  size_t smem = 16;
  for (int i = 0; i < count; ++i)
    if (steps[i] > 0) {
      order.push_back(i);
      nslots += nets[i]->team_p;
      maxteam = std::max(maxteam, nets[i]->team_p);
      smem = std::max(smem, team_smem(nets[i]->team_rc, nets[i]->team_p));
    }
  if (order.empty()) return G4S_OK;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    const g4s_net *x = nets[a], *y = nets[b];
    if ((x->team_p > 1) != (y->team_p > 1)) return x->team_p > 1;
    if (x->team_p != y->team_p) return x->team_p > y->team_p;
    return (double)x->v.n * steps[a] * x->v.nsyn > (double)y->v.n * steps[b] * y->v.nsyn;
  });
  int rc = L.reserve(count, nslots);
  if (rc) return rc;
  bool pair = true;  // every network of the round has its interleaved rows
  for (int i : order) pair = pair && nets[i]->v.pair != nullptr;
  int nt = nets[order[0]]->team_nt_eff;  // threads per CTA: the networks' own when they agree
  for (int i : order)
    if (nets[i]->team_nt_eff != nt) nt = kTeamNT;
  int gmax = 0;
  G4S_CUDA(team_max_blocks(smem, &gmax, nt));  // also raises the kernel's shared-memory ceiling
  if (gmax < maxteam) return set_error(G4S_ERR_CUDA, "team larger than the co-resident grid");
  const int grid = std::min(nslots, gmax);
  // this round's descriptors, in pinned host memory the graph copies from
  int k = 0;
  for (int i : order) {
    g4s_net *n = nets[i];
    TeamItem &it = L.h_items[i];
    it.v = n->v;
    it.seg = n->seg;
    it.list = n->list;
    it.rec = reinterpret_cast<unsigned long long *>(n->gs + 1);
    it.t_abs0 = n->t_abs;
    it.steps = steps[i];
    it.last = last[i] ? 1 : 0;
    it.team = n->team_p;
    it.rc = (int)n->team_rc;
    it.sync = n->gs;
    it.mode = deliver_mode_of(n);
    it.cap = team_window(n->team_rc, n->team_p);
    if ((uint64_t)n->tag_next + (uint64_t)steps[i] + 2 >= 0xFFFFFFFFull) {  // tags would wrap: start over
      G4S_CUDA(cudaMemsetAsync(n->list, 0, (size_t)n->v.n * 4 * sizeof(unsigned long long), s));
      n->tag_next = 0;
    }
    it.tag0 = n->tag_next;
    n->tag_next += (uint32_t)steps[i];
    for (int r = 0; r < n->team_p; ++r) L.h_slots[k++] = make_int2(i, r);
  }
  for (int i = 0; i < count; ++i)
    if (steps[i] <= 0) L.h_items[i].steps = 0;
  L.h_ctl[0] = nslots;
  L.h_ctl[1] = 0;
  L.direct = count > 1;
  if (L.direct) {
    // Many networks: the set changes from round to round (a server admits and retires
    // requests), so a graph would be captured and instantiated for almost every round, at a
    // cost that grows with the networks.  Launched directly instead, in a fixed number of
    // calls: descriptors up, one kernel clearing every network's per-launch words, the team
    // kernel between two events, one kernel packing every network's results, one copy down.
    size_t total = 0;
    for (int i : order) {
      L.h_off[i] = (int64_t)total;
      total += round_pack_bytes(steps[i]);
    }
    if ((rc = L.reserve_pack(total))) return rc;
    L.nets.assign(nets, nets + count);
    L.steps.assign(steps, steps + count);
    G4S_CUDA(cudaMemcpyAsync(L.d_items, L.h_items, sizeof(TeamItem) * count, cudaMemcpyHostToDevice, s));
    G4S_CUDA(cudaMemcpyAsync(L.d_slots, L.h_slots, sizeof(int2) * nslots, cudaMemcpyHostToDevice, s));
    G4S_CUDA(cudaMemcpyAsync(L.d_ctl, L.h_ctl, 8, cudaMemcpyHostToDevice, s));
    G4S_CUDA(cudaMemcpyAsync(L.d_off, L.h_off, sizeof(int64_t) * count, cudaMemcpyHostToDevice, s));
    G4S_CUDA(launch_round_clear(L.d_items, count, s));
    G4S_CUDA(cudaEventRecord(L.e0, s));
    G4S_CUDA(launch_team(L.d_items, L.d_slots, L.d_ctl, L.d_ctl + 1, grid, smem, limit_ns, stall, s, pair, nt));
    G4S_CUDA(cudaEventRecord(L.e1, s));
    G4S_CUDA(launch_round_gather(L.d_items, L.d_off, count, L.d_pack, s));
    G4S_CUDA(cudaMemcpyAsync(L.h_pack, L.d_pack, total, cudaMemcpyDeviceToHost, s));
    L.order = order;
    return G4S_OK;
  }
  // The round's graph: clear the networks' per-chunk arrays, error words and spike records,
  // upload the descriptors, the persistent launch between two timing events, and copy
  // back each network's per-step counts, offsets and stamps and its status words.  Its
  // shape depends only on which networks run, their teams and chunk lengths, and the
  // launch parameters; the descriptors' contents are read from pinned memory at replay.
  // A graph must not outlive the buffers it copies to and from: a network freed and another
  // created in its place (often at the same device and pinned host addresses) gets a new
  // graph, so the key holds each network's creation number as well as its addresses.
  auto u = [](const void *p) { return (uint64_t)(uintptr_t)p; };
  std::vector<uint64_t> sig = {(uint64_t)count, (uint64_t)nslots, (uint64_t)grid, (uint64_t)smem, limit_ns,
                               (uint64_t)stall, (uint64_t)pair, (uint64_t)nt, u(L.d_items), u(L.d_slots), u(L.d_ctl), u(L.h_items),
                               u(L.h_slots), u(L.h_ctl), u(L.h_status), u(L.e0), u(L.e1)};
  for (int i : order) {
    const g4s_net *n = nets[i];
    for (uint64_t x : {(uint64_t)i, n->serial, (uint64_t)n->team_p, (uint64_t)n->chunk_steps, u(n->v.counts), u(n->v.stamps),
                       u(n->v.status), u(n->gs), u(n->v.base), u(n->h_counts), u(n->h_base), u(n->h_stamps)})
      sig.push_back(x);
  }
  if (!L.exec || sig != L.sig) {
    L.drop_graph();
    G4S_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
    for (int i : order) {
      const g4s_net *n = nets[i];
      const size_t cs = (size_t)n->chunk_steps;
      if (e == cudaSuccess) e = cudaMemsetAsync(n->v.counts, 0, cs * sizeof(int), s);
      if (e == cudaSuccess) e = cudaMemsetAsync(n->v.stamps, 0, (cs * 2 + 2) * 8, s);
      if (e == cudaSuccess) e = cudaMemsetAsync(n->v.status, 0, sizeof(int), s);
      // error word and the team's spike records (two sets of kRecLines 128-byte lines per rank)
      if (e == cudaSuccess) e = cudaMemsetAsync(n->gs, 0, sizeof(GridSync) * (1 + 2 * (size_t)n->team_p * kRecLines), s);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(L.d_items, L.h_items, sizeof(TeamItem) * count, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(L.d_slots, L.h_slots, sizeof(int2) * nslots, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(L.d_ctl, L.h_ctl, 8, cudaMemcpyHostToDevice, s);
    // (external records: the graph records the events at every replay)
    if (e == cudaSuccess) e = cudaEventRecordWithFlags(L.e0, s, cudaEventRecordExternal);
    if (e == cudaSuccess) e = launch_team(L.d_items, L.d_slots, L.d_ctl, L.d_ctl + 1, grid, smem, limit_ns, stall, s, pair, nt);
    if (e == cudaSuccess) e = cudaEventRecordWithFlags(L.e1, s, cudaEventRecordExternal);
    for (int i : order) {
      const g4s_net *n = nets[i];
      const size_t cs = (size_t)n->chunk_steps;
      if (e == cudaSuccess) e = cudaMemcpyAsync(n->h_counts, n->v.counts, cs * 4, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaMemcpyAsync(n->h_base, n->v.base, cs * 8, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaMemcpyAsync(n->h_stamps, n->v.stamps, cs * 16, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaMemcpyAsync(L.h_status + 2 * i, n->v.status, sizeof(int), cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(L.h_status + 2 * i + 1, &n->gs->error, sizeof(int), cudaMemcpyDeviceToHost, s);
    }
    cudaGraph_t g = nullptr;
    const cudaError_t e_end = cudaStreamEndCapture(s, &g);
    if (e == cudaSuccess) e = e_end;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&L.exec, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      L.exec = nullptr;
      return cuda_error(e, "capturing the team round as a CUDA graph");
    }
    L.sig = sig;
  }
  G4S_CUDA(cudaGraphLaunch(L.exec, s));
  L.order = order;
  return G4S_OK;
}

static int team_round_finish(TeamLaunch &L, cudaStream_t s, double *kernel_ms, int64_t *launches) {
  if (L.order.empty()) return G4S_OK;  // nothing was launched
  G4S_CUDA(cudaStreamSynchronize(s));
  float ms = 0.0f;
  G4S_CUDA(cudaEventElapsedTime(&ms, L.e0, L.e1));
  *kernel_ms += ms;
  *launches += 1;
  if (L.direct)  // each network's share of the pack into its own pinned per-step buffers
    for (int i : L.order) {
      g4s_net *n = L.nets[(size_t)i];
      const size_t st = (size_t)L.steps[(size_t)i];
      const unsigned char *p = L.h_pack + L.h_off[i];
      std::memcpy(L.h_status + 2 * i, p, 8);
      std::memcpy(n->h_counts, p + 8, st * 4);
      std::memcpy(n->h_base, p + 8 + ((st * 4 + 7) & ~(size_t)7), st * 8);
      std::memcpy(n->h_stamps, p + 8 + ((st * 4 + 7) & ~(size_t)7) + st * 8, st * 16);
    }
  for (int i : L.order) {
    const int rc = status_rc(L.h_status[2 * i], L.h_status[2 * i + 1], "team step kernel");
    if (rc) return rc;
  }
  return G4S_OK;
}

static int team_round(g4s_net *const *nets, const int *steps, const bool *last, int count, TeamLaunch &L,
                      cudaStream_t s, unsigned long long limit_ns, int stall, double *kernel_ms, int64_t *launches) {
  const int rc = team_round_start(nets, steps, last, count, L, s, limit_ns, stall);
  return rc ? rc : team_round_finish(L, s, kernel_ms, launches);
}

static int run_net(g4s_net *n, int32_t steps, int32_t alg_in) {
  if (steps < 0) return set_error(G4S_ERR_INVALID, "steps must be >= 0");
  if (alg_in < 0 || alg_in > kAlgAuto) return set_error(G4S_ERR_INVALID, "unknown algorithm");
  if (n->t_abs + steps > (int64_t)INT32_MAX) return set_error(G4S_ERR_INVALID, "step counter limit");
  const int alg = resolve_alg(n, alg_in);
  NetView &v = n->v;
  if (n->shape.k_hint <= 0) n->shape.k_hint = (int)std::max<int64_t>(1, v.n / 20);
  if (alg == kAlgSKL) {
    int rc0 = prepare_team(n);
    if (rc0) return rc0;
  }
  const bool team = alg == kAlgSKL && n->team_ok && n->team_ready;
  const auto w0 = std::chrono::steady_clock::now();
  G4S_CUDA(cudaEventRecord(n->ev0, n->stream));
  int64_t remaining = steps, spikes = 0, launches = 0;
  double kernel_ms = 0.0;
  if (team) {
    // Chunks as team rounds, pipelined: once a round has ended and its raster is copied
    // down, the next round is launched, and the host sorts and files the finished chunk
    // while the GPU runs the next one.
    std::vector<int> mc;
    std::vector<long long> mb;
    std::vector<unsigned long long> ms;
    int cs = 0;
    auto start = [&]() -> int {
      cs = (int)std::min<int64_t>(remaining, n->chunk_steps);
      const bool last_chunk = remaining == cs;
      g4s_net *one[1] = {n};
      const int rc = team_round_start(one, &cs, &last_chunk, 1, n->launch, n->stream, n->barrier_ns, n->barrier_stall);
      n->barrier_stall = 0;
      remaining -= cs;
      return rc;
    };
    int rc = remaining > 0 ? start() : G4S_OK;
    if (rc) return rc;
    while (cs > 0) {
      if ((rc = team_round_finish(n->launch, n->stream, &kernel_ms, &launches))) return rc;
      // this chunk's per-step arrays, out of the pinned buffers the next round's graph
      // writes, and its raster, out of the device buffer the next round overwrites
      mc.assign(n->h_counts, n->h_counts + cs);
      mb.assign(n->h_base, n->h_base + cs);
      ms.assign(n->h_stamps, n->h_stamps + 2 * (size_t)cs);
      if ((rc = chunk_copy_raster(n, cs, n->stream))) return rc;
      G4S_CUDA(cudaStreamSynchronize(n->stream));
      const int done = cs;
      const int64_t t0 = n->t_abs;
      n->t_abs += done;
      cs = 0;
      const int rs = remaining > 0 ? start() : G4S_OK;
      int64_t chunk_spikes = 0;  // (the finished chunk is filed even if the next launch failed)
      chunk_finish_from(n, done, mc.data(), mb.data(), ms.data(), t0, &chunk_spikes);
      spikes += chunk_spikes;
      if (rs) return rs;
    }
  }
  while (!team && remaining > 0) {
    // (host-driven chunks stay short enough for their graphs to instantiate quickly)
    const int64_t chunk = alg == kAlgSKL ? n->chunk_legacy : std::min<int64_t>(n->chunk_legacy, kStepGraphSteps);
    const int cs = (int)std::min<int64_t>(remaining, chunk);
    const bool last_chunk = remaining == cs;
    if (alg == kAlgSKL) {
      G4S_CUDA(cudaMemsetAsync(v.counts, 0, (size_t)cs * sizeof(int), n->stream));
      G4S_CUDA(cudaMemsetAsync(v.stamps, 0, ((size_t)cs * 2 + 2) * 8, n->stream));
      G4S_CUDA(cudaMemsetAsync(n->gs, 0, sizeof(GridSync), n->stream));
      G4S_CUDA(cudaEventRecord(n->ek0, n->stream));
      G4S_CUDA(launch_persistent(v, n->t_abs, cs, last_chunk, n->gs, n->barrier_ns, n->shape.group,
                                 n->barrier_stall, n->stream));
      n->barrier_stall = 0;
      launches += 1;
      G4S_CUDA(cudaEventRecord(n->ek1, n->stream));
    } else {
      // The chunk as a CUDA graph (two launches per step would otherwise each cost a host
      // launch and a gap on the GPU): the chunk's first step from pinned memory, the
      // clears, then update and delivery for every step between two timing events.  A
      // chunk is captured only when its graph will be replayed (a graph of this shape
      // exists, or at least two more chunks of its length follow); otherwise it is
      // launched step by step.
      *n->h_t0 = n->t_abs;
      const std::vector<uint64_t> key = {(uint64_t)alg, (uint64_t)cs, (uint64_t)last_chunk,
                                         (uint64_t)n->shape.group, (uint64_t)n->shape.blocks_per_sm,
                                         (uint64_t)n->shape.k_hint};
      cudaGraphExec_t exec = nullptr;
      for (auto &gr : n->step_graphs)
        if (gr.key == key) exec = gr.exec;
      const bool replayed = exec || (!last_chunk && remaining >= 2 * (int64_t)cs);
      if (!replayed) {
        G4S_CUDA(cudaMemcpyAsync(n->d_t0, n->h_t0, sizeof(long long), cudaMemcpyHostToDevice, n->stream));
        G4S_CUDA(cudaMemsetAsync(v.counts, 0, (size_t)cs * sizeof(int), n->stream));
        G4S_CUDA(cudaMemsetAsync(v.stamps, 0, ((size_t)cs * 2 + 2) * 8, n->stream));
        G4S_CUDA(cudaEventRecord(n->ek0, n->stream));
        for (int lt = 0; lt < cs; ++lt) {
          G4S_CUDA(launch_update(v, n->d_t0, lt, last_chunk && lt == cs - 1, n->stream));
          G4S_CUDA(launch_deliver(v, lt, alg, n->shape, n->stream));
        }
        G4S_CUDA(cudaEventRecord(n->ek1, n->stream));
      } else if (!exec) {
        if ((int)n->step_graphs.size() >= kStepGraphs) {  // the oldest goes
          cudaGraphExecDestroy(n->step_graphs.front().exec);
          n->step_graphs.erase(n->step_graphs.begin());
        }
        G4S_CUDA(cudaStreamBeginCapture(n->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = cudaMemcpyAsync(n->d_t0, n->h_t0, sizeof(long long), cudaMemcpyHostToDevice, n->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(v.counts, 0, (size_t)cs * sizeof(int), n->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(v.stamps, 0, ((size_t)cs * 2 + 2) * 8, n->stream);
        if (e == cudaSuccess) e = cudaEventRecordWithFlags(n->ek0, n->stream, cudaEventRecordExternal);
        for (int lt = 0; lt < cs && e == cudaSuccess; ++lt) {
          e = launch_update(v, n->d_t0, lt, last_chunk && lt == cs - 1, n->stream);
          if (e == cudaSuccess) e = launch_deliver(v, lt, alg, n->shape, n->stream);
        }
        if (e == cudaSuccess) e = cudaEventRecordWithFlags(n->ek1, n->stream, cudaEventRecordExternal);
        cudaGraph_t g = nullptr;
        const cudaError_t e_end = cudaStreamEndCapture(n->stream, &g);
        if (e == cudaSuccess) e = e_end;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, g, 0);
        if (g) cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_error(e, "capturing a chunk of the step kernels");
        n->step_graphs.push_back({key, exec});
      }
      if (exec) G4S_CUDA(cudaGraphLaunch(exec, n->stream));
      launches += 2 * (int64_t)cs;
    }
    {
      int rc = check_status(n, alg == kAlgSKL ? "persistent step kernel" : "step kernels");
      if (rc) return rc;
      float kms = 0.0f;
      G4S_CUDA(cudaEventElapsedTime(&kms, n->ek0, n->ek1));
      kernel_ms += kms;
    }
    int64_t chunk_spikes = 0;
    int rc = absorb_chunk(n, cs, &chunk_spikes);
    if (rc) return rc;
    spikes += chunk_spikes;
    remaining -= cs;
  }
  G4S_CUDA(cudaEventRecord(n->ev1, n->stream));
  G4S_CUDA(cudaEventSynchronize(n->ev1));
  float ms = 0.0f;
  G4S_CUDA(cudaEventElapsedTime(&ms, n->ev0, n->ev1));
  n->last_ms = ms;
  n->last_wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - w0).count();
  n->last_spikes = spikes;
  n->total_spikes += spikes;
  n->last_alg = alg;
  n->last_kernel_ms = kernel_ms;
  n->last_launches = launches;
  return G4S_OK;
}

// Several networks advanced together by the SKL team kernel: network i runs steps[i]
// further steps; each round advances every unfinished network by up to its chunk length
// in one persistent launch.
static int run_nets(g4s_net *const *nets, const int32_t *steps, int count, double *dev_ms, int64_t *launches) {
  if (count <= 0) return set_error(G4S_ERR_INVALID, "count must be > 0");
  for (int i = 0; i < count; ++i)
    if (!nets[i]) return set_error(G4S_ERR_INVALID, "null handle in batch");
  // Neurons per CTA of the batch: kBatchSlice, unless the teams that gives leave SMs idle
  // (few networks, as at a server's start and end): then the smallest slice of a fixed
  // ladder (half octaves down to a lone network's), whose teams still fit one CTA per SM
  // together.  (A ladder, so that a network's team, and its segment table, change only when
  // the batch changes by a factor.)
  static const int64_t kSlices[] = {kBatchSlice, 6144, 4096, 3072, 2048, 1536, 1024, 768, 512, 384, 256, 192, kSoloSlice};
  int64_t slice = kBatchSlice;
  if (count > 1) {
    int gmax = 0;
    if (team_max_blocks(kTeamSmemLimit, &gmax) != cudaSuccess || gmax < 1) {
      (void)cudaGetLastError();
      gmax = 0;
    }
    const int64_t pcap = std::min(gmax, kMaxTeam);
    auto slots = [&](int64_t sl) {
      int64_t t = 0;
      for (int i = 0; i < count; ++i)
        if (steps[i] > 0) t += std::min(pcap, (nets[i]->v.n + sl - 1) / sl);
      return t;
    };
    for (size_t k = 1; gmax > 0 && k < sizeof(kSlices) / sizeof(kSlices[0]) && slots(kSlices[k]) <= gmax; ++k)
      slice = kSlices[k];
  }
  std::vector<int64_t> remaining(count);
  for (int i = 0; i < count; ++i) {
    if (steps[i] < 0 || nets[i]->t_abs + steps[i] > (int64_t)INT32_MAX)
      return set_error(G4S_ERR_INVALID, "bad step count in batch");
    for (int j = 0; j < i; ++j)
      if (nets[j] == nets[i]) return set_error(G4S_ERR_INVALID, "a handle appears twice in the batch");
    int rc = prepare_team(nets[i], count > 1, slice);
    if (rc) return rc;
    if (!nets[i]->team_ok)
      return set_error(G4S_ERR_INVALID, "a network of the batch does not fit the team kernel");
    remaining[i] = steps[i];
    nets[i]->last_spikes = 0;
  }
  static thread_local TeamLaunch L;
  cudaStream_t s = nets[0]->stream;
  std::vector<int> cs(count);
  std::unique_ptr<bool[]> last(new bool[count]);
  double kms = 0.0;
  int64_t nl = 0;
  const auto w0 = std::chrono::steady_clock::now();
  for (;;) {
    bool any = false;
    for (int i = 0; i < count; ++i) {
      cs[i] = (int)std::min<int64_t>(remaining[i], nets[i]->chunk_steps);
      last[i] = cs[i] > 0 && cs[i] == remaining[i];
      any = any || cs[i] > 0;
    }
    if (!any) break;
    int rc = team_round(nets, cs.data(), last.get(), count, L, s, nets[0]->barrier_ns, 0, &kms, &nl);
    if (rc) return rc;
    for (int i = 0; i < count; ++i)
      if (cs[i] > 0 && (rc = chunk_copy_raster(nets[i], cs[i], s))) return rc;
    G4S_CUDA(cudaStreamSynchronize(s));
    for (int i = 0; i < count; ++i)
      if (cs[i] > 0) {
        int64_t sp = 0;
        chunk_finish(nets[i], cs[i], &sp);
        nets[i]->last_spikes += sp;
        nets[i]->total_spikes += sp;
        remaining[i] -= cs[i];
      }
  }
  const double wall = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - w0).count();
  for (int i = 0; i < count; ++i) {
    nets[i]->last_alg = kAlgSKL;
    nets[i]->last_kernel_ms = kms;
    nets[i]->last_ms = wall;
    nets[i]->last_wall_ms = wall;
    nets[i]->last_launches = nl;
  }
  if (dev_ms) *dev_ms = kms;
  if (launches) *launches = nl;
  return G4S_OK;
}

// ---------------------------------------------------------------------------------------
// Autotuner measurement: a device snapshot of the mutable state and the host record,
// each candidate timed on `probe` steps from the snapshot, the snapshot restored.
// Candidates: SKL with the default team and with teams of 1, 2, 4, ... CTAs up to the
// co-resident grid (those that fit), AB and AP.
// ---------------------------------------------------------------------------------------
struct StateSnapshot {
  float2 *vu = nullptr;
  long long *acc = nullptr;
  SpikeStat *ss = nullptr;
  float *il = nullptr;
  int64_t t_abs = 0, total = 0;
  size_t nr = 0, nc = 0;
  ~StateSnapshot() {
    cudaFree(vu);
    cudaFree(acc);
    cudaFree(ss);
    cudaFree(il);
  }
};

static int snapshot_take(g4s_net *n, StateSnapshot &s) {
  const size_t N = (size_t)n->v.n;
  G4S_CUDA(cudaMalloc((void **)&s.vu, N * sizeof(float2)));
  G4S_CUDA(cudaMalloc((void **)&s.acc, N * sizeof(long long)));
  G4S_CUDA(cudaMalloc((void **)&s.ss, N * sizeof(SpikeStat)));
  G4S_CUDA(cudaMalloc((void **)&s.il, N * sizeof(float)));
  G4S_CUDA(cudaMemcpyAsync(s.vu, n->v.vu, N * sizeof(float2), cudaMemcpyDeviceToDevice, n->stream));
  G4S_CUDA(cudaMemcpyAsync(s.acc, n->v.acc, N * sizeof(long long), cudaMemcpyDeviceToDevice, n->stream));
  G4S_CUDA(cudaMemcpyAsync(s.ss, n->v.sstat, N * sizeof(SpikeStat), cudaMemcpyDeviceToDevice, n->stream));
  G4S_CUDA(cudaMemcpyAsync(s.il, n->v.ilast, N * sizeof(float), cudaMemcpyDeviceToDevice, n->stream));
  G4S_CUDA(cudaStreamSynchronize(n->stream));
  s.t_abs = n->t_abs;
  s.total = n->total_spikes;
  s.nr = n->rt.size();
  s.nc = n->counts.size();
  return G4S_OK;
}

static int snapshot_restore(g4s_net *n, const StateSnapshot &s) {
  const size_t N = (size_t)n->v.n;
  G4S_CUDA(cudaMemcpyAsync(n->v.vu, s.vu, N * sizeof(float2), cudaMemcpyDeviceToDevice, n->stream));
  G4S_CUDA(cudaMemcpyAsync(n->v.acc, s.acc, N * sizeof(long long), cudaMemcpyDeviceToDevice, n->stream));
  G4S_CUDA(cudaMemcpyAsync(n->v.sstat, s.ss, N * sizeof(SpikeStat), cudaMemcpyDeviceToDevice, n->stream));
  G4S_CUDA(cudaMemcpyAsync(n->v.ilast, s.il, N * sizeof(float), cudaMemcpyDeviceToDevice, n->stream));
  G4S_CUDA(cudaStreamSynchronize(n->stream));
  n->t_abs = s.t_abs;
  n->total_spikes = s.total;
  n->rt.resize(s.nr);
  n->rid.resize(s.nr);
  n->counts.resize(s.nc);
  n->upd_ms.resize(s.nc);
  n->step_ms.resize(s.nc);
  return G4S_OK;
}

static int autotune(g4s_net *n, int32_t probe, TuneChoice *best, double *best_us) {
  probe = std::max(8, std::min(probe, 4000));
  StateSnapshot snap;
  int rc = snapshot_take(n, snap);
  if (rc) return rc;
  const int keep_p = n->want_p;
  std::vector<TuneChoice> cand;
  int pmax = 0;
  if (team_max_blocks(team_smem(1, 1), &pmax) != cudaSuccess) pmax = 1;
  (void)cudaGetLastError();
  pmax = std::min(pmax, kMaxTeam);
  std::vector<int> teams = {0};
  for (int p = 1; p <= pmax; p *= 2) teams.push_back(p);
  if (pmax > 1) teams.push_back(pmax);
  // each team size with both CTA sizes of the team kernel, by segment runs and, where a
  // rank's segment of a row averages half the automatic threshold or more, by eight-lane
  // groups too
  for (int p : teams)
    for (int nt : {kTeamNT, kTeamNTSmall}) {
      cand.push_back(TuneChoice{kAlgSKL, p, kDeliverRun, nt});
      const int pe = p == 0 ? pmax : p;
      if (pe > 1 && 2 * (int64_t)n->v.nsyn >= (int64_t)kGroupMinSegment * pe)
        cand.push_back(TuneChoice{kAlgSKL, p, kDeliverGroup, nt});
    }
  cand.push_back(TuneChoice{kAlgAB, 0, kDeliverRun});
  cand.push_back(TuneChoice{kAlgAP, 0, kDeliverRun});
  const int keep_mode = n->deliver_mode, keep_nt = n->team_nt;
  double best_t = 1e300, rate = 0.0;
  TuneChoice pick = cand[0];
  for (const TuneChoice &c : cand) {
    if (c.alg == kAlgSKL) {
      n->want_p = c.team;
      n->deliver_mode = c.mode;
      n->team_nt = c.nt;
      n->team_ready = false;
      n->team_ok = true;
      if ((rc = prepare_team(n))) break;
      if (!n->team_ok || (c.team > 0 && n->team_p != c.team)) continue;  // does not fit
    }
    if ((rc = run_net(n, 8, c.alg)) || (rc = snapshot_restore(n, snap))) break;
    if ((rc = run_net(n, probe, c.alg))) break;
    const double t = n->last_kernel_ms * 1e3 / probe;
    rate = (double)n->last_spikes / ((double)n->v.n * probe) * 1000.0;
    if ((rc = snapshot_restore(n, snap))) break;
    if (t < best_t) {
      best_t = t;
      pick = c;
      if (c.alg == kAlgSKL && c.team == 0) pick.team = n->team_p;
    }
  }
  n->want_p = keep_p;
  n->deliver_mode = keep_mode;
  n->team_nt = keep_nt;
  n->team_ready = false;
  n->team_ok = true;
  if (rc) return rc;
  n->tune = pick;
  n->tuned = true;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[tune_key(n, rate)] = pick;
  }
  *best = pick;
  *best_us = best_t;
  return G4S_OK;
}

// ---------------------------------------------------------------------------------------
// Result files in the reference's formats.
// ---------------------------------------------------------------------------------------
static int mkdirs(const std::string &path) {
  std::string cur;
  for (size_t i = 0; i <= path.size(); ++i) {
    if (i == path.size() || path[i] == '/') {
      if (!cur.empty() && mkdir(cur.c_str(), 0775) != 0 && errno != EEXIST)
        return set_error(G4S_ERR_IO, "mkdir " + cur + ": " + strerror(errno));
    }
    if (i < path.size()) cur.push_back(path[i]);
  }
  return G4S_OK;
}

static void write_record(std::ofstream &o, float a, float b, float c, float d, float v, float u, float I, int64_t id,
                         int nospks) {
  o << a << " " << b << " " << c << " " << d << " " << v << " " << u << " " << I << " " << id << " " << nospks
    << "\n";
}

static int write_results(g4s_net *n, const std::string &dir, double elapsed, double ewd) {
  int rc = mkdirs(dir);
  if (rc) return rc;
  const std::string p = dir.back() == '/' ? dir : dir + "/";
  const int64_t N = n->v.n;
  std::vector<float> v(N), u(N), I(N), a(N), b(N), c(N), d(N);
  std::vector<int32_t> nos(N);
  rc = g4s_net_state(n, v.data(), u.data(), I.data(), a.data(), b.data(), c.data(), d.data(), nos.data());
  if (rc) return rc;
  {
    std::ofstream o(p + "neuroninfo.csv");
    if (!o.is_open()) return set_error(G4S_ERR_IO, "cannot open " + p + "neuroninfo.csv");
    o << "a b c d v u I id nospks" << "\n";
    for (int64_t i = 0; i < N; ++i) write_record(o, a[i], b[i], c[i], d[i], -65.0f, b[i] * -65.0f, 0.0f, i, 0);
  }
  {
    std::ofstream o(p + "spiketimes.csv");
    if (!o.is_open()) return set_error(G4S_ERR_IO, "cannot open " + p + "spiketimes.csv");
    o << "SpkTime NeuronID" << "\n";
    for (size_t q = 0; q < n->rt.size(); ++q) o << n->rt[q] << " " << n->rid[q] << "\n";
  }
  {
    std::ofstream o(p + "computetime.csv");
    if (!o.is_open()) return set_error(G4S_ERR_IO, "cannot open " + p + "computetime.csv");
    o << "TimeStep SpksPerStep TimeKernelUpdate TimeSpent" << "\n";
    for (size_t t = 0; t < n->counts.size(); ++t)
      o << t << " " << n->counts[t] << " " << (double)n->upd_ms[t] << " " << (double)n->step_ms[t] << "\n";
  }
  {
    std::ofstream o(p + "sim_overview.csv");
    if (!o.is_open()) return set_error(G4S_ERR_IO, "cannot open " + p + "sim_overview.csv");
    o << "N elapsed(ms) elapsedwithdata(ms) totalspkcount" << "\n";
    o << N << " " << elapsed << " " << ewd << " " << n->total_spikes;
  }
  {
    std::ofstream o(p + "neuroninfoafter.csv");
    if (!o.is_open()) return set_error(G4S_ERR_IO, "cannot open " + p + "neuroninfoafter.csv");
    o << "a b c d v u I id nospks" << "\n";
    for (int64_t i = 0; i < N; ++i) write_record(o, a[i], b[i], c[i], d[i], v[i], u[i], I[i], i, nos[i]);
  }
  return G4S_OK;
}

// ---------------------------------------------------------------------------------------
// Exported entry points.
// ---------------------------------------------------------------------------------------
extern "C" {

int g4s_abi_version(void) { return G4S_ABI_VERSION; }

const char *g4s_last_error(void) { return g_last_error.c_str(); }

int g4s_set_device(int32_t device) {
  G4S_CUDA(cudaSetDevice(device));
  return G4S_OK;
}

static int create_net(const g4s_net_desc *desc, cudaMemPool_t pool, g4s_net **out) {
  if (!out) return set_error(G4S_ERR_INVALID, "null output handle");
  *out = nullptr;
  g4s_net *n = nullptr;
  int rc = alloc_net(desc, &n, pool);
  if (rc) return rc;
  if (desc->conn_law == G4S_CONN_GLIBC) {
    const size_t cnt = (size_t)n->v.n * (size_t)n->v.stride;
    std::vector<int32_t> idx;
    std::vector<float> w;
    try {
      idx.resize(cnt);
      w.resize(cnt);
    } catch (...) {
      free_net(n);
      return set_error(G4S_ERR_NOMEM, "host tables");
    }
    rc = conn_glibc_host((unsigned)desc->seed, (int32_t)n->v.n, n->v.nsyn, n->v.stride, idx.data(), w.data());
    if (!rc) rc = g4s_net_load_tables(n, idx.data(), w.data(), n->v.stride);
  } else {
    cudaError_t e = launch_conngen(n->v, desc->self_loops, n->stream);
    if (e != cudaSuccess) rc = cuda_error(e, "connectivity kernel");
    if (!rc) rc = check_status(n, "connectivity kernel");
    if (!rc) rc = finish_tables(n, false);  // (generated rows are in draw order)
  }
  if (!rc) rc = reset_net(n);
  if (rc) {
    free_net(n);
    return rc;
  }
  *out = n;
  return G4S_OK;
}

int g4s_net_create(const g4s_net_desc *desc, g4s_net **out) { return create_net(desc, nullptr, out); }

int g4s_net_create_from_tables(const g4s_net_desc *desc, const int32_t *idx, const float *w, int32_t stride,
                               g4s_net **out) {
  if (!out || !idx || !w) return set_error(G4S_ERR_INVALID, "null argument");
  *out = nullptr;
  g4s_net *n = nullptr;
  int rc = alloc_net(desc, &n);
  if (rc) return rc;
  rc = g4s_net_load_tables(n, idx, w, stride);
  if (!rc) rc = reset_net(n);
  if (rc) {
    free_net(n);
    return rc;
  }
  *out = n;
  return G4S_OK;
}

int g4s_net_load_tables(g4s_net *n, const int32_t *idx, const float *w, int32_t stride) {
  if (!n || !idx || !w) return set_error(G4S_ERR_INVALID, "null argument");
  NetView &v = n->v;
  if (stride != v.stride)
    return set_error(G4S_ERR_INVALID, "table stride must be " + std::to_string(v.stride));
  const size_t cnt = (size_t)v.n * (size_t)v.stride, bytes = cnt * 4;
  // every target must be a neuron of this network or negative (an unused slot): checked on
  // all host cores, block by block (the largest target of 4096, a loop the compiler
  // vectorises; a block over the limit is searched for its first offending entry), the
  // first offending entry of the table reported
  {
    const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    const size_t parts = cnt >= ((size_t)1 << 22) ? hw : 1, per = (cnt + parts - 1) / parts;
    const int32_t nn = (int32_t)v.n;  // (n < 2^31)
    std::vector<size_t> bad(parts, SIZE_MAX);
    auto scan = [&](size_t p) {
      const size_t end = std::min(cnt, (p + 1) * per);
      for (size_t k0 = p * per; k0 < end; k0 += 4096) {
        const size_t k1 = std::min(end, k0 + 4096);
        int32_t mx = INT32_MIN;
        for (size_t k = k0; k < k1; ++k) mx = std::max(mx, idx[k]);
        if (mx < nn) continue;
        for (size_t k = k0; k < k1; ++k)
          if (idx[k] >= nn) {
            bad[p] = k;
            return;
          }
      }
    };
    std::vector<std::thread> pool;
    for (size_t p = 1; p < parts; ++p) pool.emplace_back(scan, p);
    scan(0);
    for (auto &t : pool) t.join();
    for (size_t k : bad)
      if (k != SIZE_MAX)
        return set_error(G4S_ERR_INVALID, "table entry " + std::to_string(k) + " targets neuron " +
                                              std::to_string(idx[k]) + " >= n");
  }
  G4S_CUDA(cudaMemcpyAsync(const_cast<int *>(v.idx), idx, bytes, cudaMemcpyHostToDevice, n->stream));
  G4S_CUDA(cudaMemcpyAsync(const_cast<float *>(v.w), w, bytes, cudaMemcpyHostToDevice, n->stream));
  return finish_tables(n, true);
}

int g4s_net_set_geometry(g4s_net *n, int32_t owner_blocks, int32_t delivery) {
  if (!n) return set_error(G4S_ERR_INVALID, "null handle");
  if (owner_blocks < 0) return set_error(G4S_ERR_INVALID, "owner_blocks must be >= 0 (0 = automatic)");
  if (delivery != kDeliverAuto && delivery != kDeliverRun && delivery != kDeliverGroup)
    return set_error(G4S_ERR_INVALID,
                     "delivery must be -1 (automatic), 0 (segment runs) or 1 (eight lanes a spike)");
  n->want_p = owner_blocks;
  n->deliver_mode = delivery;
  n->team_ready = false;
  n->team_ok = true;
  return G4S_OK;
}

int g4s_net_set_block_threads(g4s_net *n, int32_t threads) {
  if (!n) return set_error(G4S_ERR_INVALID, "null handle");
  if (threads != 0 && threads != kTeamNT && threads != kTeamNTSmall)
    return set_error(G4S_ERR_INVALID, "threads must be 1024, 768 or 0 (automatic)");
  n->team_nt = threads;
  n->team_ready = false;
  n->team_ok = true;
  return G4S_OK;
}

int g4s_net_get_block_threads(g4s_net *n, int32_t *threads) {
  if (!n || !threads) return set_error(G4S_ERR_INVALID, "null argument");
  const int rc = prepare_team(n);
  if (rc) return rc;
  *threads = n->team_nt_eff;
  return G4S_OK;
}

int g4s_net_get_geometry(g4s_net *n, int32_t *owner_blocks, int64_t *slice) {
  if (!n) return set_error(G4S_ERR_INVALID, "null handle");
  int rc = prepare_team(n);
  if (rc) return rc;
  const bool ok = n->team_ok && n->team_ready;
  if (owner_blocks) *owner_blocks = ok ? n->team_p : 0;
  if (slice) *slice = ok ? n->team_rc : 0;
  return G4S_OK;
}

int g4s_net_get_delivery(g4s_net *n, int32_t *delivery) {
  if (!n || !delivery) return set_error(G4S_ERR_INVALID, "null argument");
  const int rc = prepare_team(n);
  if (rc) return rc;
  *delivery = n->team_ok && n->team_ready && n->team_p > 1 ? deliver_mode_of(n) : kDeliverAuto;
  return G4S_OK;
}

int g4s_net_autotune(g4s_net *n, int32_t probe_steps, int32_t *algorithm, int32_t *team, double *us_per_step) {
  if (!n) return set_error(G4S_ERR_INVALID, "null handle");
  TuneChoice c;
  double us = 0.0;
  int rc = autotune(n, probe_steps, &c, &us);
  if (rc) return rc;
  if (algorithm) *algorithm = c.alg;
  if (team) *team = c.team;
  if (us_per_step) *us_per_step = us;
  return G4S_OK;
}

int g4s_nets_run(g4s_net **nets, const int32_t *steps, int32_t count, double *device_ms, int64_t *launches) {
  if (!nets || !steps) return set_error(G4S_ERR_INVALID, "null argument");
  return run_nets(nets, steps, count, device_ms, launches);
}

int g4s_net_reset(g4s_net *n) {
  if (!n) return set_error(G4S_ERR_INVALID, "null handle");
  return reset_net(n);
}

int g4s_net_run(g4s_net *n, int32_t steps, int32_t algorithm) {
  if (!n) return set_error(G4S_ERR_INVALID, "null handle");
  return run_net(n, steps, algorithm);
}

int g4s_net_get_info(g4s_net *n, g4s_net_info *info) {
  if (!n || !info) return set_error(G4S_ERR_INVALID, "null argument");
  info->n = n->v.n;
  info->nsyn = n->v.nsyn;
  info->stride = n->v.stride;
  info->steps_done = n->t_abs;
  info->total_spikes = n->total_spikes;
  info->raster_size = (int64_t)n->rt.size();
  info->last_run_ms = n->last_ms;
  info->last_run_wall_ms = n->last_wall_ms;
  info->last_run_spikes = n->last_spikes;
  info->last_algorithm = n->last_alg;
  info->persistent_blocks = persistent_blocks();
  info->device_bytes = (int64_t)n->device_bytes;
  info->last_run_kernel_ms = n->last_kernel_ms;
  info->last_run_launches = n->last_launches;
  return G4S_OK;
}

int g4s_pinned_alloc(uint64_t bytes, void **out) {
  if (!out) return set_error(G4S_ERR_INVALID, "null output pointer");
  *out = nullptr;
  G4S_CUDA(cudaMallocHost(out, bytes ? (size_t)bytes : 16));
  return G4S_OK;
}

int g4s_pinned_free(void *p) {
  if (p) G4S_CUDA(cudaFreeHost(p));
  return G4S_OK;
}

int g4s_net_raster(g4s_net *n, int32_t *t, int32_t *id, int64_t cap, int64_t *size) {
  if (!n) return set_error(G4S_ERR_INVALID, "null handle");
  const int64_t s = (int64_t)n->rt.size();
  if (size) *size = s;
  const int64_t m = std::min(s, cap);
  if (m > 0) {
    if (!t || !id) return set_error(G4S_ERR_INVALID, "null raster buffer");
    // large rasters on several host threads (a fresh destination is mostly page faults)
    const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    const int64_t parts = m >= ((int64_t)1 << 21) ? (int64_t)hw : 1, per = (m + parts - 1) / parts;
    auto part = [&](int64_t p) {
      const int64_t lo = p * per, hi = std::min(m, lo + per);
      if (lo >= hi) return;
      memcpy(t + lo, n->rt.data() + lo, (size_t)(hi - lo) * 4);
      memcpy(id + lo, n->rid.data() + lo, (size_t)(hi - lo) * 4);
    };
    std::vector<std::thread> pool;
    for (int64_t p = 1; p < parts; ++p) pool.emplace_back(part, p);
    part(0);
    for (auto &th : pool) th.join();
  }
  return G4S_OK;
}

int g4s_net_counts(g4s_net *n, int32_t *counts, int64_t cap, int64_t *size) {
  if (!n) return set_error(G4S_ERR_INVALID, "null handle");
  const int64_t s = (int64_t)n->counts.size();
  if (size) *size = s;
  const int64_t m = std::min(s, cap);
  if (m > 0) {
    if (!counts) return set_error(G4S_ERR_INVALID, "null counts buffer");
    memcpy(counts, n->counts.data(), (size_t)m * 4);
  }
  return G4S_OK;
}

int g4s_net_step_times(g4s_net *n, float *upd, float *step, int64_t cap, int64_t *size) {
  if (!n) return set_error(G4S_ERR_INVALID, "null handle");
  const int64_t s = (int64_t)n->upd_ms.size();
  if (size) *size = s;
  const int64_t m = std::min(s, cap);
  if (m > 0) {
    if (upd) memcpy(upd, n->upd_ms.data(), (size_t)m * 4);
    if (step) memcpy(step, n->step_ms.data(), (size_t)m * 4);
  }
  return G4S_OK;
}

int g4s_net_state(g4s_net *n, float *v, float *u, float *i_last, float *a, float *b, float *c, float *d,
                  int32_t *nospks) {
  if (!n) return set_error(G4S_ERR_INVALID, "null handle");
  const size_t N = (size_t)n->v.n;
  std::vector<float2> vu;
  std::vector<float4> p;
  std::vector<SpikeStat> ss;
  try {
    if (v || u) vu.resize(N);
    if (a || b || c || d) p.resize(N);
    if (nospks) ss.resize(N);
  } catch (...) {
    return set_error(G4S_ERR_NOMEM, "host staging");
  }
  if (v || u) G4S_CUDA(cudaMemcpyAsync(vu.data(), n->v.vu, N * 8, cudaMemcpyDeviceToHost, n->stream));
  if (a || b || c || d) G4S_CUDA(cudaMemcpyAsync(p.data(), n->v.abcd, N * 16, cudaMemcpyDeviceToHost, n->stream));
  if (nospks) G4S_CUDA(cudaMemcpyAsync(ss.data(), n->v.sstat, N * sizeof(SpikeStat), cudaMemcpyDeviceToHost, n->stream));
  if (i_last) G4S_CUDA(cudaMemcpyAsync(i_last, n->v.ilast, N * 4, cudaMemcpyDeviceToHost, n->stream));
  G4S_CUDA(cudaStreamSynchronize(n->stream));
  for (size_t i = 0; i < N; ++i) {
    if (v) v[i] = vu[i].x;
    if (u) u[i] = vu[i].y;
    if (a) a[i] = p[i].x;
    if (b) b[i] = p[i].y;
    if (c) c[i] = p[i].z;
    if (d) d[i] = p[i].w;
    if (nospks) nospks[i] = ss[i].nospks;
  }
  return G4S_OK;
}

int g4s_net_currents(g4s_net *n, int64_t *acc) {
  if (!n || !acc) return set_error(G4S_ERR_INVALID, "null argument");
  G4S_CUDA(cudaMemcpyAsync(acc, n->v.acc, (size_t)n->v.n * 8, cudaMemcpyDeviceToHost, n->stream));
  G4S_CUDA(cudaStreamSynchronize(n->stream));
  return G4S_OK;
}

int g4s_net_tables(g4s_net *n, int64_t row0, int64_t nrows, int32_t *idx, float *w) {
  if (!n) return set_error(G4S_ERR_INVALID, "null handle");
  if (row0 < 0 || nrows < 0 || row0 + nrows > n->v.n) return set_error(G4S_ERR_INVALID, "row range");
  const size_t off = (size_t)row0 * (size_t)n->v.stride, cnt = (size_t)nrows * (size_t)n->v.stride;
  if (idx) G4S_CUDA(cudaMemcpyAsync(idx, n->v.idx + off, cnt * 4, cudaMemcpyDeviceToHost, n->stream));
  if (w) G4S_CUDA(cudaMemcpyAsync(w, n->v.w + off, cnt * 4, cudaMemcpyDeviceToHost, n->stream));
  G4S_CUDA(cudaStreamSynchronize(n->stream));
  return G4S_OK;
}

int g4s_net_stats(g4s_net *n, double *rate_hz, double *isi_cv, int64_t *total_spikes) {
  if (!n) return set_error(G4S_ERR_INVALID, "null handle");
  double h[2] = {0, 0};
  G4S_CUDA(cudaMemsetAsync(n->d_stats, 0, 16, n->stream));
  G4S_CUDA(launch_stats(n->v, n->d_stats, n->stream));
  G4S_CUDA(cudaMemcpyAsync(h, n->d_stats, 16, cudaMemcpyDeviceToHost, n->stream));
  G4S_CUDA(cudaStreamSynchronize(n->stream));
  if (rate_hz) *rate_hz = n->t_abs ? (double)n->total_spikes * 1000.0 / ((double)n->v.n * (double)n->t_abs) : 0.0;
  if (isi_cv) *isi_cv = h[1] > 0 ? h[0] / h[1] : 0.0;
  if (total_spikes) *total_spikes = n->total_spikes;
  return G4S_OK;
}

int g4s_net_set_barrier_timeout(g4s_net *n, uint64_t ns) {
  if (!n) return set_error(G4S_ERR_INVALID, "null handle");
  n->barrier_ns = ns;
  return G4S_OK;
}

int g4s_inject_fault(g4s_net *n, int32_t kind) {
  if (kind == G4S_FAULT_ALLOC) {
    g_fail_next_alloc.store(1);
    return G4S_OK;
  }
  if (kind == G4S_FAULT_BARRIER_STALL) {
    if (!n) return set_error(G4S_ERR_INVALID, "null handle");
    n->barrier_stall = 1;
    return G4S_OK;
  }
  return set_error(G4S_ERR_INVALID, "unknown fault kind");
}

int g4s_net_destroy(g4s_net *n) {
  if (!n) return set_error(G4S_ERR_INVALID, "null handle");
  free_net(n);
  return G4S_OK;
}

int g4s_net_write_results(g4s_net *n, const char *dir, const float *init_state, double elapsed_ms,
                          double elapsed_with_data_ms) {
  (void)init_state;
  if (!n || !dir) return set_error(G4S_ERR_INVALID, "null argument");
  return write_results(n, dir, elapsed_ms, elapsed_with_data_ms);
}

int g4s_run_protocol(int32_t n, int32_t nsyn, int32_t iterations, int32_t algorithm, int32_t mode, uint64_t seed,
                     int32_t conn_law, const char *results_root) {
  if (!results_root) return set_error(G4S_ERR_INVALID, "null results root");
  if (iterations < 0) return set_error(G4S_ERR_INVALID, "iterations must be >= 0");
  if (algorithm < -1 || algorithm > kAlgAuto) return set_error(G4S_ERR_INVALID, "algorithm must be -1..5");
  if (mode < -1 || mode > 2) return set_error(G4S_ERR_INVALID, "mode must be -1..2");
  g4s_net_desc d{};
  d.n = n;
  d.nsyn = nsyn;
  d.exc_permille = 800;
  d.self_loops = conn_law == G4S_CONN_GLIBC ? 1 : 0;
  d.conn_law = conn_law;
  d.seed = seed;
  d.drive_scale = 1.0f;
  d.record_raster = 1;
  g4s_net *net = nullptr;
  int rc = g4s_net_create(&d, &net);
  if (rc) return rc;
  static const float kModeScale[3] = {0.5f, 1.0f, 1.5f};
  for (int m = 0; m < 3; ++m) {
    if (mode >= 0 && m != mode) continue;
    for (int a = 0; a < 5; ++a) {
      const int alg = algorithm < 0 ? a : algorithm;
      if (algorithm >= 0 && a > 0) break;
      net->desc.drive_scale = kModeScale[m];
      if ((rc = reset_net(net))) break;
      char sub[256];
      snprintf(sub, sizeof sub, "/Results/N%dNsyn%dRegime%dAlg%d/", n, nsyn, m, alg);
      const auto w0 = std::chrono::steady_clock::now();
      if ((rc = run_net(net, iterations, alg))) break;
      const double ewd = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - w0).count();
      if ((rc = write_results(net, std::string(results_root) + sub, net->last_ms, ewd))) break;
      printf("Regime %d Alg %d: %d steps, %lld spikes, %.3f ms device, %.3f ms with data\n", m, alg, iterations,
             (long long)net->total_spikes, net->last_ms, ewd);
    }
    if (rc) break;
  }
  g4s_net_destroy(net);
  return rc;
}

int g4s_conn_glibc(uint32_t seed, int32_t n, int32_t nsyn, int32_t stride, int32_t *idx, float *w) {
  if (!idx || !w) return set_error(G4S_ERR_INVALID, "null table buffer");
  return conn_glibc_host(seed, n, nsyn, stride, idx, w);
}

int g4s_net_stream_raster(g4s_net *n, const char *path) {
  if (!n) return set_error(G4S_ERR_INVALID, "null handle");
  if (n->rstream) {
    RasterFile *f = n->rstream;
    n->rstream = nullptr;
    int rc = raster_close(f);
    if (rc) return rc;
  }
  if (!path) return G4S_OK;
  if (!n->desc.record_raster) return set_error(G4S_ERR_STATE, "the raster is not recorded (record_raster = 0)");
  return raster_open(path, n->v.n, n->t_abs, &n->rstream);
}

int g4s_net_write_raster_file(g4s_net *n, const char *path) {
  if (!n || !path) return set_error(G4S_ERR_INVALID, "null argument");
  if (n->rid.size() != (size_t)n->total_spikes || n->counts.size() != (size_t)n->t_abs)
    return set_error(G4S_ERR_STATE, "the host raster does not hold every step since the reset "
                                    "(not recorded, or streamed to a file)");
  return raster_write_all(path, n->v.n, 0, n->counts, n->rid);
}

int g4s_net_save_tables(g4s_net *n, const char *path) {
  if (!n || !path) return set_error(G4S_ERR_INVALID, "null argument");
  const size_t cnt = (size_t)n->v.n * (size_t)n->v.stride;
  std::vector<int32_t> idx;
  std::vector<float> w;
  try {
    idx.resize(cnt);
    w.resize(cnt);
  } catch (...) {
    return set_error(G4S_ERR_NOMEM, "host tables");
  }
  int rc = g4s_net_tables(n, 0, n->v.n, idx.data(), w.data());
  if (rc) return rc;
  TableHeader h{};
  h.n = n->v.n;
  h.nsyn = n->v.nsyn;
  h.stride = n->v.stride;
  h.seed = n->desc.seed;
  h.conn_law = n->desc.conn_law;
  h.self_loops = n->desc.self_loops;
  h.exc_permille = n->desc.exc_permille;
  h.flags = 1;
  return tables_write(path, h, idx.data(), w.data());
}

int g4s_net_create_from_file(const g4s_net_desc *desc, const char *path, g4s_net **out) {
  if (!desc || !path || !out) return set_error(G4S_ERR_INVALID, "null argument");
  *out = nullptr;
  TableHeader h{};
  int rc = tables_read_header(path, &h);
  if (rc) return rc;
  if (h.n != desc->n || h.nsyn != desc->nsyn)
    return set_error(G4S_ERR_INVALID, std::string(path) + " holds a network of n=" + std::to_string(h.n) +
                                          ", nsyn=" + std::to_string(h.nsyn));
  const size_t cnt = (size_t)h.n * (size_t)h.stride;
  std::vector<int32_t> idx;
  std::vector<float> w;
  try {
    idx.resize(cnt);
    w.resize(cnt);
  } catch (...) {
    return set_error(G4S_ERR_NOMEM, "host tables");
  }
  if ((rc = tables_read(path, h, idx.data(), w.data()))) return rc;
  return g4s_net_create_from_tables(desc, idx.data(), w.data(), h.stride, out);
}

}  // extern "C"

namespace g4s {
int net_create_pooled(const g4s_net_desc *desc, cudaMemPool_t pool, g4s_net **out) {
  return create_net(desc, pool, out);
}
}  // namespace g4s
