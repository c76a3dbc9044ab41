// g4s_noalloc.cu — g4s_run_noalloc: the SKL team kernel on caller-owned device arrays,
// without any allocation.
//
// Some callers cannot call cudaMalloc while they step a network: real-time loops that
// must not pay the device-wide synchronisation an allocation or a free may imply, and
// hosts whose device memory is owned by a capped pool that this library cannot draw
// from.  For them this entry point uses only memory it already has: the caller passes the
// network's arrays and the output buffers, and the kernel's scratch (the team's per-step
// spike records and overflow ids, the per-row segment table of a multi-CTA team, the error
// word and the work-queue words) lives in one file-scope __device__ array of fixed size,
// which every GPU that loads the library holds until the process exits.  The call copies
// nothing from host memory: the launch descriptor reaches the device as a kernel argument.
//
// Limits: at most kNoAllocMaxNeurons neurons and kNoAllocMaxTeam CTAs, and at most 16384
// neurons per CTA (the shared-memory slice of the team kernel).  Every call shares the
// scratch array and leaves its contents behind; calls that overlap on the GPU (on
// different streams, or without ordering between them) race on it and must not be made.
// A multi-CTA call rebuilds the per-row segment table from the caller's tables (a binary
// search of every row per team boundary, reading about team x log2(stride) targets a row),
// since it cannot know whether they changed since the last call.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/gpu4snn.h"
#include "g4s_internal.h"

using namespace g4s;

namespace {

constexpr int64_t kNoAllocMaxNeurons = 131072;
constexpr int kNoAllocMaxTeam = 8;
constexpr int64_t kNoAllocMaxSlice = 16384;

// Layout of the scratch array.
constexpr size_t kOffSync = 0;                                       // GridSync (128 B): error word
constexpr size_t kOffRec = 128;                                      // spike records: [2][team][4 x 16] u64
constexpr size_t kOffCtl = kOffRec + 2 * kNoAllocMaxTeam * kRecLines * 128;  // int[4]: slot count, queue head, status
constexpr size_t kOffSlots = kOffCtl + 128;                          // int2[kNoAllocMaxTeam]
constexpr size_t kOffItem = kOffSlots + 256;                         // TeamItem
constexpr size_t kOffList = 16384;                                   // u64[4][kNoAllocMaxNeurons]: overflow, dense ids
constexpr size_t kOffSeg = kOffList + 4 * kNoAllocMaxNeurons * 8;  // u16[kNoAllocMaxNeurons][kNoAllocMaxTeam + 1]
constexpr size_t kScratchBytes = kOffSeg + (size_t)kNoAllocMaxNeurons * (kNoAllocMaxTeam + 1) * 2;

static_assert(sizeof(GridSync) <= kOffRec - kOffSync, "error word");
static_assert(sizeof(int2) * kNoAllocMaxTeam <= kOffItem - kOffSlots, "slots");
static_assert(sizeof(TeamItem) <= kOffList - kOffItem, "item");
static_assert(kNoAllocMaxTeam <= 32, "one setup thread per slot");
// about 6.5 MB: the documented size of the array in gpu4snn.h
static_assert(kScratchBytes > 6400000 && kScratchBytes < 6600000, "scratch size as documented");

// Writes the work-queue words, the team's slots and the launch descriptor into the
// scratch array.  The descriptor arrives by value as a kernel argument, so the call stages
// nothing through host memory.
__global__ void k_noalloc_setup(TeamItem item, int *ctl, int2 *slots, TeamItem *dst) {
  const int r = threadIdx.x;
  if (r < item.team) slots[r] = make_int2(0, r);
  if (r == 0) {
    ctl[0] = item.team;  // slots in the queue
    ctl[1] = 0;          // queue head
    ctl[2] = 0;          // status word
    *dst = item;
  }
}

}  // namespace

// The scratch of g4s_run_noalloc (about 6.5 MB per GPU, held until exit).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// In host code g_noalloc_scratch names a host-side stand-in, not device memory: its
// device address is looked up once per device, with that device current, and cached.
static std::mutex g_scratch_mu;
static void *g_scratch_dev[256];

static int scratch_address(unsigned char **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
  if (dev < 0 || dev >= 256) return set_error(G4S_ERR_CUDA, "device index out of range");
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_dev[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return cuda_error(e, "cudaGetSymbolAddress of the no-alloc scratch");
    // once per device, outside any stream capture of the caller's launches
    if ((e = team_smem_ceiling()) != cudaSuccess) return cuda_error(e, "team kernel shared-memory ceiling");
    g_scratch_dev[dev] = p;
  }
  *out = static_cast<unsigned char *>(g_scratch_dev[dev]);
  return G4S_OK;
}

extern "C" int g4s_run_noalloc(const g4s_dev_net *d, int64_t t_abs0, int32_t steps, int32_t team, int32_t last,
                               int32_t *d_counts, int64_t *d_base, int32_t *d_raster, int64_t raster_cap,
                               int32_t *d_status, void *stream) {
  if (!d) return set_error(G4S_ERR_INVALID, "null network");
  if (d->n < 2 || d->n > kNoAllocMaxNeurons)
    return set_error(G4S_ERR_INVALID, "g4s_run_noalloc: n must be in [2, " + std::to_string(kNoAllocMaxNeurons) +
                                          "], got " + std::to_string(d->n));
  if (team < 1 || team > kNoAllocMaxTeam)
    return set_error(G4S_ERR_INVALID, "g4s_run_noalloc: team must be in [1, " + std::to_string(kNoAllocMaxTeam) +
                                          "], got " + std::to_string(team));
  const int64_t rc = (d->n + team - 1) / team;
  if (rc > kNoAllocMaxSlice || team_smem(rc, team) == 0)
    return set_error(G4S_ERR_INVALID, "g4s_run_noalloc: more than " + std::to_string(kNoAllocMaxSlice) +
                                          " neurons per CTA; use a larger team");
  if (d->nsyn < 1 || d->stride < d->nsyn || d->stride % 4 != 0 || d->stride > kMaxSortedNsyn)
    return set_error(G4S_ERR_INVALID, "g4s_run_noalloc: need 1 <= nsyn <= stride <= 16384, stride % 4 == 0");
  if (d->nexc < 0 || d->nexc > d->n) return set_error(G4S_ERR_INVALID, "g4s_run_noalloc: bad nexc");
  if (steps < 0 || t_abs0 < 0 || t_abs0 + steps > (int64_t)INT32_MAX)
    return set_error(G4S_ERR_INVALID, "g4s_run_noalloc: bad step range");
  if (!d->vu || !d->abcd || !d->acc || !d->i_last || !d->spike_stat || !d->idx || !d->w)
    return set_error(G4S_ERR_INVALID, "g4s_run_noalloc: null network array");
  if (steps > 0 && (!d_counts || !d_base)) return set_error(G4S_ERR_INVALID, "g4s_run_noalloc: null counts/base");
  if (raster_cap < 0 || (raster_cap > 0 && !d_raster))
    return set_error(G4S_ERR_INVALID, "g4s_run_noalloc: bad raster buffer");
  if (steps == 0) return G4S_OK;

  unsigned char *scr = nullptr;
  int rc0 = scratch_address(&scr);
  if (rc0) return rc0;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  GridSync *sync = reinterpret_cast<GridSync *>(scr + kOffSync);
  int *ctl = reinterpret_cast<int *>(scr + kOffCtl);
  int2 *slots = reinterpret_cast<int2 *>(scr + kOffSlots);
  TeamItem *item = reinterpret_cast<TeamItem *>(scr + kOffItem);
  unsigned long long *list = reinterpret_cast<unsigned long long *>(scr + kOffList);
  uint16_t *seg = reinterpret_cast<uint16_t *>(scr + kOffSeg);

  TeamItem h{};
  NetView &v = h.v;
  v.n = d->n;
  v.nexc = d->nexc;
  v.nsyn = d->nsyn;
  v.stride = d->stride;
  v.seed = d->seed;
  v.ge = d->ge;
  v.gi = d->gi;
  v.vu = static_cast<float2 *>(d->vu);
  v.abcd = static_cast<float4 *>(d->abcd);
  v.acc = reinterpret_cast<long long *>(d->acc);
  v.ilast = d->i_last;
  v.sstat = static_cast<SpikeStat *>(d->spike_stat);
  v.idx = d->idx;
  v.w = d->w;
  v.raster = d_raster;
  v.raster_cap = raster_cap;
  v.counts = d_counts;
  v.base = reinterpret_cast<long long *>(d_base);
  v.stamps = nullptr;
  v.status = ctl + 2;
  h.seg = seg;
  h.list = list;
  h.rec = reinterpret_cast<unsigned long long *>(scr + kOffRec);
  h.cap = team_window(rc, team);
  h.tag0 = 0;
  h.t_abs0 = t_abs0;
  h.steps = steps;
  h.last = last ? 1 : 0;
  h.team = team;
  h.rc = (int)rc;
  h.sync = sync;
  // Everything that must start at zero: error word, spike records and overflow ids (their
  // tags restart with every call), step counts; then the queue words and the descriptor.
  cudaError_t e = cudaMemsetAsync(scr, 0, kOffSlots, s);
  if (e == cudaSuccess && team > 1) e = cudaMemsetAsync(list, 0, (size_t)d->n * 4 * sizeof(unsigned long long), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_counts, 0, (size_t)steps * sizeof(int32_t), s);
  if (e == cudaSuccess) {
    k_noalloc_setup<<<1, 32, 0, s>>>(h, ctl, slots, item);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && team > 1) e = launch_segoff(v, team, rc, seg, s);
  if (e == cudaSuccess)
    e = launch_team(item, slots, ctl, ctl + 1, team, team_smem(rc, team), 2000000000ull, 0, s, false);
  if (e == cudaSuccess && d_status) e = cudaMemcpyAsync(d_status, &sync->error, sizeof(int32_t), cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return cuda_error(e, "g4s_run_noalloc launch");
  return G4S_OK;
}
