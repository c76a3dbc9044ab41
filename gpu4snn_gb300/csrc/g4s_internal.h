// g4s_internal.h — declarations shared by the host library's translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "g4s_types.h"

struct g4s_net;  // the handle of the C ABI
struct g4s_net_desc;

namespace g4s {

// Propagation schemes, numbered as the reference's `dynamic` (gpu4snn.cu:1083).
constexpr int kAlgAP = 0;
constexpr int kAlgN = 1;
constexpr int kAlgS = 2;
constexpr int kAlgAB = 3;
constexpr int kAlgSKL = 4;
constexpr int kAlgAuto = 5;

// Launch shape of a delivery scheme (the autotuner's output).
struct DeliverShape {
  int k_hint = 0;         // S: expected spikes per step, sizes the oversubscribed grid
  int group = 0;          // AP and SKL: threads per spiking row (0 = flat split for SKL)
  int blocks_per_sm = 4;  // AP and AB: resident blocks per SM
};

cudaError_t launch_init(const NetView &v, cudaStream_t s);
cudaError_t launch_conngen(const NetView &v, int self_loops, cudaStream_t s);
// t0: device word holding the absolute step of the chunk's step 0
cudaError_t launch_update(const NetView &v, const long long *t0, int lt, bool last, cudaStream_t s);
cudaError_t launch_deliver(const NetView &v, int lt, int alg, const DeliverShape &sh, cudaStream_t s);
cudaError_t launch_persistent(const NetView &v, int64_t t_abs0, int nsteps, bool last_chunk, GridSync *gs,
                              unsigned long long limit_ns, int group, int stall, cudaStream_t s);
cudaError_t launch_stats(const NetView &v, double *out, cudaStream_t s);
int persistent_blocks();

// SKL team kernel (g4s_team.cu).
constexpr int kMaxSortedNsyn = 16384;          // rows are sorted in shared memory
constexpr size_t kTeamSmemLimit = 200 * 1024;  // shared memory per CTA for currents + spikes
constexpr int64_t kPrezSlice = 12288;          // slices up to this size precompute the next drive
constexpr int64_t kVuSlice = 2048;             // ... keep v, u in shared memory for the whole launch
constexpr int64_t kAbcdSlice = 2048;           // ... keep a, b, c, d in shared memory (larger slices
                                               // keep them in global memory: the L1 left by a larger
                                               // shared-memory carve-out holds fewer table loads in flight)
constexpr int64_t kSoloSlice = 128;            // neurons per CTA of a network running alone (at
                                               // most: it spreads over every SM; measured best from
                                               // N = 2500 to 10^6)
constexpr int64_t kBatchSlice = 8192;          // neurons per CTA of a batched network (measured on the
                                               // 256-network ensemble: 510 ms against 534 at 4096 and
                                               // 824 at 16384; served requests 41.9/s, 40.1, 32.7)
constexpr int kStepGraphSteps = 512;          // longest chunk of the host-driven schemes (one CUDA graph)
constexpr int kStepGraphs = 4;                 // captured chunks kept per network
constexpr int kMaxTeam = 192;                  // CTAs of one team (three record slots per thread)
constexpr int kMinWindow = 1024;               // spike ids a multi-CTA rank can stage per delivery window
constexpr int kMaxWindow = 4096;
constexpr int kFlatMax = 8192;                 // synapses of a step a rank delivers flat (else by runs)
constexpr int64_t kFlatSlice = 4096;           // ... on slices up to this size
// Spike records of a multi-CTA team: per rank and step parity kRecLines lines of 16
// tagged 64-bit words (count, then up to 16 kRecLines - 1 ids); readers fetch the second
// line of a rank only if it had enough spikes in the previous step (g4s_team.cu).
constexpr int kRecLines = 2;
constexpr int kRecWords = 16;

// Shared-memory layout of one team rank (byte offsets; the optional arrays are present
// when their flag is set).  `cap` is the delivery window of a multi-CTA team (0 for one CTA).
struct TeamLayout {
  unsigned abcd, vu, a, b, own, z, cnt, off, xoff, inl, pay, spk, sb, pre, ex, wsum, bytes;
  bool abcd_sm, vu_sm, prez, flat;
};
__host__ __device__ inline unsigned team_align16(size_t x) { return (unsigned)((x + 15) & ~(size_t)15); }
__host__ __device__ inline TeamLayout team_layout(int64_t rc, int team, int cap) {
  TeamLayout L{};
  L.abcd_sm = rc <= kAbcdSlice;
  L.vu_sm = rc <= kVuSlice;
  L.prez = rc <= kPrezSlice;
  L.flat = team > 1 && rc <= kFlatSlice;
  size_t o = 0;
  L.abcd = (unsigned)o;
  if (L.abcd_sm) o += (size_t)rc * 16;
  L.vu = (unsigned)o;
  if (L.vu_sm) o += (size_t)rc * 8;
  L.a = (unsigned)o;
  o = team_align16(o + (size_t)rc * 4);
  L.b = (unsigned)o;
  o = team_align16(o + (size_t)rc * 4);
  L.own = (unsigned)o;
  o = team_align16(o + (size_t)rc * 4);
  L.z = (unsigned)o;
  if (L.prez) o = team_align16(o + (size_t)rc * 4);
  L.cnt = L.off = L.xoff = L.inl = L.pay = L.spk = L.sb = L.pre = L.ex = L.wsum = (unsigned)o;
  if (team > 1) {
    L.cnt = (unsigned)o;  // spikes per rank
    o = team_align16(o + (size_t)(team + 1) * 4);
    L.off = (unsigned)o;  // their offsets in the step's list
    o = team_align16(o + (size_t)(team + 1) * 4);
    L.xoff = (unsigned)o;  // offsets of the ids not in the lines read by the first pass
    o = team_align16(o + (size_t)(team + 1) * 4);
    L.inl = (unsigned)o;  // ids of each rank in the lines read by the first pass
    o = team_align16(o + (size_t)(team + 1) * 4);
    L.pay = (unsigned)o;  // payloads of the record lines
    o = team_align16(o + (size_t)team * kRecLines * kRecWords * 4);
    L.spk = (unsigned)o;  // the delivery window: spike ids of the step
    o = team_align16(o + (size_t)cap * 4);
    L.sb = L.pre = L.ex = L.wsum = (unsigned)o;
  }
  if (L.flat) {
    L.sb = (unsigned)o;  // flat delivery: first slot of each spike's segment
    o = team_align16(o + (size_t)cap * 2);
    L.pre = (unsigned)o;  // ... offset of each spike's segment in the concatenation
    o = team_align16(o + (size_t)(cap + 1) * 4);
    L.ex = (unsigned)o;  // ... spike of every synapse of the concatenation
    o = team_align16(o + (size_t)kFlatMax * 2);
    L.wsum = (unsigned)o;  // ... per-warp sums of the scan
    o = team_align16(o + 33 * 4);
  }
  L.bytes = (unsigned)o;
  return L;
}
// Delivery window of a multi-CTA rank: what is left of the shared-memory limit, at most
// kMaxWindow ids; 0 if less than kMinWindow is left (the geometry does not fit).
inline int team_window(int64_t rc, int team) {
  if (team <= 1) return 0;
  const size_t kPerId = rc <= kFlatSlice ? 4 + 2 + 4 : 4;  // id (segment start, segment offset)
  const size_t base = team_layout(rc, team, 0).bytes + 64;  // + alignment of the arrays
  if (base + (size_t)kMinWindow * kPerId > kTeamSmemLimit) return 0;
  const size_t cap = (kTeamSmemLimit - base) / kPerId;
  return (int)(cap > (size_t)kMaxWindow ? kMaxWindow : cap & ~(size_t)7);
}
// Rows sorted by target (unsigned, so unused slots last), equal targets by weight bits;
// generated = rows as the connectivity kernel writes them (distinct targets, unused slots
// (-1, 0.0f)), which a narrower key sorts into the same order.
cudaError_t launch_sort_rows(const NetView &v, bool generated, cudaStream_t s);
// *unsorted <- 1 if some row is not in launch_sort_rows' order, else 0
cudaError_t launch_rows_sorted(const NetView &v, int *unsorted, cudaStream_t s);
// A launch over many networks: clear (before it) and pack (after it) every network's
// per-launch words; network i's share of the pack is round_pack_bytes(steps_i) bytes at
// off[i]: status word, team error word, counts, raster offsets, stamps.
inline size_t round_pack_bytes(int steps) { return 8 + (((size_t)steps * 4 + 7) & ~(size_t)7) + (size_t)steps * 24; }
cudaError_t launch_round_clear(const TeamItem *items, int count, cudaStream_t s);
cudaError_t launch_round_gather(const TeamItem *items, const int64_t *off, int count, unsigned char *pack,
                                cudaStream_t s);
cudaError_t launch_segoff(const NetView &v, int team, int64_t rc, uint16_t *seg, cudaStream_t s);
// out (3 words): the largest in-degree, the largest sum(|q| >> 16) + 1 over a neuron's
// inputs (with mag, n words of scratch; else 0), the largest (|q| >> 16) + 1 (without mag)
cudaError_t launch_inbound(const NetView &v, unsigned *cnt, unsigned long long *mag, unsigned long long *out,
                           cudaStream_t s);
// team_max_blocks also raises the kernel's shared-memory ceiling: call it once before the
// first launch_team (which may then be captured in a CUDA graph)
// Threads per CTA of the team kernel: 1024 (the default; the most reads in flight) or 768
// (80 registers a thread instead of 64: no spills, faster when a step's work is small).
constexpr int kTeamNT = 1024;
constexpr int kTeamNTSmall = 768;
// pair: the tables are read from v.pair (interleaved rows) instead of v.idx and v.w;
// nt: kTeamNT or kTeamNTSmall threads per CTA
cudaError_t launch_team(const TeamItem *items, const int2 *slots, const int *nslots, int *slot_head, int grid,
                        size_t smem, unsigned long long limit_ns, int stall, cudaStream_t s, bool pair,
                        int nt = kTeamNT);
// v.pair <- the rows of v.idx and v.w interleaved (after every change of the tables)
cudaError_t launch_pairs(const NetView &v, cudaStream_t s);
cudaError_t team_max_blocks(size_t smem, int *out, int nt = kTeamNT);
// mean duration in ms of the last k simulated steps of a handle with a step time (0: none)
double net_recent_step_ms(const g4s_net *n, int64_t k);
// the team kernel's team-independent buffers of a handle (its interleaved rows and spike
// lists), made ready ahead of its first team run; nothing for tables the kernel cannot run
int net_prepare_rows(g4s_net *n);
// g4s_net_create with the handle's device memory from a stream-ordered pool (a server's)
int net_create_pooled(const g4s_net_desc *desc, cudaMemPool_t pool, g4s_net **out);
cudaError_t team_smem_ceiling();  // the part of team_max_blocks that launch_team needs
// shared memory of one rank of a team of `team` CTAs with `rc` neurons each (0: does not fit)
size_t team_smem(int64_t rc, int team);

// A handle's arrays, stream and absolute step, for the library's other translation units
// (the on-device FP64 check, g4s_fp64check.cu).
const NetView &net_view(const g4s_net *n);
cudaStream_t net_stream(const g4s_net *n);
int64_t net_steps_done(const g4s_net *n);
// CTAs of the team the handle's last planned geometry uses (solo or batched), without
// planning anything (1 when no team geometry is planned)
int net_team_size(const g4s_net *n);

// Binary files (g4s_formats.cu): the raster, streamed by a writer thread, and the tables.
struct RasterFile;
int raster_open(const char *path, int64_t n, int64_t t0, RasterFile **out);
void raster_push(RasterFile *f, const int32_t *counts, int cs, const int32_t *ids, int64_t nids);
int raster_close(RasterFile *f);
int raster_write_all(const char *path, int64_t n, int64_t t0, const std::vector<int32_t> &counts,
                     const std::vector<int32_t> &ids);
struct TableHeader {
  int64_t n;
  int32_t nsyn, stride;
  uint64_t seed;
  int32_t conn_law, self_loops, exc_permille, flags;  // flags: 1 = rows sorted by target
  int32_t pad[2];
};
int tables_write(const char *path, const TableHeader &h, const int32_t *idx, const float *w);
int tables_read_header(const char *path, TableHeader *h);
int tables_read(const char *path, const TableHeader &h, int32_t *idx, float *w);

// Error reporting (thread-local message behind g4s_last_error()).
int set_error(int code, const std::string &msg);
int cuda_error(cudaError_t e, const char *what);

// Host generator of the reference's glibc-rand tables (gpu4snn.cu:873-898).
int conn_glibc_host(unsigned seed, int32_t n, int32_t nsyn, int32_t stride, int32_t *idx, float *w);

}  // namespace g4s
