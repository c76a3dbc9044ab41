// g4s_internal.h — declarations shared by the host library's translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "g4s_types.h"

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
cudaError_t launch_update(const NetView &v, int64_t t_abs0, int lt, bool last, cudaStream_t s);
cudaError_t launch_deliver(const NetView &v, int lt, int alg, const DeliverShape &sh, cudaStream_t s);
cudaError_t launch_persistent(const NetView &v, int64_t t_abs0, int nsteps, bool last_chunk, GridSync *gs,
                              unsigned long long limit_ns, int group, int stall, cudaStream_t s);
cudaError_t launch_stats(const NetView &v, double *out, cudaStream_t s);
int persistent_blocks();

// SKL team kernel (g4s_team.cu).
constexpr int kMaxSortedNsyn = 16384;          // rows are sorted in shared memory
constexpr size_t kTeamSmemLimit = 200 * 1024;  // shared memory per CTA for currents + spikes
constexpr int64_t kPrezSlice = 12288;          // slices up to this size precompute the next drive
constexpr int64_t kSoloSlice = 2048;           // neurons per CTA of a network running alone
constexpr int64_t kBatchSlice = 2048;          // neurons per CTA of a batched network (measured: fewer,
                                               // larger slices made the config-4 ensemble 1.4x slower)
cudaError_t launch_sort_rows(const NetView &v, cudaStream_t s);
cudaError_t launch_segoff(const NetView &v, int team, int64_t rc, uint16_t *seg, cudaStream_t s);
cudaError_t launch_inbound(const NetView &v, unsigned *cnt, unsigned long long *mag, unsigned long long *out,
                           cudaStream_t s);
cudaError_t launch_team(const TeamItem *items, const int2 *slots, const int *nslots, int *slot_head, int grid,
                        size_t smem, unsigned long long limit_ns, int stall, cudaStream_t s);
cudaError_t team_max_blocks(size_t smem, int *out);
size_t team_smem(int64_t rc);

// Error reporting (thread-local message behind g4s_last_error()).
int set_error(int code, const std::string &msg);
int cuda_error(cudaError_t e, const char *what);

// Host generator of the reference's glibc-rand tables (gpu4snn.cu:873-898).
int conn_glibc_host(unsigned seed, int32_t n, int32_t nsyn, int32_t stride, int32_t *idx, float *w);

}  // namespace g4s
