// g4s_kernels.cu — sm_103a kernels of one network's simulation step, and their launchers.
//
//   k_init_state   neuron parameters and initial state        (initNeuron, gpu4snn.cu:286-320)
//   k_conngen      distinct-target tables, Philox law          (host generator, gpu4snn.cu:873-905)
//   k_update       update fused with spike compaction          (stateupdate, gpu4snn.cu:334-417)
//   k_deliver_*    spike delivery, four schemes:
//                    N  thread per spiking neuron              (deliverspks1, gpu4snn.cu:420-443)
//                    S  thread per 4 synapses, oversubscribed  (deliverspks2, gpu4snn.cu:446-467)
//                    AP thread group per spiking row           (propagatespikes, gpu4snn.cu:323-331)
//                    AB persistent grid over the synapse range (AB_deliverspks, gpu4snn.cu:554-584)
//   k_persistent   all steps of a chunk in one cooperative launch with timed grid barriers
//                                                              (SKL_deliverspks, gpu4snn.cu:669-716)
//   k_stats        FP64 firing rate and ISI CV reductions
//
// Delivery reads the compacted spike list of the step (int32 ids), streams each spiking row
// with 128-bit evict-first loads (int32 targets, fp32 weights) and adds Q32.32 weights into
// the L2-resident current array with red.global.add.u64, so the result does not depend on
// the order of the additions.
#include <cuda_runtime.h>

#include <algorithm>

#include <cstdio>

#include "g4s_device.cuh"
#include "g4s_internal.h"

namespace g4s {

// ---------------------------------------------------------------------------------------
// Initial state.
// ---------------------------------------------------------------------------------------
__global__ void k_init_state(NetView v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < v.n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float r = izh_r(v.seed, i);
    const float4 p = izh_abcd(r, i < v.nexc);
    v.abcd[i] = p;
    if (v.rpar) v.rpar[i] = r;
    v.vu[i] = make_float2(-65.0f, __fmul_rn(p.y, -65.0f));
    v.acc[i] = 0;
    v.ilast[i] = 0.0f;
    SpikeStat s;
    s.nospks = 0;
    s.last = -1;
    s.nisi = 0;
    s.pad = 0;
    s.s1 = 0;
    s.s2 = 0;
    v.sstat[i] = s;
  }
}

// ---------------------------------------------------------------------------------------
// Connectivity.  One warp per row keeps the row's accepted targets in a shared-memory set:
// a bitmap of the n targets when that is the smaller (bits > 0 words), else an
// open-addressing hash of 2^log2h ints.  Draws are consumed in the order the oracle
// defines: block b, word r, lane l is draw 128b + 32r + l.  Within one word round, a draw
// is fresh iff its target is not in the set and no lower lane drew the same target
// (__match_any_sync: only the lowest such lane inserts); fresh draws are accepted in lane
// order until the row holds nsyn targets.
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ bool set_insert(int *set, unsigned mask, int log2h, int t) {
  unsigned h = ((unsigned)t * 0x9E3779B1u) >> (32 - log2h);
  for (unsigned probe = 0; probe <= mask; ++probe) {
    const int old = atomicCAS(set + h, -1, t);
    if (old == -1) return true;
    if (old == t) return false;
    h = (h + 1) & mask;
  }
  return false;  // unreachable: the set is sized for twice the row plus one round
}

__device__ __forceinline__ bool bit_insert(int *bits, int t) {
  const unsigned b = 1u << (t & 31);
  return (atomicOr(reinterpret_cast<unsigned *>(bits) + (t >> 5), b) & b) == 0u;
}

__global__ void k_conngen(NetView v, int self_loops, int log2h, int bits, int64_t row0, int64_t nrows,
                          unsigned long long max_blocks) {
  extern __shared__ __align__(16) int s_set[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  const unsigned hsize = 1u << log2h, mask = hsize - 1;
  const unsigned words = bits > 0 ? (unsigned)bits : hsize;  // (a multiple of 4)
  int *set = s_set + (size_t)wib * words;
  const int fill = bits > 0 ? 0 : -1;
  const uint64_t range = self_loops ? (uint64_t)v.n : (uint64_t)(v.n - 1);
  const float wscale = __fdiv_rn(1000.0f, (float)v.nsyn);
  for (int64_t rr = (int64_t)blockIdx.x * wpb + wib; rr < nrows; rr += (int64_t)gridDim.x * wpb) {
    const int64_t row = row0 + rr;
    int *ri = const_cast<int *>(v.idx) + row * v.stride;
    float *rw = const_cast<float *>(v.w) + row * v.stride;
    for (unsigned j = lane; j < words / 4; j += 32) reinterpret_cast<int4 *>(set)[j] = make_int4(fill, fill, fill, fill);
    __syncwarp();
    int accepted = 0;
    for (unsigned long long b = 0; accepted < v.nsyn; ++b) {
      if (b >= max_blocks) {
        if (lane == 0) atomicCAS(v.status, 0, kErrConnCode);
        break;
      }
      const U64x4 o = philox(v.seed, kStreamConn, (uint64_t)row, 32ull * b + lane, 0);
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        uint64_t t = __umul64hi(o.x[r], range);
        if (!self_loops && t >= (uint64_t)row) t += 1;
        const int ti = (int)t;
        const unsigned same = __match_any_sync(0xFFFFFFFFu, ti);
        const bool leader = (__ffs(same) - 1) == lane;
        bool fresh = false;
        if (leader) fresh = bits > 0 ? bit_insert(set, ti) : set_insert(set, mask, log2h, ti);
        const unsigned fb = __ballot_sync(0xFFFFFFFFu, fresh);
        const int pos = accepted + __popc(fb & ((1u << lane) - 1u));
        if (fresh && pos < v.nsyn) ri[pos] = ti;
        accepted += __popc(fb);
        __syncwarp();
        if (accepted >= v.nsyn) break;
      }
    }
    const float sc = row < v.nexc ? __fmul_rn(wscale, 0.5f) : __fmul_rn(wscale, -1.0f);
    for (int j = lane * 4; j < v.nsyn; j += 128) {
      const U64x4 o = philox(v.seed, kStreamWeight, (uint64_t)row, (uint64_t)(j >> 2), 0);
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (j + q < v.nsyn) rw[j + q] = __fmul_rn(sc, u24(o.x[q]));
    }
    for (int j = v.nsyn + lane; j < v.stride; j += 32) {
      ri[j] = -1;
      rw[j] = 0.0f;
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------------------
// Update of one neuron; returns its spike flag.  Writes the current back only when it was
// non-zero, and the spike statistics only on a spike.
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ bool update_one(const NetView &v, int64_t i, int64_t t_abs, bool last) {
  float2 s = v.vu[i];
  const float4 p = v.abcd[i];
  const long long a = __ldcg(v.acc + i);
  const float g = i < v.nexc ? v.ge : v.gi;
  const float z = normal(v.seed, (uint64_t)i, (uint64_t)t_abs);
  float I;
  const bool spk = izh_step(s.x, s.y, I, p, g, z, a);
  v.vu[i] = s;
  if (a != 0) v.acc[i] = 0;
  if (last) v.ilast[i] = I;
  if (spk) {
    SpikeStat st = v.sstat[i];
    st.nospks += 1;
    if (st.last >= 0) {
      const long long isi = t_abs - st.last;
      st.nisi += 1;
      st.s1 += isi;
      st.s2 += isi * isi;
    }
    st.last = (int)t_abs;
    v.sstat[i] = st;
  }
  return spk;
}

// Update all neurons of step lt (absolute step t_abs) and append the spiking ids to the
// raster at base_t, one global atomic per block tile.
template <int NT>
__device__ __forceinline__ void update_phase(const NetView &v, int lt, int64_t t_abs, long long base_t,
                                             bool last, int *s_warp, long long *s_slot) {
  for (int64_t tile = blockIdx.x; tile * NT < v.n; tile += gridDim.x) {
    const int64_t i = tile * NT + threadIdx.x;
    bool spk = false;
    if (i < v.n) spk = update_one(v, i, t_abs, last);
    int total;
    const int slot = block_compact<NT>(spk, s_warp, &total);
    if (threadIdx.x == 0 && total) *s_slot = atomicAdd(v.counts + lt, total);
    __syncthreads();
    if (spk) {
      const long long pos = base_t + *s_slot + slot;
      if (pos < v.raster_cap)
        v.raster[pos] = (int)i;
      else
        atomicCAS(v.status, 0, kErrOverflowCode);
    }
    __syncthreads();
  }
}

// (the chunk's first step is read from device memory, so that a captured chunk replays for
// any chunk of the run)
template <int NT>
__global__ void __launch_bounds__(NT) k_update(NetView v, const long long *t0, int lt, int last) {
  const int64_t t_abs0 = *t0;
  __shared__ int s_warp[NT / 32 + 1];
  __shared__ long long s_slot;
  const long long base_t = lt == 0 ? 0ll : __ldcg(v.base + lt - 1) + __ldcg(v.counts + lt - 1);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    v.base[lt] = base_t;
    v.stamps[2 * lt] = globaltimer();
  }
  update_phase<NT>(v, lt, t_abs0 + lt, base_t, last != 0, s_warp, &s_slot);
}

// ---------------------------------------------------------------------------------------
// Delivery.
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ void deliver_vec(const NetView &v, int row, uint32_t j) {
  const size_t off = (size_t)row * (size_t)(v.stride >> 2) + j;
  const uint64_t pol = policy_evict_first();
  const int4 t = ld_stream_i4(reinterpret_cast<const int4 *>(v.idx) + off, pol);
  const float4 w = ld_stream_f4(reinterpret_cast<const float4 *>(v.w) + off, pol);
  deliver4(v.acc, t, w);
}

// Flat split of the step's K x (stride/4) vectors over all threads of the grid; the
// (row, vector) pair advances by a fixed stride without a division per iteration.
__device__ __forceinline__ void deliver_flat(const NetView &v, const int *list, int K) {
  const uint32_t rv = (uint32_t)(v.stride >> 2);
  const uint64_t total = (uint64_t)K * rv;
  const uint64_t g0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t gs = (uint64_t)gridDim.x * blockDim.x;
  if (g0 >= total) return;
  uint64_t q = g0 / rv;
  uint32_t j = (uint32_t)(g0 - q * rv);
  const uint64_t dq = gs / rv;
  const uint32_t dj = (uint32_t)(gs - dq * rv);
  for (uint64_t g = g0; g < total; g += gs) {
    deliver_vec(v, __ldcg(list + q), j);
    q += dq;
    j += dj;
    if (j >= rv) {
      j -= rv;
      q += 1;
    }
  }
}

// Groups of `group` consecutive threads take whole spiking rows.
__device__ __forceinline__ void deliver_groups(const NetView &v, const int *list, int K, int group) {
  const uint32_t rv = (uint32_t)(v.stride >> 2);
  const int gpb = blockDim.x / group;
  const int lig = threadIdx.x % group;
  const int64_t ngroups = (int64_t)gridDim.x * gpb;
  for (int64_t q = (int64_t)blockIdx.x * gpb + threadIdx.x / group; q < K; q += ngroups) {
    const int row = __ldcg(list + q);
    for (uint32_t j = lig; j < rv; j += group) deliver_vec(v, row, j);
  }
}

__device__ __forceinline__ void step_list(const NetView &v, int lt, const int *&list, int &K) {
  K = __ldcg(v.counts + lt);
  list = v.raster + __ldcg(v.base + lt);
}

__device__ __forceinline__ void stamp_delivery(const NetView &v, int lt) {
  if (blockIdx.x == 0 && threadIdx.x == 0) v.stamps[2 * lt + 1] = globaltimer();
}

// N: one thread per spiking neuron walks its whole row.
__global__ void k_deliver_n(NetView v, int lt) {
  stamp_delivery(v, lt);
  const int *list;
  int K;
  step_list(v, lt, list, K);
  const uint32_t rv = (uint32_t)(v.stride >> 2);
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < K; q += (int64_t)gridDim.x * blockDim.x) {
    const int row = __ldcg(list + q);
    for (uint32_t j = 0; j < rv; ++j) deliver_vec(v, row, j);
  }
}

// S and AB: flat split (S launches an oversubscribed grid, AB a persistent one).
__global__ void k_deliver_flat(NetView v, int lt) {
  stamp_delivery(v, lt);
  const int *list;
  int K;
  step_list(v, lt, list, K);
  deliver_flat(v, list, K);
}

// AP: a thread group per spiking row (the nested fan-out, without device launches).
__global__ void k_deliver_ap(NetView v, int lt, int group) {
  stamp_delivery(v, lt);
  const int *list;
  int K;
  step_list(v, lt, list, K);
  deliver_groups(v, list, K, group);
}

// ---------------------------------------------------------------------------------------
// SKL: every step of the chunk in one cooperative launch.  Per step: update + compaction,
// barrier, delivery (flat or grouped), barrier.  The running raster offset is kept in a
// register by every block (the step's count is final after the first barrier).
// ---------------------------------------------------------------------------------------
template <int NT>
__global__ void __launch_bounds__(NT) k_persistent(NetView v, int64_t t_abs0, int nsteps, int last_chunk,
                                                   GridSync *gs, unsigned long long limit_ns, int group,
                                                   int stall) {
  __shared__ int s_warp[NT / 32 + 1];
  __shared__ long long s_slot;
  unsigned epoch = 0;
  long long base = 0;
  const unsigned nb = gridDim.x + (unsigned)stall;  // stall > 0 only under fault injection
  for (int lt = 0; lt < nsteps; ++lt) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      v.base[lt] = base;
      v.stamps[2 * lt] = globaltimer();
    }
    update_phase<NT>(v, lt, t_abs0 + lt, base, last_chunk && lt == nsteps - 1, s_warp, &s_slot);
    if (!grid_barrier(gs, nb, epoch, limit_ns)) return;
    stamp_delivery(v, lt);
    const int K = __ldcg(v.counts + lt);
    const int *list = v.raster + base;
    if (group > 0)
      deliver_groups(v, list, K, group);
    else
      deliver_flat(v, list, K);
    if (!grid_barrier(gs, nb, epoch, limit_ns)) return;
    base += K;
  }
}

// ---------------------------------------------------------------------------------------
// FP64 statistics: sum of per-neuron ISI CVs and the number of neurons with >= 2 ISIs.
// ---------------------------------------------------------------------------------------
__global__ void k_stats(NetView v, double *out) {
  double cv = 0.0, cnt = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < v.n; i += (int64_t)gridDim.x * blockDim.x) {
    const SpikeStat s = v.sstat[i];
    if (s.nisi >= 2) {
      const double m = (double)s.nisi;
      const double mean = (double)s.s1 / m;
      const double var = (double)((long long)s.nisi * s.s2 - s.s1 * s.s1) / (m * m);
      cv += sqrt(var) / mean;
      cnt += 1.0;
    }
  }
  for (int o = 16; o; o >>= 1) {
    cv += __shfl_down_sync(0xFFFFFFFFu, cv, o);
    cnt += __shfl_down_sync(0xFFFFFFFFu, cnt, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(out, cv);
    atomicAdd(out + 1, cnt);
  }
}

// ---------------------------------------------------------------------------------------
// Launchers.
// ---------------------------------------------------------------------------------------
static int sm_count() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
  }
  return n;
}

static unsigned grid_for(int64_t work, int nt, int cap_per_sm) {
  int64_t g = (work + nt - 1) / nt;
  const int64_t cap = (int64_t)sm_count() * cap_per_sm;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (unsigned)g;
}

cudaError_t launch_init(const NetView &v, cudaStream_t s) {
  k_init_state<<<grid_for(v.n, 256, 32), 256, 0, s>>>(v);
  return cudaGetLastError();
}

cudaError_t launch_conngen(const NetView &v, int self_loops, cudaStream_t s) {
  int log2h = 5;
  while ((1 << log2h) < 2 * v.nsyn + 64) ++log2h;
  // the target bitmap (n bits, in 16-byte units) where it is smaller than the hash
  const int64_t bm_words = ((v.n + 127) / 128) * 4;
  const int bits = bm_words < ((int64_t)1 << log2h) ? (int)bm_words : 0;
  const size_t per_warp = bits > 0 ? (size_t)4 * bits : (size_t)4 << log2h;
  if (per_warp > 200 * 1024) return cudaErrorInvalidValue;
  // one ceiling for every network (concurrent host threads generating tables of different
  // fan-outs must not lower it under one another's launch)
  cudaError_t e = cudaFuncSetAttribute(k_conngen, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  if (e != cudaSuccess) return e;
  // warps per CTA (at most 8): the most resident warps per SM
  int wpb = 1, best = 0, occ_best = 1;
  for (int w = 1; w <= 8 && per_warp * w <= 200 * 1024; ++w) {
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_conngen, w * 32, per_warp * w);
    if (occ * w > best) best = occ * w, wpb = w, occ_best = occ < 1 ? 1 : occ;
  }
  const size_t smem = per_warp * wpb;
  const uint64_t range = self_loops ? (uint64_t)v.n : (uint64_t)(v.n - 1);
  // generous cap on draw blocks (a full row needs about range * ln(range) draws)
  unsigned long long max_blocks = (64ull * (range + (uint64_t)v.nsyn) + 4096ull) / 128ull + 64ull;
  int64_t g = (v.n + wpb - 1) / wpb;
  const int64_t cap = (int64_t)sm_count() * occ_best * 8;
  if (g > cap) g = cap;
  k_conngen<<<(unsigned)g, wpb * 32, smem, s>>>(v, self_loops, log2h, bits, 0, v.n, max_blocks);
  return cudaGetLastError();
}

constexpr int kUpdNT = 256;
constexpr int kPerNT = 512;

cudaError_t launch_update(const NetView &v, const long long *t0, int lt, bool last, cudaStream_t s) {
  k_update<kUpdNT><<<grid_for(v.n, kUpdNT, 8), kUpdNT, 0, s>>>(v, t0, lt, last ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t launch_deliver(const NetView &v, int lt, int alg, const DeliverShape &sh, cudaStream_t s) {
  switch (alg) {
    case kAlgN:
      k_deliver_n<<<grid_for(v.n, 128, 64), 128, 0, s>>>(v, lt);
      break;
    case kAlgS: {
      const int64_t vecs = (int64_t)(sh.k_hint > 0 ? sh.k_hint : 1) * (v.stride >> 2);
      k_deliver_flat<<<grid_for(vecs, 256, 64), 256, 0, s>>>(v, lt);
      break;
    }
    case kAlgAP: {
      const int group = sh.group > 0 ? sh.group : 64;
      k_deliver_ap<<<(unsigned)(sm_count() * sh.blocks_per_sm), 256, 0, s>>>(v, lt, group);
      break;
    }
    case kAlgAB:
      k_deliver_flat<<<(unsigned)(sm_count() * sh.blocks_per_sm), 256, 0, s>>>(v, lt);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

int persistent_blocks() {
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_persistent<kPerNT>, kPerNT, 0);
  if (occ < 1) occ = 1;
  return occ * sm_count();
}

cudaError_t launch_persistent(const NetView &v, int64_t t_abs0, int nsteps, bool last_chunk, GridSync *gs,
                              unsigned long long limit_ns, int group, int stall, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)persistent_blocks());
  cfg.blockDim = dim3(kPerNT);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_persistent<kPerNT>, v, t_abs0, nsteps, last_chunk ? 1 : 0, gs, limit_ns,
                            group, stall);
}

cudaError_t launch_stats(const NetView &v, double *out, cudaStream_t s) {
  k_stats<<<grid_for(v.n, 256, 8), 256, 0, s>>>(v, out);
  return cudaGetLastError();
}

}  // namespace g4s
