// g4s_team.cu — the SKL step loop as an owner-computes team kernel (the GB300 design of
// SKL_deliverspks, gpu4snn.cu:669-716), for one network or many, plus the table
// preparation it needs.
//
// Teams.  A launch runs a list of networks (TeamItem); network i is simulated by a team
// of T_i CTAs.  The CTAs of the cooperative, persistent grid take (network, rank) slots
// from one ordered queue; multi-CTA teams come first in the queue, so a team's members
// start together.  A single network on the whole GPU is a one-item launch with a team of
// one CTA per SM; a batched ensemble is a many-item launch where most networks fit one
// CTA.
//
// Target ownership.  Team rank r owns the neurons [r Rc, (r+1) Rc) of its network and
// keeps their synaptic currents in shared memory for the whole launch, as two 32-bit
// words per neuron: the Q32.32 current q = A * 2^16 + B, with B the sum of the weights'
// low 16 bits and A the sum of their high 48 bits.  Shared-memory 32-bit atomics are
// about five times faster than 64-bit ones on this part, and the split is exact as long
// as no neuron has 65536 or more incoming synapses and the sum of |q_i| / 2^16 + 1 over
// its incoming synapses stays below 2^31; k_inbound checks both once per table (the
// host falls back to the global-atomic persistent kernel otherwise).  Small slices also
// keep v, u (and a, b, c, d) in shared memory for the launch.
//
// Per step, for each team:
//   update    every rank updates its own neurons (current read from and cleared in shared
//             memory; drive precomputed in shared memory during the previous step) and
//             collects its spikes in shared memory;
//   exchange  one-CTA team: nothing, the spike list stays in shared memory.  Larger team:
//             each rank publishes its spike count and ids as 64-bit words, each tagged
//             with a step number that never repeats for the network's buffers, so a
//             reader that sees the tag it expects needs no fence to trust the payload:
//             two 128-byte record lines (count and 31 ids), further ids in a per-rank
//             overflow list.  Every rank reads, in one pass, line 0 of every rank and
//             line 1 of the ranks that had more than kLine1After spikes in the previous
//             step (16-byte slots, polled until their tags are current, with a time
//             limit), so the records double as the team barrier; ids beyond the lines
//             read are polled word by word.  The step's ids are staged in shared memory;
//             a step with more ids than the window writes a dense tagged list in global
//             memory instead, read directly by the delivery.  Records are cleared before
//             each launch.  Two record sets (by step parity) suffice: a rank writes step
//             t+2's words only after every rank has published step t+1, i.e. finished
//             reading step t.
//   delivery  one-CTA team: whole spiking rows, 128-bit loads, flat over all threads.
//             Larger team: every rank reads, for every spike, the segment of the spiking
//             row whose targets fall in its slice (rows are sorted by target and a per-row
//             offset table gives the segment).  The run and group mappings read the rows
//             interleaved as (target, weight bits) pairs, so a segment of ~7 synapses is one
//             contiguous run of sectors instead of two half-used ones: at 7,000 spikes per
//             step this cut the delivery by a third.  Flat mapping (at least kFlatMinSpikes
//             staged spikes, at most kFlatMax synapses for the rank, and, in a 768-thread
//             CTA, fewer than NT/2 spikes): the segment bounds
//             of all spikes at once, a block scan, every synapse of the concatenation
//             mapped to its spike in shared memory, and thread i walks synapses i, i+NT,
//             ... with eight reads in flight.  Run mapping (otherwise): a warp takes 32
//             spikes, scans their segment lengths and walks the concatenated segments,
//             eight synapses per lane in flight, each lane finding its synapse's spike by
//             a shuffle search.  Group mapping (the team's choice for long segments): the
//             warp's 32 spikes in 8 rounds of 4, eight lanes walking each spike's segment,
//             no search.  Each weight goes into the rank's own shared memory.
//   tail      the raster and the spike statistics of this rank's spikes, and the next
//             step's drive, handed out in chunks of 32 neurons to warps as they finish
//             delivering (the flat mapping computes each thread's own neuron's drive
//             while its reads are in flight).
//   The raster records the spike ids of every step while its buffer has room.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "g4s_device.cuh"
#include "g4s_internal.h"

namespace g4s {

// ---------------------------------------------------------------------------------------
// Row sort: every row's (target, weight) pairs in ascending target order, unused slots
// (negative targets, i.e. huge as unsigned) last.  One CTA of NT threads per row, a bitonic
// network over p2 = E * NT 64-bit keys (target << 32 | weight bits); thread t holds the
// keys of elements t, t + NT, ..., in registers.  A compare-exchange over distance j takes
// place in registers when j >= NT (the partner is the same thread's), through shuffles
// when j < 32 (the partner is in the same warp), and through shared memory between warps
// otherwise, so that only those stages need block barriers.
// ---------------------------------------------------------------------------------------
template <int E>
__global__ void __launch_bounds__(1024) k_sort_rows(NetView v, int p2) {
  extern __shared__ unsigned long long s_key[];
  const int NT = blockDim.x, t = threadIdx.x;
  for (int64_t row = blockIdx.x; row < v.n; row += gridDim.x) {
    int *ri = const_cast<int *>(v.idx) + row * v.stride;
    float *rw = const_cast<float *>(v.w) + row * v.stride;
    unsigned long long key[E];
#pragma unroll
    for (int r = 0; r < E; ++r) {
      const int e = r * NT + t;
      key[r] = e < v.stride ? ((unsigned long long)(unsigned)ri[e] << 32) | __float_as_uint(rw[e])
                            : 0xFFFFFFFFFFFFFFFFull;
    }
    for (int k = 2; k <= p2; k <<= 1)
      for (int j = k >> 1; j > 0; j >>= 1) {
        if (j >= NT) {
          const int rj = j / NT;
#pragma unroll
          for (int RJ = 1; RJ < E; RJ <<= 1)  // (each distance unrolled: registers, not memory)
            if (rj == RJ) {
#pragma unroll
              for (int r = 0; r < E; ++r)
                if ((r & RJ) == 0) {
                  const bool asc = ((r * NT + t) & k) == 0;
                  const unsigned long long a = key[r], b = key[r | RJ];
                  if ((a > b) == asc) {
                    key[r] = b;
                    key[r | RJ] = a;
                  }
                }
            }
        } else {
          if (j >= 32) {
            __syncthreads();  // (the previous stage's reads are done)
#pragma unroll
            for (int r = 0; r < E; ++r) s_key[r * NT + t] = key[r];
            __syncthreads();
          }
#pragma unroll
          for (int r = 0; r < E; ++r) {
            const int e = r * NT + t;
            const unsigned long long o = j >= 32 ? s_key[e ^ j] : __shfl_xor_sync(0xFFFFFFFFu, key[r], j);
            const bool keep_min = ((e & j) == 0) == ((e & k) == 0);
            key[r] = keep_min ? (o < key[r] ? o : key[r]) : (o > key[r] ? o : key[r]);
          }
        }
      }
#pragma unroll
    for (int r = 0; r < E; ++r) {
      const int e = r * NT + t;
      if (e < v.stride) {
        ri[e] = (int)(key[r] >> 32);
        rw[e] = __uint_as_float((unsigned)key[r]);
      }
    }
  }
}

// Generated rows (distinct targets, every unused slot (-1, 0.0f)) in the same order as
// k_sort_rows' by a bucket sort of narrower keys: 32-bit key target << pb | slot (n << pb
// | slot for an unused slot), 2^pb >= p2 and (n << pb) + p2 - 1 below 2^32 - 1, unique, so
// that every key names the slot its weight comes from.  Bucket of a key: its target >> sh
// (targets taken as n for unused slots; n >> sh < nb), monotone in the key, about two to
// four keys each as the targets are drawn uniformly.  Per row: the weights into shared
// memory; a histogram whose atomics also give each key its rank in its bucket; a block
// scan of the counts; each key stored at its bucket's start + its rank; one thread per
// bucket orders the bucket's keys by insertion; the row written back (target from the
// key, weight gathered from the shared copy).  E keys a thread, element r * NT + t.
template <int E>
__global__ void __launch_bounds__(1024) k_sort_gen(NetView v, int pb, int nb, int sh) {
  extern __shared__ __align__(16) unsigned s_gen[];
  const int NT = blockDim.x, t = threadIdx.x, lane = t & 31, warp = t >> 5;
  unsigned *s_cnt = s_gen;                                  // nb counts, then bucket starts
  unsigned *s_part = s_cnt + nb;                            // 32 warp sums
  unsigned *s_key = s_part + 32;                            // stride keys, by bucket
  float *s_w = reinterpret_cast<float *>(s_key + v.stride);  // the row's weights
  const unsigned n = (unsigned)v.n, smask = (1u << pb) - 1u, lim = n << pb;
  const int per = nb / NT;  // buckets a thread scans (nb is a multiple of NT)
  for (int64_t row = blockIdx.x; row < v.n; row += gridDim.x) {
    int *ri = const_cast<int *>(v.idx) + row * v.stride;
    float *rw = const_cast<float *>(v.w) + row * v.stride;
    for (int b = t; b < nb; b += NT) s_cnt[b] = 0u;
    unsigned key[E];
#pragma unroll
    for (int r = 0; r < E; ++r) {
      const int e = r * NT + t;
      if (e < v.stride) {
        const unsigned ti = (unsigned)ri[e];
        key[r] = ((ti < n ? ti : n) << pb) | (unsigned)e;
        s_w[e] = rw[e];
      }
    }
    __syncthreads();
    unsigned rank[E];
#pragma unroll
    for (int r = 0; r < E; ++r)
      if (r * NT + t < v.stride) rank[r] = atomicAdd(s_cnt + ((key[r] >> pb) >> sh), 1u);
    __syncthreads();
    // exclusive scan of the counts: thread t's buckets t*per .. t*per+per-1, then warps
    unsigned mine = 0;
    for (int q = 0; q < per; ++q) mine += s_cnt[t * per + q];
    unsigned incl = mine;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const unsigned o = __shfl_up_sync(0xFFFFFFFFu, incl, d);
      if (lane >= d) incl += o;
    }
    if (lane == 31) s_part[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      const int nw = NT >> 5;
      unsigned x = lane < nw ? s_part[lane] : 0u, xi = x;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const unsigned o = __shfl_up_sync(0xFFFFFFFFu, xi, d);
        if (lane >= d) xi += o;
      }
      if (lane < nw) s_part[lane] = xi - x;
    }
    __syncthreads();
    unsigned start = s_part[warp] + incl - mine;
    for (int q = 0; q < per; ++q) {
      const unsigned c = s_cnt[t * per + q];
      s_cnt[t * per + q] = start;
      start += c;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < E; ++r)
      if (r * NT + t < v.stride) s_key[s_cnt[(key[r] >> pb) >> sh] + rank[r]] = key[r];
    __syncthreads();
    for (int b = t; b < nb; b += NT) {
      const unsigned lo = s_cnt[b], hi = b + 1 < nb ? s_cnt[b + 1] : (unsigned)v.stride;
      for (unsigned i = lo + 1; i < hi; ++i) {
        const unsigned x = s_key[i];
        unsigned j = i;
        while (j > lo && s_key[j - 1] > x) {
          s_key[j] = s_key[j - 1];
          --j;
        }
        s_key[j] = x;
      }
    }
    __syncthreads();
    for (int e = t; e < v.stride; e += NT) {
      const unsigned k = s_key[e];
      ri[e] = k < lim ? (int)(k >> pb) : -1;
      rw[e] = s_w[k & smask];
    }
    __syncthreads();  // (before the next row overwrites the shared arrays)
  }
}

// Rows already in the sort's order (ascending 64-bit keys target << 32 | weight bits, the
// targets taken as unsigned so that unused slots come last)?  *unsorted = 1 if not.
// One warp per row, consecutive lanes on consecutive slots.
__global__ void k_rows_sorted(NetView v, int *unsorted) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  bool bad = false;
  for (int64_t row = warp; row < v.n; row += nwarps) {
    const int *ri = v.idx + row * v.stride;
    const float *rw = v.w + row * v.stride;
    for (int j = lane; j + 1 < v.stride; j += 32) {
      const unsigned long long a = ((unsigned long long)(unsigned)ri[j] << 32) | __float_as_uint(rw[j]);
      const unsigned long long b = ((unsigned long long)(unsigned)ri[j + 1] << 32) | __float_as_uint(rw[j + 1]);
      bad |= a > b;
    }
  }
  if (__any_sync(0xFFFFFFFFu, bad) && lane == 0) *unsorted = 1;
}

// Segment table: seg[row][k] = first slot of the sorted row whose target is >= k*Rc, for
// k = 0..T (unused slots compare as huge and lie beyond seg[row][T]).  One warp per row,
// one binary search per boundary.
__global__ void k_segoff(NetView v, int T, int64_t Rc, uint16_t *seg) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t row = warp; row < v.n; row += nwarps) {
    const int *ri = v.idx + row * v.stride;
    for (int k = lane; k <= T; k += 32) {
      const int64_t bound = (int64_t)k * Rc;
      int lo = 0, hi = v.stride;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if ((int64_t)(unsigned)ri[mid] < bound)
          lo = mid + 1;
        else
          hi = mid;
      }
      seg[row * (T + 1) + k] = (uint16_t)lo;
    }
  }
}

// Interleaved rows for the team kernel: pair[g] = (target, weight bits) of slot g.
__global__ void k_pairs(NetView v, int2 *pair) {
  const int64_t total = v.n * (int64_t)v.stride;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x)
    pair[g] = make_int2(v.idx[g], __float_as_int(v.w[g]));
}

// Exactness bound of the split accumulation: per target, the number of incoming synapses
// and the sum of (|q| >> 16) + 1 over them; out[0] = max count, out[1] = max sum.
// Per neuron the in-degree and, with mag, sum(|q| >> 16) + 1 over its inputs; without mag,
// the largest (|q| >> 16) + 1 of the table into *term instead.
__global__ void k_inbound(NetView v, unsigned *cnt, unsigned long long *mag, unsigned long long *term) {
  const int64_t total = v.n * (int64_t)v.stride;
  unsigned long long mx = 0;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x) {
    const int t = v.idx[g];
    if (t < 0) continue;
    atomicAdd(cnt + t, 1u);
    const long long q = wfix(v.w[g]);
    const unsigned long long a = ((unsigned long long)(q < 0 ? -q : q) >> 16) + 1ull;
    if (mag)
      atomicAdd(mag + t, a);
    else
      mx = max(mx, a);
  }
  if (!mag) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) mx = max(mx, __shfl_xor_sync(0xFFFFFFFFu, mx, d));
    if ((threadIdx.x & 31) == 0) atomicMax(term, mx);
  }
}

__global__ void k_inbound_max(int64_t n, const unsigned *cnt, const unsigned long long *mag,
                              unsigned long long *out) {
  unsigned long long mc = 0, mm = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    mc = max(mc, (unsigned long long)cnt[i]);
    if (mag) mm = max(mm, mag[i]);
  }
  atomicMax(out, mc);
  atomicMax(out + 1, mm);
}

// Split-accumulator add: A += q >> 16 (arithmetic), B += q & 0xFFFF.
__device__ __forceinline__ void acc_add(unsigned base_a, unsigned base_b, unsigned off, long long q) {
  asm volatile("red.shared.add.s32 [%0], %1;" ::"r"(base_a + off * 4u), "r"((int)(q >> 16)) : "memory");
  asm volatile("red.shared.add.u32 [%0], %1;" ::"r"(base_b + off * 4u), "r"((unsigned)(q & 0xFFFF)) : "memory");
}

__device__ __forceinline__ void acc_add4(unsigned base_a, unsigned base_b, int lo, const int4 t, const float4 w) {
  if (t.x >= 0) acc_add(base_a, base_b, (unsigned)(t.x - lo), wfix(w.x));
  if (t.y >= 0) acc_add(base_a, base_b, (unsigned)(t.y - lo), wfix(w.y));
  if (t.z >= 0) acc_add(base_a, base_b, (unsigned)(t.z - lo), wfix(w.z));
  if (t.w >= 0) acc_add(base_a, base_b, (unsigned)(t.w - lo), wfix(w.w));
}

// Last index r in [0, n) with a[r] <= x, for a non-decreasing a[0..n] with a[0] <= x < a[n].
__device__ __forceinline__ int find_run(const int *a, int n, int x) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (a[mid] <= x)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// Scalars of one CTA shared by the phases of a step; the per-step counters come in pairs
// (by step parity) so that one is cleared while the other is in use.
struct TeamShared {
  int nown[2];  // spikes of this rank in the step
  int work[2];  // next chunk of the next step's drive
  int fail;     // the exchange gave up (time limit, or the team's error word was set)
  int slot;     // queue slot taken by this CTA
};

// Record words of a rank per step: word 0 = spike count, words 1.. = ids (kInline inline);
// a thread of an NT-thread CTA reads up to slots_per_thread(NT) 16-byte slots of a step's
// records.
constexpr int kRankWords = kRecLines * kRecWords;
constexpr int kInline = kRankWords - 1;
__host__ __device__ constexpr int slots_per_thread(int nt) { return (kMaxTeam * kRankWords / 2 + nt - 1) / nt; }
constexpr int kLine1After = 7;
constexpr int kFlatMinSpikes = 128;  // fewer spikes: run delivery (the flat one's scan costs more)  // line 1 of a rank is read if it had more spikes in the previous step

// Gives up a wait: first error wins, every CTA of the team leaves at its next check.
__device__ __forceinline__ void give_up(TeamShared &sh, GridSync *gs) {
  atomicCAS(&gs->error, 0, kErrTimeoutCode);
  *(volatile int *)&sh.fail = 1;
}

// One tagged word of another rank, polled until it carries `tag` (or the time limit).
__device__ __forceinline__ int tagged_id(const unsigned long long *p, unsigned tag, TeamShared &sh, GridSync *gs,
                                         unsigned long long lim) {
  unsigned long long w = ld_relaxed_u64(p);
  if ((unsigned)(w >> 32) == tag) return (int)(unsigned)w;
  const unsigned long long t0 = globaltimer();
  for (;;) {
    w = ld_relaxed_u64(p);
    if ((unsigned)(w >> 32) == tag) return (int)(unsigned)w;
    if (*(volatile int *)&sh.fail || ld_relaxed(&gs->error) != 0 || globaltimer() - t0 > lim) {
      give_up(sh, gs);
      return 0;
    }
  }
}

// ---------------------------------------------------------------------------------------
// One team member's share of one network for the steps of this launch.
// ---------------------------------------------------------------------------------------
constexpr int kUpd = 4;  // neurons a thread updates per round of the team kernel's update

template <int NT, bool kPair>
__device__ void team_run(const TeamItem &it, int rank, unsigned char *s_raw, TeamShared &sh,
                         unsigned long long limit_ns, int stall) {
  const NetView &v = it.v;
  const int T = it.team, rc = it.rc;
  const TeamLayout L = team_layout(rc, T, it.cap);
  float4 *s_abcd = reinterpret_cast<float4 *>(s_raw + L.abcd);
  float2 *s_vu = reinterpret_cast<float2 *>(s_raw + L.vu);
  int *s_a = reinterpret_cast<int *>(s_raw + L.a);
  unsigned *s_b = reinterpret_cast<unsigned *>(s_raw + L.b);
  int *s_own = reinterpret_cast<int *>(s_raw + L.own);
  float *s_z = reinterpret_cast<float *>(s_raw + L.z);
  int *s_cnt = reinterpret_cast<int *>(s_raw + L.cnt);
  int *s_off = reinterpret_cast<int *>(s_raw + L.off);
  int *s_xoff = reinterpret_cast<int *>(s_raw + L.xoff);
  int *s_inl = reinterpret_cast<int *>(s_raw + L.inl);
  unsigned *s_pay = reinterpret_cast<unsigned *>(s_raw + L.pay);
  uint16_t *s_sb = reinterpret_cast<uint16_t *>(s_raw + L.sb);
  int *s_pre = reinterpret_cast<int *>(s_raw + L.pre);
  uint16_t *s_ex = reinterpret_cast<uint16_t *>(s_raw + L.ex);
  int *s_wsum = reinterpret_cast<int *>(s_raw + L.wsum);
  int *s_spk = reinterpret_cast<int *>(s_raw + L.spk);
  const int64_t lo = min((int64_t)rank * rc, v.n);
  const int64_t hi = min(lo + rc, v.n);
  const int cnt = (int)(hi - lo);
  const unsigned base_a = (unsigned)__cvta_generic_to_shared(s_a);
  const unsigned base_b = (unsigned)__cvta_generic_to_shared(s_b);
  const unsigned segw = (unsigned)T + 1;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int kWarps = NT / 32;
  constexpr int kSlots = slots_per_thread(NT);
  const bool solo = T == 1;   // the whole network in this CTA: no exchange
  const bool lead = rank == 0 && threadIdx.x == 0;
  // synapse `off` of the tables: one 8-byte load from the interleaved rows, or two loads
  auto synapse = [&](long long off, int &t, float &w) {
    if constexpr (kPair) {
      const int2 p = __ldg(v.pair + off);
      t = p.x;
      w = __int_as_float(p.y);
    } else {
      t = __ldg(v.idx + off);
      w = __ldg(v.w + off);
    }
  };
  // neuron state of the slice: shared memory for the launch when it fits, else global
  float2 *vu = L.vu_sm ? s_vu : v.vu + lo;
  const float4 *abcd = L.abcd_sm ? s_abcd : v.abcd + lo;
  const float *rp = L.abcd_sm ? nullptr : (v.rpar ? v.rpar + lo : nullptr);  // a,b,c,d recomputed from r

  for (int i = threadIdx.x; i < cnt; i += NT) {
    const long long q = __ldcg(v.acc + lo + i);
    s_a[i] = (int)(q >> 16);
    s_b[i] = (unsigned)(q & 0xFFFF);
    if (L.vu_sm) s_vu[i] = v.vu[lo + i];
    if (L.abcd_sm) s_abcd[i] = v.abcd[lo + i];
  }
  if (!solo)  // the first step reads one record line per rank
    for (int r = threadIdx.x; r <= T; r += NT) s_cnt[r] = 0;
  if (threadIdx.x == 0) {
    sh.nown[0] = sh.nown[1] = 0;
    sh.work[0] = sh.work[1] = 0;
    sh.fail = 0;
  }
  __syncthreads();

  long long base = 0;
  for (int lt = 0; lt < it.steps; ++lt) {
    const int64_t t_abs = it.t_abs0 + lt;
    const bool last = it.last && lt == it.steps - 1;
    const int par = lt & 1;
    if (threadIdx.x == 0) {
      sh.nown[par ^ 1] = 0;  // last used by the previous step, next by the following one
      sh.work[par ^ 1] = 0;
    }
    if (lead) {
      v.base[lt] = base;
      if (v.stamps) v.stamps[2 * lt] = globaltimer();
    }
    // ---- update of the owned neurons, four per thread per round: the state loads of all
    // four first (a slice whose state lives in global memory takes one memory round trip
    // per round), then each neuron in turn
    const bool use_z = L.prez && lt > 0;
    for (int i0 = threadIdx.x; i0 < cnt; i0 += kUpd * NT) {
      float2 sv[kUpd];
      float rr[kUpd];
#pragma unroll
      for (int u = 0; u < kUpd; ++u) {
        const int i = i0 + u * NT, j = i < cnt ? i : i0;
        sv[u] = vu[j];
        rr[u] = rp ? rp[j] : 0.0f;
      }
#pragma unroll
      for (int u = 0; u < kUpd; ++u) {
        const int i = i0 + u * NT;
        if (i < cnt) {
          const int64_t nn = lo + i;
          const float4 p = rp ? izh_abcd(rr[u], nn < v.nexc) : abcd[i];
          const long long a = (long long)s_a[i] * 65536 + s_b[i];
          s_a[i] = 0;
          s_b[i] = 0;
          const float z = use_z ? s_z[i] : normal(v.seed, (uint64_t)nn, (uint64_t)t_abs);
          float I;
          const bool k = izh_step(sv[u].x, sv[u].y, I, p, nn < v.nexc ? v.ge : v.gi, z, a);
          vu[i] = sv[u];
          if (last) v.ilast[nn] = I;
          if (k) s_own[atomicAdd(&sh.nown[par], 1)] = (int)nn;
        }
      }
    }
    __syncthreads();
    const int nown = sh.nown[par];
    const unsigned long long lim = lt == 0 ? limit_ns * 16 : limit_ns;  // members may start late
    if (stall != 0 && solo) {
      // injected fault of a one-CTA team: wait for a member that does not exist
      if (threadIdx.x == 0) {
        const unsigned long long t0 = globaltimer();
        while (ld_relaxed(&it.sync->error) == 0 && globaltimer() - t0 <= lim) {
        }
        give_up(sh, it.sync);
      }
      __syncthreads();
      return;
    }
    int K = nown, my_off = 0;
    const int *list = s_own;
    const unsigned tag = it.tag0 + (unsigned)lt + 1u;
    const unsigned long long *recs = it.rec + (size_t)par * T * kRankWords;
    const unsigned long long *ovf_all = it.list + (size_t)par * v.n;
    unsigned long long *dense = it.list + (size_t)(2 + par) * v.n;
    bool gl = false;    // the step's ids are read from the dense list in global memory
    bool flat = false;  // flat delivery from shared memory
    int F = 0;          // ... synapses of the concatenated segments
    const bool zwant = L.prez && lt + 1 < it.steps;  // the next step's drive is precomputed
    int zdone = 0;      // ... for neurons [0, zdone) already
    if (!solo) {
      // ---- publish: both record lines of this rank (count, ids, padding), ids beyond
      // them in the overflow list; every word tagged with the step, so no fence is needed
      {
        const unsigned long long tg = (unsigned long long)tag << 32;
        unsigned long long *ovf = it.list + (size_t)par * v.n + lo;
        for (int j = kInline + threadIdx.x; j < nown; j += NT) st_relaxed_u64(ovf + j, tg | (unsigned)s_own[j]);
        if (threadIdx.x < kRankWords) {
          const int j = threadIdx.x;
          const unsigned pay = j == 0 ? (unsigned)nown : (j - 1 < nown ? (unsigned)s_own[j - 1] : 0xFFFFFFFFu);
          st_relaxed_u64(it.rec + ((size_t)par * T + rank) * kRankWords + j, tg | pay);
        }
      }
      // ---- first pass: line 0 of every rank and line 1 of the ranks that had more than
      // kLine1After spikes in the previous step, as 16-byte slots (slot x = words 2x, 2x+1 of the
      // step's records, rank x / 16), up to three per thread; each warp polls its slots
      // until all carry the step's tag, then the payloads go to shared memory
      unsigned need = 0;
#pragma unroll
      for (int k = 0; k < kSlots; ++k) {
        const int x = threadIdx.x + k * NT;
        if (x < T * 16 && ((x & 15) < 8 || s_cnt[x >> 4] > kLine1After)) need |= 1u << k;
      }
      unsigned long long t0 = 0;
      for (int iter = 0;; ++iter) {
        ulonglong2 a[kSlots];
#pragma unroll
        for (int k = 0; k < kSlots; ++k)
          if (need & (1u << k)) a[k] = ld_relaxed_u64x2(recs + 2 * (threadIdx.x + k * NT));
#pragma unroll
        for (int k = 0; k < kSlots; ++k)
          if ((need & (1u << k)) && (unsigned)(a[k].x >> 32) == tag && (unsigned)(a[k].y >> 32) == tag) {
            const int x = threadIdx.x + k * NT;
            s_pay[2 * x] = (unsigned)a[k].x;
            s_pay[2 * x + 1] = (unsigned)a[k].y;
            need &= ~(1u << k);
          }
        if (__all_sync(0xFFFFFFFFu, need == 0) && stall == 0) break;
        int f = 0;
        if (lane == 0) {
          const unsigned long long now = globaltimer();
          if (iter == 0) t0 = now;
          f = *(volatile int *)&sh.fail;
          if (!f && warp == 0 && ld_relaxed(&it.sync->error) != 0) f = 1;
          if (!f && now - t0 > lim) {
            give_up(sh, it.sync);
            f = 1;
          }
          if (f) *(volatile int *)&sh.fail = 1;
        }
        if (__shfl_sync(0xFFFFFFFFu, f, 0)) break;
      }
      __syncthreads();
      if (sh.fail) return;
      if (warp == 0) {
        // per rank: count, ids in the lines read (15 or 31), offsets of all ids and of
        // those beyond the lines read
        constexpr int kPer = kMaxTeam / 32;
        int c[kPer], xr[kPer], sc = 0, sx = 0;
#pragma unroll
        for (int k = 0; k < kPer; ++k) {
          const int r = lane * kPer + k;
          c[k] = 0;
          xr[k] = 0;
          if (r < T) {
            const int inl = s_cnt[r] > kLine1After ? kInline : kRecWords - 1;
            c[k] = (int)s_pay[r * kRankWords];
            xr[k] = max(0, c[k] - inl);
            s_inl[r] = inl;
          }
          sc += c[k];
          sx += xr[k];
        }
        int ic = sc, ix = sx;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int yc = __shfl_up_sync(0xFFFFFFFFu, ic, o), yx = __shfl_up_sync(0xFFFFFFFFu, ix, o);
          if (lane >= o) {
            ic += yc;
            ix += yx;
          }
        }
        int ec = ic - sc, ex = ix - sx;
#pragma unroll
        for (int k = 0; k < kPer; ++k) {
          const int r = lane * kPer + k;
          if (r < T) {
            s_cnt[r] = c[k];
            s_off[r] = ec;
            s_xoff[r] = ex;
          }
          ec += c[k];
          ex += xr[k];
        }
        if (lane == 31) {
          s_off[T] = ec;
          s_xoff[T] = ex;
        }
      }
      __syncthreads();
      K = s_off[T];
      my_off = s_off[rank];
      list = s_spk;
      if (K > it.cap) {
        // many spikes: instead of staging windows, every rank writes its ids (tagged) at
        // its offset in the step's dense list, which the delivery reads directly
        gl = true;
        const unsigned long long tg = (unsigned long long)tag << 32;
        for (int j = threadIdx.x; j < nown; j += NT) st_relaxed_u64(dense + my_off + j, tg | (unsigned)s_own[j]);
      }
    }
    if (lead && v.stamps) v.stamps[2 * lt + 1] = globaltimer();
    if (lead) v.counts[lt] = K;

    {
      const int Kw = K;
      if (!solo && !gl && K > 0) {
        // ---- stage the step's spike ids in shared memory: the first pass's payloads,
        // then ids beyond the lines read, polled from the records or the overflow list
        {
#pragma unroll
          for (int k = 0; k < kSlots; ++k) {
            const int x = threadIdx.x + k * NT;
            if (x < T * 16) {
              const int r = x >> 4, w0 = 2 * (x & 15), c = min(s_cnt[r], s_inl[r]), o = s_off[r] - 1;
              if (w0 >= 1 && w0 - 1 < c) s_spk[o + w0] = (int)s_pay[2 * x];
              if (w0 < c) s_spk[o + w0 + 1] = (int)s_pay[2 * x + 1];
            }
          }
          const int X = s_xoff[T];
          for (int e = threadIdx.x; e < X; e += NT) {
            const int r = find_run(s_xoff, T, e);
            const int j = s_inl[r] + e - s_xoff[r];
            s_spk[s_off[r] + j] = tagged_id(
                j < kInline ? recs + (size_t)r * kRankWords + 1 + j : ovf_all + (size_t)r * rc + j, tag, sh, it.sync, lim);
          }
        }
        __syncthreads();
        if (sh.fail) return;
      }
      // (a smaller CTA takes the flat mapping only for steps too small to give most of its
      // warps a 32-spike batch of the run mapping, which measured faster above that)
      if (!solo && !gl && K >= kFlatMinSpikes && L.flat && K <= 4 * NT && (NT >= 1024 || K < NT / 2)) {
        // segment bounds and their offsets in the concatenation (for the flat delivery):
        // thread t takes spikes 4t .. 4t+3 (K <= 4 NT); a block scan of their
        // lengths (every warp scans the warp sums itself), then each thread marks the
        // synapses of its spikes with the spike's index
        const uint64_t pkeep = policy_evict_last();
        int len[4], b4[4], sum = 0;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int q = threadIdx.x * 4 + u;
          len[u] = 0;
          b4[u] = 0;
          if (q < K) {
            const uint16_t *so = it.seg + (size_t)s_spk[q] * segw + rank;
            b4[u] = ld_keep_u16(so, pkeep);
            len[u] = ld_keep_u16(so + 1, pkeep) - b4[u];
          }
          sum += len[u];
        }
        int incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
          if (lane >= o) incl += y;
        }
        if (lane == 31) s_wsum[warp] = incl;
        __syncthreads();
        const int ws = lane < kWarps ? s_wsum[lane] : 0;
        int wi = ws;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(0xFFFFFFFFu, wi, o);
          if (lane >= o) wi += y;
        }
        F = __shfl_sync(0xFFFFFFFFu, wi, 31);
        flat = F <= kFlatMax;
        if (flat) {
          int pre = __shfl_sync(0xFFFFFFFFu, wi - ws, warp) + incl - sum;
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int q = threadIdx.x * 4 + u;
            if (q < K) {
              s_pre[q] = pre;
              s_sb[q] = (uint16_t)b4[u];
              for (int f = pre; f < pre + len[u]; ++f) s_ex[f] = (uint16_t)q;
            }
            pre += len[u];
          }
        }
        __syncthreads();
      }
      if (solo) {
        // ---- delivery, one-CTA team: flat over K whole rows of stride/4 vectors
        const int rv = v.stride >> 2;
        const int total = Kw * rv;
        const int dq = NT / rv, dj = NT - dq * rv;
        int q = threadIdx.x / rv, j = threadIdx.x - q * rv;
        const int4 *ti = reinterpret_cast<const int4 *>(v.idx);
        const float4 *wi = reinterpret_cast<const float4 *>(v.w);
        const uint64_t pol = policy_evict_first();
        for (int g = threadIdx.x; g < total; g += 2 * NT) {
          const size_t o0 = (size_t)list[q] * rv + j;
          int q1 = q + dq, j1 = j + dj;
          if (j1 >= rv) {
            j1 -= rv;
            q1 += 1;
          }
          const bool h1 = g + NT < total;
          const size_t o1 = h1 ? (size_t)list[q1] * rv + j1 : o0;
          const int4 t0 = ld_stream_i4(ti + o0, pol), t1 = ld_stream_i4(ti + o1, pol);
          const float4 w0 = ld_stream_f4(wi + o0, pol), w1 = ld_stream_f4(wi + o1, pol);
          acc_add4(base_a, base_b, 0, t0, w0);
          if (h1) acc_add4(base_a, base_b, 0, t1, w1);
          q = q1 + dq;
          j = j1 + dj;
          if (j >= rv) {
            j -= rv;
            q += 1;
          }
        }
      } else if (flat) {
        // ---- delivery, larger team, flat: each thread walks synapses f = tid, tid + NT,
        // ... of the concatenated segments (consecutive lanes, consecutive synapses),
        // eight table reads in flight, no shuffles; its next-step drive is computed
        // while the reads are in flight
        for (int f0 = threadIdx.x, pass = 0; pass == 0 || f0 < F; f0 += 8 * NT, ++pass) {
          int t[8];
          float w[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const int f = f0 + u * NT;
            t[u] = -1;
            w[u] = 0.0f;
            if (f < F) {
              const int q = s_ex[f];
              const long long off = (long long)s_spk[q] * v.stride + s_sb[q] + (f - s_pre[q]);
              // (the separate arrays: consecutive lanes read consecutive synapses here, and
              // two 4-byte loads measured faster than one 8-byte load of the interleaved rows)
              t[u] = __ldg(v.idx + off);
              w[u] = __ldg(v.w + off);
            }
          }
          if (pass == 0 && zwant && threadIdx.x < cnt)
            s_z[threadIdx.x] = normal(v.seed, (uint64_t)(lo + threadIdx.x), (uint64_t)(t_abs + 1));
#pragma unroll
          for (int u = 0; u < 8; ++u)
            if (t[u] >= 0) acc_add(base_a, base_b, (unsigned)(t[u] - (int)lo), wfix(w[u]));
        }
        zdone = zwant ? min(cnt, NT) : 0;
      } else if (it.mode == kDeliverGroup) {
        // ---- delivery, larger team, eight lanes a spike (long segments): warps take the
        // step's spikes in batches of 32 as in the run mapping (`wpb` warps sharing a batch's
        // rounds when there are fewer batches than warps); a batch is walked in 8 rounds of 4
        // spikes, lane group g (lanes 8g .. 8g+7) reading spike 4r+g's segment in contiguous
        // 64-synapse steps, eight reads a lane in flight.  No search: a segment's synapses
        // need no shuffles to find their spike.  The next batch's ids and bounds are loaded
        // while the current one is walked.
        const uint64_t pkeep = policy_evict_last();
        const int nbatch = (Kw + 31) >> 5;
        const int wpb = nbatch >= kWarps ? 1 : min(8, kWarps / max(nbatch, 1));
        const int groups = kWarps / wpb, gw = warp / wpb, wi = warp % wpb;
        const int sub = lane & 7, grp = lane >> 3;
        int s = 0, b = 0, e = 0;
        auto fetch = [&](int batch) {
          const int q = batch * 32 + lane;
          s = 0;
          b = 0;
          e = 0;
          if (gw < groups && batch < nbatch && q < Kw) {
            s = gl ? tagged_id(dense + q, tag, sh, it.sync, lim) : list[q];
            const uint16_t *so = it.seg + (size_t)s * segw + rank;
            b = ld_keep_u16(so, pkeep);
            e = ld_keep_u16(so + 1, pkeep);
          }
        };
        fetch(gw);
        for (int batch = gw; gw < groups && batch < nbatch; batch += groups) {
          const long long rowb = (long long)s * v.stride + b;  // segment start of this lane's spike
          const int len = e - b;
          fetch(batch + groups);  // next batch, in flight meanwhile
          for (int r = wi; r < 8; r += wpb) {
            const long long rb = __shfl_sync(0xFFFFFFFFu, rowb, r * 4 + grp);
            const int ln = __shfl_sync(0xFFFFFFFFu, len, r * 4 + grp);
            for (int k0 = 0; k0 < ln; k0 += 64) {
              int t[8];
              float w[8];
#pragma unroll
              for (int u = 0; u < 8; ++u) {
                const int k = k0 + u * 8 + sub;
                t[u] = -1;
                w[u] = 0.0f;
                if (k < ln) synapse(rb + k, t[u], w[u]);
              }
#pragma unroll
              for (int u = 0; u < 8; ++u)
                if (t[u] >= 0) acc_add(base_a, base_b, (unsigned)(t[u] - (int)lo), wfix(w[u]));
            }
          }
        }
      } else {
        // ---- delivery, larger team: this rank's segment of every spiking row.  Spikes go
        // to warps in batches of 32; when there are fewer batches than warps, `wpb` warps
        // share a batch and split its run.  The next batch's spike ids and segment bounds
        // are loaded before the current run is walked.
        const uint64_t pkeep = policy_evict_last();
        const int nbatch = (Kw + 31) >> 5;
        const int wpb = nbatch >= kWarps ? 1 : kWarps / max(nbatch, 1);
        const int groups = kWarps / wpb, gw = warp / wpb, wi = warp % wpb;
        int s = 0, b = 0, len = 0;
        auto fetch = [&](int batch) {
          const int q = batch * 32 + lane;
          s = 0;
          b = 0;
          len = 0;
          if (gw < groups && batch < nbatch && q < Kw) {
            s = gl ? tagged_id(dense + q, tag, sh, it.sync, lim) : list[q];
            const uint16_t *so = it.seg + (size_t)s * segw + rank;
            b = ld_keep_u16(so, pkeep);
            len = ld_keep_u16(so + 1, pkeep) - b;
          }
        };
        fetch(gw);
        for (int batch = gw; gw < groups && batch < nbatch; batch += groups) {
          int incl = len;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= o) incl += y;
          }
          const int total = __shfl_sync(0xFFFFFFFFu, incl, 31);
          const int excl = incl - len;
          const long long rowoff = (long long)s * v.stride + b - excl;  // synapse f of the run: rowoff_j + f
          fetch(batch + groups);                                        // next batch, in flight meanwhile
          for (int f0 = wi * 256; f0 < total; f0 += wpb * 256) {
            int t[8];
            float w[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
              const int f = f0 + u * 32 + lane;
              // spike j of the run holding f: last lane whose exclusive prefix is <= f
              int jj = 0;
#pragma unroll
              for (int step = 16; step; step >>= 1) {
                const int e = __shfl_sync(0xFFFFFFFFu, excl, jj + step);
                if (e <= f) jj += step;
              }
              const long long off = __shfl_sync(0xFFFFFFFFu, rowoff, jj) + f;
              t[u] = -1;
              w[u] = 0.0f;
              if (f < total) {
                synapse(off, t[u], w[u]);
              }
            }
#pragma unroll
            for (int u = 0; u < 8; ++u)
              if (t[u] >= 0) acc_add(base_a, base_b, (unsigned)(t[u] - (int)lo), wfix(w[u]));
          }
        }
      }
    }
    // ---- tail, by warps as they finish delivering: the raster and the statistics of this
    // rank's spikes (from the highest thread down, i.e. warps that had no delivery batch
    // first), then the next step's drive in chunks of 32 neurons
    for (int j = NT - 1 - threadIdx.x; j < nown; j += NT) {
      const int n = s_own[j];
      const long long pos = base + my_off + j;
      if (pos < v.raster_cap) v.raster[pos] = n;
      SpikeStat st = v.sstat[n];
      st.nospks += 1;
      if (st.last >= 0) {
        const long long isi = t_abs - st.last;
        st.nisi += 1;
        st.s1 += isi;
        st.s2 += isi * isi;
      }
      st.last = (int)t_abs;
      v.sstat[n] = st;
    }
    if (zwant)
      for (;;) {
        int c = 0;
        if (lane == 0) c = atomicAdd(&sh.work[par], 1);
        c = __shfl_sync(0xFFFFFFFFu, c, 0) * 32 + zdone;
        if (c >= cnt) break;
        const int i = c + lane;
        if (i < cnt) s_z[i] = normal(v.seed, (uint64_t)(lo + i), (uint64_t)(t_abs + 1));
      }
    __syncthreads();
    if (gl && sh.fail) return;
    base += K;
  }
  // pending currents (from the last delivery) and the state back to global memory
  for (int i = threadIdx.x; i < cnt; i += NT) {
    v.acc[lo + i] = (long long)s_a[i] * 65536 + s_b[i];
    if (L.vu_sm) v.vu[lo + i] = s_vu[i];
  }
  __syncthreads();
}

// The persistent grid: CTAs take (network, rank) slots until the queue is empty.
template <int NT, bool kPair>
__global__ void __launch_bounds__(NT, 1) k_team(const TeamItem *__restrict__ items, const int2 *__restrict__ slots,
                                                const int *nslots, int *slot_head, unsigned long long limit_ns,
                                                int stall) {
  extern __shared__ __align__(16) unsigned char s_raw[];
  __shared__ TeamShared sh;
  const int ns = *nslots;
  for (;;) {
    if (threadIdx.x == 0) sh.slot = atomicAdd(slot_head, 1);
    __syncthreads();
    const int sl = sh.slot;
    __syncthreads();
    if (sl >= ns) break;
    const int2 x = slots[sl];
    // the network's descriptor in shared memory: read on every step's dependent chains
    __shared__ TeamItem s_it;
    if (threadIdx.x == 0) s_it = items[x.x];
    __syncthreads();
    if (s_it.steps > 0) team_run<NT, kPair>(s_it, x.y, s_raw, sh, limit_ns, stall);
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------------------
// Launchers.
// ---------------------------------------------------------------------------------------

size_t team_smem(int64_t rc, int team) {
  if (rc < 1 || team < 1 || team > kMaxTeam) return 0;
  const int cap = team_window(rc, team);
  if (team > 1 && cap == 0) return 0;
  const size_t bytes = team_layout(rc, team, cap).bytes;
  return bytes > kTeamSmemLimit ? 0 : (bytes < 16 ? 16 : bytes);
}

// The kernel's shared-memory ceiling is always the largest layout's (every team layout
// stays under it), so host threads that launch teams of different sizes never lower it
// under one another, and a captured launch needs no attribute call.
template <int NT>
static cudaError_t team_ceiling_nt() {
  cudaError_t e = cudaFuncSetAttribute(k_team<NT, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTeamSmemLimit);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_team<NT, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTeamSmemLimit);
  return e;
}

cudaError_t team_smem_ceiling() {
  cudaError_t e = team_ceiling_nt<kTeamNT>();
  return e == cudaSuccess ? team_ceiling_nt<kTeamNTSmall>() : e;
}

// CTAs of the team kernel with `smem` bytes of shared memory that fit an SM (both table
// layouts' instantiations; they need the same resources)
template <int NT>
static cudaError_t team_occupancy(size_t smem, int *occ) {
  int a = 0, b = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_team<NT, true>, NT, smem);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_team<NT, false>, NT, smem);
  *occ = a < b ? a : b;
  return e;
}

cudaError_t team_max_blocks(size_t smem, int *out, int nt) {
  if (smem > kTeamSmemLimit || (nt != kTeamNT && nt != kTeamNTSmall)) return cudaErrorInvalidValue;
  cudaError_t e = team_smem_ceiling();
  if (e != cudaSuccess) return e;
  int occ = 0;
  e = nt == kTeamNT ? team_occupancy<kTeamNT>(smem, &occ) : team_occupancy<kTeamNTSmall>(smem, &occ);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  *out = occ * sms;
  return cudaSuccess;
}

cudaError_t launch_team(const TeamItem *items, const int2 *slots, const int *nslots, int *slot_head, int grid,
                        size_t smem, unsigned long long limit_ns, int stall, cudaStream_t s, bool pair, int nt) {
  if (smem > kTeamSmemLimit || (nt != kTeamNT && nt != kTeamNTSmall)) return cudaErrorInvalidValue;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)nt);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (nt == kTeamNTSmall)
    return pair ? cudaLaunchKernelEx(&cfg, k_team<kTeamNTSmall, true>, items, slots, nslots, slot_head, limit_ns, stall)
                : cudaLaunchKernelEx(&cfg, k_team<kTeamNTSmall, false>, items, slots, nslots, slot_head, limit_ns, stall);
  return pair ? cudaLaunchKernelEx(&cfg, k_team<kTeamNT, true>, items, slots, nslots, slot_head, limit_ns, stall)
              : cudaLaunchKernelEx(&cfg, k_team<kTeamNT, false>, items, slots, nslots, slot_head, limit_ns, stall);
}

cudaError_t launch_rows_sorted(const NetView &v, int *unsorted, cudaStream_t s) {
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaError_t e = cudaMemsetAsync(unsorted, 0, sizeof(int), s);
  if (e != cudaSuccess) return e;
  k_rows_sorted<<<(unsigned)(sms * 8), 512, 0, s>>>(v, unsorted);
  return cudaGetLastError();
}

// One CTA per row, as many resident as fit (at most one per row).  The shared-memory
// ceiling is the same for every network, so that host threads sorting rows of different
// lengths never lower it under one another's launch.
template <typename Kernel>
static cudaError_t row_grid(Kernel kern, int nt, size_t smem, int64_t rows, unsigned *grid) {
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  if (e != cudaSuccess) return e;
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, nt, smem);
  if (occ < 1) occ = 1;
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int64_t g = (int64_t)sms * occ;
  *grid = (unsigned)(g > rows ? rows : g);
  return cudaSuccess;
}

template <int E>
static cudaError_t sort_rows_e(const NetView &v, int p2, int nt, cudaStream_t s) {
  const size_t smem = nt > 32 ? (size_t)p2 * 8 : 0;  // (one warp needs no shared memory)
  unsigned g = 0;
  cudaError_t e = row_grid(k_sort_rows<E>, nt, smem, v.n, &g);
  if (e != cudaSuccess) return e;
  k_sort_rows<E><<<g, nt, smem, s>>>(v, p2);
  return cudaGetLastError();
}

template <int E>
static cudaError_t sort_gen_e(const NetView &v, int p2, int pb, cudaStream_t s) {
  const int nt = p2 / E, nb = std::max(nt, p2 / 2);
  int sh = 0;
  while ((v.n >> sh) >= nb) ++sh;
  const size_t smem = ((size_t)nb + 32 + 2 * (size_t)v.stride) * 4;
  unsigned g = 0;
  cudaError_t e = row_grid(k_sort_gen<E>, nt, smem, v.n, &g);
  if (e != cudaSuccess) return e;
  k_sort_gen<E><<<g, nt, smem, s>>>(v, pb, nb, sh);
  return cudaGetLastError();
}

cudaError_t launch_sort_rows(const NetView &v, bool generated, cudaStream_t s) {
  int p2 = 32, pb = 5;
  while (p2 < v.stride) p2 <<= 1, ++pb;
  if ((size_t)p2 * 8 > 200 * 1024) return cudaErrorInvalidValue;
  if (generated && ((uint64_t)v.n << pb) + (uint64_t)p2 - 1 < 0xFFFFFFFFull) {
    // E keys a thread: 8 (16 for rows longer than 8192), fewer for rows shorter than 256
    const int E = p2 / 32 < 8 ? p2 / 32 : (p2 / 8 > 1024 ? 16 : 8);
    switch (E) {
      case 1: return sort_gen_e<1>(v, p2, pb, s);
      case 2: return sort_gen_e<2>(v, p2, pb, s);
      case 4: return sort_gen_e<4>(v, p2, pb, s);
      case 8: return sort_gen_e<8>(v, p2, pb, s);
      case 16: return sort_gen_e<16>(v, p2, pb, s);
      default: return cudaErrorInvalidValue;
    }
  }
  const int nt = std::min(1024, std::max(32, p2 / 4));  // four keys a thread (up to 16 for long rows)
  switch (p2 / nt) {
    case 1: return sort_rows_e<1>(v, p2, nt, s);
    case 2: return sort_rows_e<2>(v, p2, nt, s);
    case 4: return sort_rows_e<4>(v, p2, nt, s);
    case 8: return sort_rows_e<8>(v, p2, nt, s);
    case 16: return sort_rows_e<16>(v, p2, nt, s);
    default: return cudaErrorInvalidValue;
  }
}

// ---------------------------------------------------------------------------------------
// Set-up and read-back of a launch over many networks, one CTA per network.  k_round_clear
// zeroes each network's per-step counts and stamps of the launch, its status word and its
// team's error word and spike records; k_round_gather packs its status words, counts,
// raster offsets and stamps at its offset in one buffer (round_pack_bytes each), which one
// copy brings to the host.  Networks with no steps in the launch are skipped.
// ---------------------------------------------------------------------------------------
__global__ void k_round_clear(const TeamItem *items) {
  const TeamItem &it = items[blockIdx.x];
  const int s = it.steps;
  if (s <= 0) return;
  for (int i = threadIdx.x; i < s; i += blockDim.x) it.v.counts[i] = 0;
  for (int i = threadIdx.x; i < 2 * s + 2; i += blockDim.x) it.v.stamps[i] = 0ull;
  if (threadIdx.x == 0) *it.v.status = 0;
  unsigned long long *g = reinterpret_cast<unsigned long long *>(it.sync);
  const int64_t words = (int64_t)(1 + 2 * it.team * kRecLines) * (int64_t)(sizeof(GridSync) / 8);
  for (int64_t i = threadIdx.x; i < words; i += blockDim.x) g[i] = 0ull;
}

__global__ void k_round_gather(const TeamItem *items, const int64_t *off, unsigned char *pack) {
  const TeamItem &it = items[blockIdx.x];
  const int s = it.steps;
  if (s <= 0) return;
  unsigned char *p = pack + off[blockIdx.x];
  if (threadIdx.x == 0) {
    reinterpret_cast<int *>(p)[0] = *it.v.status;
    reinterpret_cast<int *>(p)[1] = it.sync->error;
  }
  int *c = reinterpret_cast<int *>(p + 8);
  long long *b = reinterpret_cast<long long *>(p + 8 + (((size_t)s * 4 + 7) & ~(size_t)7));
  unsigned long long *t = reinterpret_cast<unsigned long long *>(b + s);
  for (int i = threadIdx.x; i < s; i += blockDim.x) {
    c[i] = it.v.counts[i];
    b[i] = it.v.base[i];
  }
  for (int i = threadIdx.x; i < 2 * s; i += blockDim.x) t[i] = it.v.stamps[i];
}

cudaError_t launch_round_clear(const TeamItem *items, int count, cudaStream_t s) {
  k_round_clear<<<(unsigned)count, 256, 0, s>>>(items);
  return cudaGetLastError();
}

cudaError_t launch_round_gather(const TeamItem *items, const int64_t *off, int count, unsigned char *pack,
                                cudaStream_t s) {
  k_round_gather<<<(unsigned)count, 256, 0, s>>>(items, off, pack);
  return cudaGetLastError();
}

cudaError_t launch_segoff(const NetView &v, int team, int64_t rc, uint16_t *seg, cudaStream_t s) {
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int64_t blocks = (v.n + 7) / 8;
  if (blocks > (int64_t)sms * 16) blocks = (int64_t)sms * 16;
  k_segoff<<<(unsigned)blocks, 256, 0, s>>>(v, team, rc, seg);
  return cudaGetLastError();
}

cudaError_t launch_inbound(const NetView &v, unsigned *cnt, unsigned long long *mag, unsigned long long *out,
                           cudaStream_t s) {
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaError_t e = cudaMemsetAsync(cnt, 0, (size_t)v.n * 4, s);
  if (e == cudaSuccess && mag) e = cudaMemsetAsync(mag, 0, (size_t)v.n * 8, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(out, 0, 24, s);
  if (e != cudaSuccess) return e;
  k_inbound<<<(unsigned)(sms * 8), 512, 0, s>>>(v, cnt, mag, out + 2);
  k_inbound_max<<<(unsigned)(sms * 2), 512, 0, s>>>(v.n, cnt, mag, out);
  return cudaGetLastError();
}

cudaError_t launch_pairs(const NetView &v, cudaStream_t s) {
  if (!v.pair) return cudaErrorInvalidValue;
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  k_pairs<<<(unsigned)(sms * 8), 512, 0, s>>>(v, const_cast<int2 *>(v.pair));
  return cudaGetLastError();
}

}  // namespace g4s
