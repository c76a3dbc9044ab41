// g4s_owner.cu — the SKL step loop with owner-computes delivery (the GB300 design of
// SKL_deliverspks, gpu4snn.cu:669-716), plus the table preparation it needs.
//
// Target ownership.  The neurons are split into C contiguous slices of Rc = ceil(N/C),
// one per CTA of a cooperative grid of one CTA per SM.  A CTA keeps the synaptic current
// of its slice in shared memory for the whole launch, as two 32-bit words per neuron:
// the Q32.32 current q = A * 2^16 + B, with B the sum of the weights' low 16 bits and A
// the sum of their high 48 bits.  Shared-memory 32-bit atomics are about five times
// faster than 64-bit ones on this part, and the split is exact as long as no neuron has
// 65536 or more incoming synapses and the sum of |q_i| / 2^16 + 1 over its incoming
// synapses stays below 2^31; k_inbound checks both once per table (the host falls back
// to the global-atomic persistent kernel otherwise).
//
// Per step:
//   update    each CTA updates its own neurons (current read from and cleared in shared
//             memory), buffers its spikes in shared memory and appends them to the global
//             spike list of the step with one atomic per CTA;
//   barrier   grid barrier with a bounded spin;
//   delivery  every CTA streams, for every spike of the step, the segment of the spiking
//             row whose targets fall in its slice (rows are sorted by target and a
//             per-row offset table gives the segment) and adds each weight into its own
//             shared memory.  A warp takes 32 spikes at once, scans their segment lengths
//             and walks the concatenated segments, four synapses per lane in flight;
//   barrier   block barrier (the next update reads only this CTA's shared memory).
// No global atomic per synapse and no global current array inside the launch.
#include <cuda_runtime.h>

#include <cstdint>

#include "g4s_device.cuh"
#include "g4s_internal.h"

namespace g4s {

// ---------------------------------------------------------------------------------------
// Row sort: every row's (target, weight) pairs in ascending target order, unused slots
// (negative targets, i.e. huge as unsigned) last.  One CTA per row, bitonic network over
// 64-bit keys (target << 32 | weight bits) in shared memory.
// ---------------------------------------------------------------------------------------
__global__ void k_sort_rows(NetView v, int p2) {
  extern __shared__ unsigned long long s_key[];
  for (int64_t row = blockIdx.x; row < v.n; row += gridDim.x) {
    int *ri = const_cast<int *>(v.idx) + row * v.stride;
    float *rw = const_cast<float *>(v.w) + row * v.stride;
    for (int j = threadIdx.x; j < p2; j += blockDim.x)
      s_key[j] = j < v.stride ? ((unsigned long long)(unsigned)ri[j] << 32) | __float_as_uint(rw[j])
                              : 0xFFFFFFFFFFFFFFFFull;
    __syncthreads();
    for (int k = 2; k <= p2; k <<= 1)
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int i = threadIdx.x; i < p2; i += blockDim.x) {
          const int l = i ^ j;
          if (l > i) {
            const unsigned long long a = s_key[i], b = s_key[l];
            const bool up = (i & k) == 0;
            if ((a > b) == up) {
              s_key[i] = b;
              s_key[l] = a;
            }
          }
        }
        __syncthreads();
      }
    for (int j = threadIdx.x; j < v.stride; j += blockDim.x) {
      const unsigned long long x = s_key[j];
      ri[j] = (int)(x >> 32);
      rw[j] = __uint_as_float((unsigned)x);
    }
    __syncthreads();
  }
}

// Segment table: seg[row][k] = first slot of the sorted row whose target is >= k*Rc, for
// k = 0..C (unused slots compare as huge and lie beyond seg[row][C]).  One warp per row,
// one binary search per boundary.
__global__ void k_segoff(NetView v, int C, int64_t Rc, uint16_t *seg) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t row = warp; row < v.n; row += nwarps) {
    const int *ri = v.idx + row * v.stride;
    for (int k = lane; k <= C; k += 32) {
      const int64_t bound = (int64_t)k * Rc;
      int lo = 0, hi = v.stride;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if ((int64_t)(unsigned)ri[mid] < bound)
          lo = mid + 1;
        else
          hi = mid;
      }
      seg[row * (C + 1) + k] = (uint16_t)lo;
    }
  }
}

// Exactness bound of the split accumulation: per target, the number of incoming synapses
// and the sum of (|q| >> 16) + 1 over them; out[0] = max count, out[1] = max sum.
__global__ void k_inbound(NetView v, unsigned *cnt, unsigned long long *mag) {
  const int64_t total = v.n * (int64_t)v.stride;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x) {
    const int t = v.idx[g];
    if (t < 0) continue;
    const long long q = wfix(v.w[g]);
    const unsigned long long a = (unsigned long long)(q < 0 ? -q : q) >> 16;
    atomicAdd(cnt + t, 1u);
    atomicAdd(mag + t, a + 1ull);
  }
}

__global__ void k_inbound_max(int64_t n, const unsigned *cnt, const unsigned long long *mag,
                              unsigned long long *out) {
  unsigned long long mc = 0, mm = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    mc = max(mc, (unsigned long long)cnt[i]);
    mm = max(mm, mag[i]);
  }
  atomicMax(out, mc);
  atomicMax(out + 1, mm);
}

// ---------------------------------------------------------------------------------------
// Grid barrier of the owner kernel: monotone arrival counter, bounded spin (see
// grid_barrier); every CTA leaves its loop on a timeout or on the error word.
// ---------------------------------------------------------------------------------------

// Split-accumulator add: A += q >> 16 (arithmetic), B += q & 0xFFFF.
__device__ __forceinline__ void acc_add(unsigned base_a, unsigned base_b, unsigned off, long long q) {
  asm volatile("red.shared.add.s32 [%0], %1;" ::"r"(base_a + off * 4u), "r"((int)(q >> 16)) : "memory");
  asm volatile("red.shared.add.u32 [%0], %1;" ::"r"(base_b + off * 4u), "r"((unsigned)(q & 0xFFFF)) : "memory");
}

// ---------------------------------------------------------------------------------------
// The step loop.
// ---------------------------------------------------------------------------------------
template <int NT>
__global__ void __launch_bounds__(NT, 1)
    k_owner(NetView v, OwnerGeom geo, const uint16_t *__restrict__ seg, int64_t t_abs0, int nsteps, int last_chunk,
            GridSync *gs, unsigned long long limit_ns, int stall) {
  extern __shared__ __align__(16) unsigned char s_raw[];
  const int rc = (int)geo.rc;
  int *s_a = reinterpret_cast<int *>(s_raw);
  unsigned *s_b = reinterpret_cast<unsigned *>(s_raw + (size_t)rc * 4);
  int *s_spk = reinterpret_cast<int *>(s_raw + (size_t)rc * 8);
  __shared__ int s_nspk;
  __shared__ long long s_gpos;

  const int C = (int)gridDim.x;
  const unsigned nb = gridDim.x + (unsigned)stall;  // stall > 0 only under fault injection
  const int k = blockIdx.x;
  const int64_t lo = min((int64_t)k * rc, v.n);
  const int64_t hi = min(lo + rc, v.n);
  const int cnt = (int)(hi - lo);
  const unsigned base_a = (unsigned)__cvta_generic_to_shared(s_a);
  const unsigned base_b = (unsigned)__cvta_generic_to_shared(s_b);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int kWarps = NT / 32;
  const unsigned segw = (unsigned)C + 1;

  for (int i = threadIdx.x; i < cnt; i += NT) {
    const long long q = __ldcg(v.acc + lo + i);
    s_a[i] = (int)(q >> 16);
    s_b[i] = (unsigned)(q & 0xFFFF);
  }
  if (threadIdx.x == 0) s_nspk = 0;
  __syncthreads();

  unsigned epoch = 0;
  long long base = 0;
  for (int lt = 0; lt < nsteps; ++lt) {
    const int64_t t_abs = t_abs0 + lt;
    const bool last = last_chunk && lt == nsteps - 1;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      v.base[lt] = base;
      v.stamps[2 * lt] = globaltimer();
    }
    // ---- update of the owned neurons, two per thread per round with the loads first
    for (int i0 = threadIdx.x; i0 < cnt; i0 += 2 * NT) {
      const int i1 = i0 + NT;
      const bool h1 = i1 < cnt;
      const int64_t n0 = lo + i0, n1 = lo + (h1 ? i1 : i0);
      float2 s0 = v.vu[n0], s1 = v.vu[n1];
      const float4 p0 = v.abcd[n0], p1 = v.abcd[n1];
      const long long a0 = (long long)s_a[i0] * 65536 + s_b[i0];
      const long long a1 = h1 ? (long long)s_a[i1] * 65536 + s_b[i1] : 0;
      s_a[i0] = 0;
      s_b[i0] = 0;
      if (h1) {
        s_a[i1] = 0;
        s_b[i1] = 0;
      }
      const float z0 = normal(v.seed, (uint64_t)n0, (uint64_t)t_abs);
      const float z1 = normal(v.seed, (uint64_t)n1, (uint64_t)t_abs);
      float I0, I1;
      const bool k0 = izh_step(s0.x, s0.y, I0, p0, n0 < v.nexc ? v.ge : v.gi, z0, a0);
      const bool k1 = izh_step(s1.x, s1.y, I1, p1, n1 < v.nexc ? v.ge : v.gi, z1, a1) && h1;
      v.vu[n0] = s0;
      if (h1) v.vu[n1] = s1;
      if (last) {
        v.ilast[n0] = I0;
        if (h1) v.ilast[n1] = I1;
      }
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const bool spk = h ? k1 : k0;
        if (!spk) continue;
        const int64_t n = h ? n1 : n0;
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
        s_spk[atomicAdd(&s_nspk, 1)] = (int)n;
      }
    }
    __syncthreads();
    const int nspk = s_nspk;
    if (threadIdx.x == 0 && nspk) s_gpos = atomicAdd(v.counts + lt, nspk);
    __syncthreads();
    for (int j = threadIdx.x; j < nspk; j += NT) {
      const long long pos = base + s_gpos + j;
      if (pos < v.raster_cap)
        v.raster[pos] = s_spk[j];
      else
        atomicCAS(v.status, 0, kErrOverflowCode);
    }
    if (threadIdx.x == 0) s_nspk = 0;
    // ---- the step's spike list is complete everywhere after this barrier
    if (!grid_barrier(gs, nb, epoch, limit_ns)) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) v.stamps[2 * lt + 1] = globaltimer();
    // ---- delivery of this step's spikes into this CTA's slice.  Spikes go to warps in
    // batches of 32; when there are fewer batches than warps, `wpb` warps share a batch
    // and split its run.  The next batch's spike ids and segment bounds are loaded before
    // the current run is walked.
    const int K = __ldcg(v.counts + lt);
    const int *list = v.raster + base;
    const int nbatch = (K + 31) >> 5;
    const int wpb = nbatch >= kWarps ? 1 : kWarps / max(nbatch, 1);
    const int groups = kWarps / wpb, gw = warp / wpb, wi = warp % wpb;
    int s = 0, b = 0, len = 0;
    auto fetch = [&](int batch) {
      const int q = batch * 32 + lane;
      s = 0;
      b = 0;
      len = 0;
      if (gw < groups && batch < nbatch && q < K) {
        s = __ldcg(list + q);
        const uint16_t *so = seg + (size_t)s * segw + k;
        b = so[0];
        len = (int)so[1] - b;
      }
    };
    fetch(gw);
    for (int batch = gw; gw < groups && batch < nbatch; batch += groups) {
      // scan this batch's segment lengths into one run
      int incl = len;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += y;
      }
      const int total = __shfl_sync(0xFFFFFFFFu, incl, 31);
      const int excl = incl - len;
      const long long rowoff = (long long)s * v.stride + b - excl;  // synapse f of the run is at rowoff_j + f
      fetch(batch + groups);                                        // next batch, in flight meanwhile
      for (int f0 = wi * 256; f0 < total; f0 += wpb * 256) {
        int t[8];
        float w[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int f = f0 + u * 32 + lane;
          // spike j of the run holding f: last lane whose exclusive prefix is <= f
          int j = 0;
#pragma unroll
          for (int step = 16; step; step >>= 1) {
            const int e = __shfl_sync(0xFFFFFFFFu, excl, j + step);
            if (e <= f) j += step;
          }
          const long long off = __shfl_sync(0xFFFFFFFFu, rowoff, j) + f;
          t[u] = -1;
          w[u] = 0.0f;
          if (f < total) {
            t[u] = __ldg(v.idx + off);
            w[u] = __ldg(v.w + off);
          }
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (t[u] >= 0) acc_add(base_a, base_b, (unsigned)(t[u] - (int)lo), wfix(w[u]));
      }
    }
    __syncthreads();
    base += K;
  }
  // pending currents (from the last delivery) back to global memory for the next launch
  for (int i = threadIdx.x; i < cnt; i += NT) v.acc[lo + i] = (long long)s_a[i] * 65536 + s_b[i];
}

// ---------------------------------------------------------------------------------------
// Launchers and geometry.
// ---------------------------------------------------------------------------------------
constexpr int kOwnNT = 1024;

size_t owner_smem(int64_t rc) { return (size_t)rc * 12 + 16; }

cudaError_t owner_max_blocks(size_t smem, int *out) {
  cudaError_t e = cudaFuncSetAttribute(k_owner<kOwnNT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int occ = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_owner<kOwnNT>, kOwnNT, smem);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  *out = occ * sms;
  return cudaSuccess;
}

cudaError_t launch_sort_rows(const NetView &v, cudaStream_t s) {
  int p2 = 32;
  while (p2 < v.stride) p2 <<= 1;
  const size_t smem = (size_t)p2 * 8;
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(k_sort_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int nt = p2 >= 4096 ? 1024 : (p2 >= 1024 ? 256 : 128);
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_sort_rows, nt, smem);
  if (occ < 1) occ = 1;
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int64_t g = (int64_t)sms * occ;
  if (g > v.n) g = v.n;
  k_sort_rows<<<(unsigned)g, nt, smem, s>>>(v, p2);
  return cudaGetLastError();
}

cudaError_t launch_segoff(const NetView &v, const OwnerGeom &geo, uint16_t *seg, cudaStream_t s) {
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int64_t blocks = (v.n + 7) / 8;
  if (blocks > (int64_t)sms * 16) blocks = (int64_t)sms * 16;
  k_segoff<<<(unsigned)blocks, 256, 0, s>>>(v, geo.p, geo.rc, seg);
  return cudaGetLastError();
}

cudaError_t launch_inbound(const NetView &v, unsigned *cnt, unsigned long long *mag, unsigned long long *out,
                           cudaStream_t s) {
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaError_t e = cudaMemsetAsync(cnt, 0, (size_t)v.n * 4, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(mag, 0, (size_t)v.n * 8, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(out, 0, 16, s);
  if (e != cudaSuccess) return e;
  k_inbound<<<(unsigned)(sms * 8), 512, 0, s>>>(v, cnt, mag);
  k_inbound_max<<<(unsigned)(sms * 2), 512, 0, s>>>(v.n, cnt, mag, out);
  return cudaGetLastError();
}

cudaError_t launch_owner(const NetView &v, const OwnerGeom &geo, const uint16_t *seg, int64_t t_abs0, int nsteps,
                         bool last_chunk, GridSync *gs, unsigned long long limit_ns, int stall, cudaStream_t s) {
  const size_t smem = owner_smem(geo.rc);
  cudaError_t e = cudaFuncSetAttribute(k_owner<kOwnNT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)geo.p);
  cfg.blockDim = dim3(kOwnNT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const int last = last_chunk ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, k_owner<kOwnNT>, v, geo, seg, t_abs0, nsteps, last, gs, limit_ns, stall);
}

}  // namespace g4s
