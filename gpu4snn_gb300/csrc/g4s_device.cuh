// g4s_device.cuh — device building blocks of the GB300 simulation step.
//
// Every float operation of the neuron update and of the normal transform is an explicit
// round-to-nearest intrinsic (__fmul_rn, __fadd_rn, ...), so no multiply-add is fused and
// the kernels compute exactly the binary32 sequence of the CPU oracle.  The equations are
// the reference's (gpu4snn.cu:286-320 parameters, :356-405 update); the random numbers are
// a counter-based Philox4x64-10 stream instead of per-neuron cuRAND XORWOW state.
#pragma once
#include <cstdint>

#include "g4s_types.h"

namespace g4s {

// ---------------------------------------------------------------------------------------
// Philox4x64-10 (Salmon et al., SC'11): key = (seed, stream), counter = (c0, c1, c2, 0).
// ---------------------------------------------------------------------------------------
struct U64x4 {
  uint64_t x[4];
};

__device__ __forceinline__ U64x4 philox(uint64_t seed, uint64_t stream, uint64_t c0, uint64_t c1,
                                        uint64_t c2) {
  uint64_t k0 = seed, k1 = stream, x0 = c0, x1 = c1, x2 = c2, x3 = 0;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += 0x9E3779B97F4A7C15ull;
      k1 += 0xBB67AE8584CAA73Bull;
    }
    const uint64_t lo0 = 0xD2E7470EE14C6C93ull * x0, hi0 = __umul64hi(0xD2E7470EE14C6C93ull, x0);
    const uint64_t lo1 = 0xCA5A826395121157ull * x2, hi1 = __umul64hi(0xCA5A826395121157ull, x2);
    const uint64_t n0 = hi1 ^ x1 ^ k0, n2 = hi0 ^ x3 ^ k1;
    x0 = n0;
    x1 = lo1;
    x2 = n2;
    x3 = lo0;
  }
  return U64x4{{x0, x1, x2, x3}};
}

constexpr float kTwoM24 = 5.9604644775390625e-08f;   // 2^-24
constexpr float kTwoM32 = 2.3283064365386963e-10f;   // 2^-32
constexpr float kTwoP32 = 4294967296.0f;             // 2^32

__device__ __forceinline__ float u24(uint64_t x) {
  return __fmul_rn(__uint2float_rn((uint32_t)(x >> 40)), kTwoM24);
}

// Natural log of a positive normal float: x = m 2^e, m in [sqrt(1/2), sqrt(2)],
// log m = 2 atanh((m-1)/(m+1)) by its Taylor series to the 11th power, e*ln2 in a short
// exact high part plus a correction (Cody & Waite).  About 1 ulp.
__device__ __forceinline__ float log_pos(float x) {
  uint32_t bits = __float_as_uint(x);
  int e = (int)(bits >> 23) - 127;
  uint32_t mb = (bits & 0x7FFFFFu) | 0x3F800000u;
  if (mb > 0x3FB504F3u) {
    mb -= 0x00800000u;
    e += 1;
  }
  const float m = __uint_as_float(mb);
  const float f = __fdiv_rn(__fsub_rn(m, 1.0f), __fadd_rn(m, 1.0f));
  const float f2 = __fmul_rn(f, f);
  float p = 0.0909090936f;
  p = __fadd_rn(__fmul_rn(p, f2), 0.111111112f);
  p = __fadd_rn(__fmul_rn(p, f2), 0.142857149f);
  p = __fadd_rn(__fmul_rn(p, f2), 0.2f);
  p = __fadd_rn(__fmul_rn(p, f2), 0.333333343f);
  const float t = __fmul_rn(f2, p);
  const float twof = __fadd_rn(f, f);
  const float series = __fadd_rn(__fmul_rn(twof, t), twof);
  const float ef = __int2float_rn(e);
  const float hi = __fmul_rn(ef, 0.693145751953125f);
  const float lo = __fmul_rn(ef, 1.42860677e-06f);
  return __fadd_rn(hi, __fadd_rn(lo, series));
}

__device__ __forceinline__ float pm1_from24(uint32_t k) {
  return __fmul_rn(__int2float_rn((int)(2u * k + 1u) - 0x1000000), kTwoM24);
}

// Philox4x32-10 (same paper), the cheaper generator of the per-step thalamic drive:
// 32x32->64 products instead of 64x64->128 ones.
__device__ __forceinline__ uint4 philox32(uint32_t k0, uint32_t k1, uint32_t c0, uint32_t c1, uint32_t c2,
                                          uint32_t c3) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    const uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
    const uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
    const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
  }
  return make_uint4(c0, c1, c2, c3);
}

// Standard normal for (neuron, step) by Marsaglia's polar method: one Philox4x32-10 call
// (key = seed words, counter = (neuron, step, attempt, 4)) gives two candidate pairs from
// the top 24 bits of words (0,1) and (2,3); up to 16 calls, z = 0 if all 32 pairs are
// rejected.  Replaces curand_normal (gpu4snn.cu:358).  The first accepted pair is chosen
// before the transform, so a warp runs the log / divide / square root once even when its
// lanes accept different pairs.
__device__ __forceinline__ float normal(uint64_t seed, uint64_t neuron, uint64_t step) {
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  float x = 0.0f, s = 2.0f;
  for (uint32_t attempt = 0; attempt < 16 && !(s < 1.0f); ++attempt) {
    const uint4 o = philox32(k0, k1, (uint32_t)neuron, (uint32_t)step, attempt, (uint32_t)kStreamNoise);
    const float x0 = pm1_from24(o.x >> 8), y0 = pm1_from24(o.y >> 8);
    const float x1 = pm1_from24(o.z >> 8), y1 = pm1_from24(o.w >> 8);
    const float s0 = __fadd_rn(__fmul_rn(x0, x0), __fmul_rn(y0, y0));
    const float s1 = __fadd_rn(__fmul_rn(x1, x1), __fmul_rn(y1, y1));
    if (s0 < 1.0f) {
      x = x0;
      s = s0;
    } else if (s1 < 1.0f) {
      x = x1;
      s = s1;
    }
  }
  if (!(s < 1.0f)) return 0.0f;
  const float q = __fdiv_rn(__fmul_rn(-2.0f, log_pos(s)), s);
  return __fmul_rn(x, __fsqrt_rn(q));
}

// Q32.32 fixed point of one weight (round to nearest even).
__device__ __forceinline__ long long wfix(float w) { return __float2ll_rn(__fmul_rn(w, kTwoP32)); }


// Neuron parameters from one uniform r (initNeuron, gpu4snn.cu:292-317; powf(r,2) -> r*r).
// a, b, c, d are a function of r and the neuron's kind, so a kernel can read r (4 bytes)
// and recompute them instead of reading 16 bytes.
__device__ __forceinline__ float izh_r(uint64_t seed, int64_t i) {
  return u24(philox(seed, kStreamParam, (uint64_t)i, 0, 0).x[0]);
}
__device__ __forceinline__ float4 izh_abcd(float r, bool exc) {
  if (exc) {
    const float r2 = __fmul_rn(r, r);
    return make_float4(0.02f, 0.2f, __fadd_rn(-65.0f, __fmul_rn(15.0f, r2)),
                       __fsub_rn(8.0f, __fmul_rn(6.0f, r2)));
  }
  return make_float4(__fadd_rn(0.02f, __fmul_rn(0.08f, r)), __fsub_rn(0.25f, __fmul_rn(0.05f, r)),
                     -65.0f, 2.0f);
}
__device__ __forceinline__ float4 izh_params(uint64_t seed, int64_t i, int64_t nexc) {
  return izh_abcd(izh_r(seed, i), i < nexc);
}

// One 1 ms step of one neuron (stateupdate, gpu4snn.cu:376-405): I = g z + Isyn, two 0.5 ms
// half-steps of v with the same u and I, u after v, threshold/reset.  Returns the spike flag.
__device__ __forceinline__ bool izh_step(float &v, float &u, float &I, const float4 abcd, float g,
                                         float z, long long acc) {
  I = __fadd_rn(__fmul_rn(g, z), __fmul_rn(__ll2float_rn(acc), kTwoM32));
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    float t1 = __fmul_rn(__fmul_rn(0.04f, v), v);
    t1 = __fadd_rn(t1, __fmul_rn(5.0f, v));
    t1 = __fadd_rn(t1, 140.0f);
    t1 = __fsub_rn(t1, u);
    t1 = __fadd_rn(t1, I);
    v = __fadd_rn(v, __fmul_rn(0.5f, t1));
  }
  u = __fadd_rn(u, __fmul_rn(abcd.x, __fsub_rn(__fmul_rn(abcd.y, v), u)));
  const bool spk = (v >= 30.0f) || !isfinite(v);
  if (spk) {
    v = abcd.z;
    u = __fadd_rn(u, abcd.w);
  }
  return spk;
}

// ---------------------------------------------------------------------------------------
// Memory helpers.
// ---------------------------------------------------------------------------------------
// Streaming 128-bit loads of the connectivity tables: read once per spike, bypass L1 and
// mark the lines evict-first so the L2-resident currents and neuron state stay cached.
__device__ __forceinline__ uint64_t policy_evict_first() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}
__device__ __forceinline__ int4 ld_stream_i4(const int4 *p, uint64_t pol) {
  int4 r;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.s32 {%0,%1,%2,%3}, [%4], %5;"
               : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
               : "l"(p), "l"(pol));
  return r;
}
__device__ __forceinline__ float4 ld_stream_f4(const float4 *p, uint64_t pol) {
  float4 r;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.f32 {%0,%1,%2,%3}, [%4], %5;"
               : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w)
               : "l"(p), "l"(pol));
  return r;
}
// The per-row segment table is small and read for every spike: keep it in L2.
__device__ __forceinline__ uint64_t policy_evict_last() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}
__device__ __forceinline__ int ld_keep_u16(const uint16_t *p, uint64_t pol) {
  unsigned short r;
  asm volatile("ld.global.nc.L2::cache_hint.u16 %0, [%1], %2;" : "=h"(r) : "l"(p), "l"(pol));
  return r;
}
// Fire-and-forget 64-bit integer reduction in L2 (exact, order independent).
__device__ __forceinline__ void red_add(long long *p, long long v) {
  asm volatile("red.relaxed.gpu.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void deliver4(long long *acc, const int4 t, const float4 w) {
  if (t.x >= 0) red_add(acc + t.x, wfix(w.x));
  if (t.y >= 0) red_add(acc + t.y, wfix(w.y));
  if (t.z >= 0) red_add(acc + t.z, wfix(w.z));
  if (t.w >= 0) red_add(acc + t.w, wfix(w.w));
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int ld_relaxed(const int *p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
// Spike records: 64-bit words (tag << 32 | payload), each single-copy atomic, so a reader
// that sees the tag it expects also sees the payload written with it.
__device__ __forceinline__ void st_relaxed_u64(unsigned long long *p, unsigned long long x) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(x) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long *p) {
  unsigned long long r;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(r) : "l"(p) : "memory");
  return r;
}
__device__ __forceinline__ ulonglong2 ld_relaxed_u64x2(const unsigned long long *p) {
  ulonglong2 r;
  asm volatile("ld.relaxed.gpu.global.v2.u64 {%0,%1}, [%2];" : "=l"(r.x), "=l"(r.y) : "l"(p) : "memory");
  return r;
}
__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Grid-wide barrier for co-resident (cooperatively launched) blocks, with a time limit.
// Arrival: one release-add per block on a monotone counter; the barrier of epoch k is
// passed when the counter reaches k * nblocks.  A block that waits longer than limit_ns,
// or sees the error word set, gives up: it records G4S_ERR_TIMEOUT (first writer wins)
// and returns false, and every block then leaves its loop at the next barrier.
__device__ __forceinline__ bool grid_barrier(GridSync *gs, unsigned nblocks, unsigned &epoch,
                                             unsigned long long limit_ns) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    epoch += 1;
    const unsigned target = epoch * nblocks;
    int ok = 1;
    __threadfence();
    atomicAdd(&gs->count, 1u);
    const unsigned long long t0 = globaltimer();
    while ((int)(ld_acquire(&gs->count) - target) < 0) {
      if (ld_relaxed(&gs->error) != 0) {
        ok = 0;
        break;
      }
      if (globaltimer() - t0 > limit_ns) {
        atomicCAS(&gs->error, 0, kErrTimeoutCode);
        ok = 0;
        break;
      }
    }
    if (ok && ld_relaxed(&gs->error) != 0) ok = 0;
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Block-wide stream compaction of one flag per thread: returns this thread's slot in the
// block's compacted run and, through *total, the block's count (threads in id order).
template <int NT>
__device__ __forceinline__ int block_compact(bool flag, int *s_warp, int *total) {
  constexpr int NW = NT / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned ballot = __ballot_sync(0xFFFFFFFFu, flag);
  const int pre = __popc(ballot & ((1u << lane) - 1u));
  if (lane == 0) s_warp[warp] = __popc(ballot);
  __syncthreads();
  if (warp == 0) {
    int c = lane < NW ? s_warp[lane] : 0;
    int incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
      if (lane >= o) incl += y;
    }
    if (lane < NW) s_warp[lane] = incl - c;
    if (lane == 31) s_warp[NW] = incl;
  }
  __syncthreads();
  *total = s_warp[NW];
  return s_warp[warp] + pre;
}

}  // namespace g4s
