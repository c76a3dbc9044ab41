// g4s_fp64check.cu — on-device FP64 check of a network's FP32 trajectory.
//
// The library computes the reference's update in FP32 (gpu4snn.cu:376-405) with exact
// Q32.32 currents.  This check runs an FP64 twin of the same network on the GPU in lockstep
// with the library's own step (the SKL scheme, one step per launch) on the same random
// draws: the float normal of each (neuron, step) and the float parameters promoted to
// double; v and u in double, every operation an explicit round-to-nearest double
// intrinsic in the C order of the reference's expressions (no fused multiply-add); the
// synaptic currents as exact Q64.64 sums of the weights — a 128-bit two's-complement
// integer per neuron, added with two 64-bit atomics and a carry — converted to double,
// correctly rounded, when the neuron consumes them.  Exact sums make the twin independent
// of the delivery order, so it equals the CPU oracle's FP64 mode bit for bit.  After every
// step it reports the maximum, 99th percentile and median of |v32 - v64| over all neurons
// (nearest-rank percentiles) and whether the two steps' spike sets agree.
//
// FP64 arithmetic on the GPU is used only here and in the statistics reductions.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/gpu4snn.h"
#include "g4s_device.cuh"
#include "g4s_internal.h"

using namespace g4s;

namespace {

struct alignas(16) Q128 {
  unsigned long long lo, hi;  // two's complement, value = (hi:lo) x 2^-64
};

// Q64.64 value of a float weight: exact for |w| >= 2^-41 (24 significant bits land on or
// above the 2^-64 bit), rounded to nearest even below.  Weights of magnitude 2^40 or more,
// infinities and NaNs do not fit: they raise *bad and count as 0.
__device__ __forceinline__ Q128 wq64(float w, int *bad) {
  const uint32_t b = __float_as_uint(w);
  const int e = (int)((b >> 23) & 0xFFu);
  Q128 q{0ull, 0ull};
  if (e == 0) return q;  // zero or subnormal (< 2^-126): rounds to 0 at 2^-64
  if (e >= 127 + 40) {
    atomicOr(bad, 1);
    return q;
  }
  const unsigned long long m = (unsigned long long)((b & 0x7FFFFFu) | 0x800000u);  // w = m 2^(e-150)
  const int sh = e - 86;                                                           // w 2^64 = m 2^sh < 2^104
  unsigned __int128 mag;
  if (sh >= 0) {
    mag = (unsigned __int128)m << sh;
  } else {
    const int r = -sh;
    if (r > 25) return q;  // m 2^-r < 2^-1: rounds to 0
    unsigned long long t = m >> r;
    const unsigned long long rem = m & ((1ull << r) - 1ull), half = 1ull << (r - 1);
    if (rem > half || (rem == half && (t & 1ull))) ++t;
    mag = t;
  }
  if (b >> 31) mag = (unsigned __int128)0 - mag;
  q.lo = (unsigned long long)mag;
  q.hi = (unsigned long long)(mag >> 64);
  return q;
}

__device__ __forceinline__ void q128_add(Q128 *a, Q128 x) {
  const unsigned long long old = atomicAdd(&a->lo, x.lo);
  const unsigned long long carry = (old + x.lo < old) ? 1ull : 0ull;  // unsigned wrap of the low word
  const unsigned long long hi = x.hi + carry;
  if (hi) atomicAdd(&a->hi, hi);
}

// (hi:lo) x 2^-64 to the nearest double (ties to even): the top 53 significant bits of the
// magnitude, rounded on the bits below them, scaled by exact powers of two.
__device__ __forceinline__ double q128_to_double(Q128 q) {
  unsigned __int128 x = ((unsigned __int128)q.hi << 64) | q.lo;
  const bool neg = (q.hi >> 63) != 0;
  if (neg) x = (unsigned __int128)0 - x;
  if (x == 0) return 0.0;
  const unsigned long long xh = (unsigned long long)(x >> 64), xl = (unsigned long long)x;
  const int bits = xh ? 128 - __clzll((long long)xh) : 64 - __clzll((long long)xl);
  unsigned long long top;
  int sh = 0;
  if (bits <= 53) {
    top = xl;
  } else {
    sh = bits - 53;
    top = (unsigned long long)(x >> sh);
    const unsigned __int128 rem = x & (((unsigned __int128)1 << sh) - 1);
    const unsigned __int128 half = (unsigned __int128)1 << (sh - 1);
    if (rem > half || (rem == half && (top & 1ull))) ++top;
    if (top == (1ull << 53)) {
      top >>= 1;
      ++sh;
    }
  }
  // 2^(sh - 64) as a double: sh - 64 lies in [-64, 11], a normal exponent
  const double scale = __longlong_as_double((long long)(1023 + sh - 64) << 52);
  const double d = __dmul_rn(__ull2double_rn(top), scale);
  return neg ? -d : d;
}

__global__ void k64_init(NetView v, double2 *vu64, Q128 *acc) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < v.n; i += (int64_t)gridDim.x * blockDim.x) {
    const double v0 = (double)v.vu[i].x;
    vu64[i] = make_double2(v0, __dmul_rn((double)v.abcd[i].y, v0));
    acc[i] = Q128{0ull, 0ull};
  }
}

// One FP64 step of every neuron (stateupdate, gpu4snn.cu:356-405, in double); the spiking
// neurons go to `list` in any order (the currents are exact sums).
__global__ void k64_step(NetView v, int64_t t, double2 *vu64, Q128 *acc, unsigned char *flag, int *list, int *count) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < v.n; i += (int64_t)gridDim.x * blockDim.x) {
    const float z = normal(v.seed, (uint64_t)i, (uint64_t)t);
    const double g = (double)(i < v.nexc ? v.ge : v.gi);
    const Q128 q = acc[i];
    acc[i] = Q128{0ull, 0ull};
    const double I = __dadd_rn(__dmul_rn(g, (double)z), q128_to_double(q));
    double vv = vu64[i].x, uu = vu64[i].y;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      double t1 = __dmul_rn(__dmul_rn(0.04, vv), vv);
      t1 = __dadd_rn(t1, __dmul_rn(5.0, vv));
      t1 = __dadd_rn(t1, 140.0);
      t1 = __dsub_rn(t1, uu);
      t1 = __dadd_rn(t1, I);
      vv = __dadd_rn(vv, __dmul_rn(0.5, t1));
    }
    const float4 p = v.abcd[i];
    uu = __dadd_rn(uu, __dmul_rn((double)p.x, __dsub_rn(__dmul_rn((double)p.y, vv), uu)));
    const bool spk = (vv >= 30.0) || !isfinite(vv);
    if (spk) {
      vv = (double)p.z;
      uu = __dadd_rn(uu, (double)p.w);
      list[atomicAdd(count, 1)] = (int)i;
    }
    flag[i] = spk ? 1 : 0;
    vu64[i] = make_double2(vv, uu);
  }
}

// Every synapse of every spiking row into the Q64.64 currents; a warp per row.
__global__ void k64_deliver(NetView v, const int *list, const int *count, Q128 *acc, int *bad) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int k = *count;
  for (int64_t s = warp; s < k; s += nwarps) {
    const int64_t row = list[s];
    const int *ri = v.idx + row * v.stride;
    const float *rw = v.w + row * v.stride;
    for (int j = lane; j < v.stride; j += 32) {
      const int tg = ri[j];
      if (tg >= 0) q128_add(acc + tg, wq64(rw[j], bad));
    }
  }
}

// |v32 - v64| per neuron, and the neurons whose spike at step t differs between the two.
__global__ void k64_compare(NetView v, int64_t t, const double2 *vu64, const unsigned char *flag, double *dv,
                            int *mismatch) {
  int mine = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < v.n; i += (int64_t)gridDim.x * blockDim.x) {
    dv[i] = fabs(__dsub_rn((double)v.vu[i].x, vu64[i].x));
    const bool s32 = v.sstat[i].last == (int)t;
    mine += (s32 != (flag[i] != 0)) ? 1 : 0;
  }
  if (mine) atomicAdd(mismatch, mine);
}

struct DevBuf {
  void *p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
};

}  // namespace

extern "C" int g4s_net_fp64_check(g4s_net *net, int32_t steps, double *dv_max, double *dv_p99, double *dv_median,
                                  int32_t *first_divergent, double *v64_out, double *u64_out) {
  if (!net) return set_error(G4S_ERR_INVALID, "null network");
  if (steps < 0) return set_error(G4S_ERR_INVALID, "g4s_net_fp64_check: negative step count");
  if (net_steps_done(net) != 0)
    return set_error(G4S_ERR_STATE, "g4s_net_fp64_check: the network must be at step 0 (after create or reset)");
  const NetView &v0 = net_view(net);
  const int64_t n = v0.n;
  cudaStream_t s = net_stream(net);
  DevBuf b_vu, b_acc, b_flag, b_list, b_cnt, b_dv;
  cudaError_t e = cudaMalloc(&b_vu.p, (size_t)n * sizeof(double2));
  if (e == cudaSuccess) e = cudaMalloc(&b_acc.p, (size_t)n * sizeof(Q128));
  if (e == cudaSuccess) e = cudaMalloc(&b_flag.p, (size_t)n);
  if (e == cudaSuccess) e = cudaMalloc(&b_list.p, (size_t)n * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&b_cnt.p, 4 * sizeof(int));  // spikes, mismatches, bad weight
  if (e == cudaSuccess) e = cudaMalloc(&b_dv.p, (size_t)n * sizeof(double));
  if (e != cudaSuccess) return cuda_error(e, "g4s_net_fp64_check: allocation");
  double2 *vu64 = static_cast<double2 *>(b_vu.p);
  Q128 *acc = static_cast<Q128 *>(b_acc.p);
  unsigned char *flag = static_cast<unsigned char *>(b_flag.p);
  int *list = static_cast<int *>(b_list.p), *cnt = static_cast<int *>(b_cnt.p);
  double *dv = static_cast<double *>(b_dv.p);
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)sms * 8));
  if ((e = cudaMemsetAsync(cnt, 0, 4 * sizeof(int), s)) != cudaSuccess) return cuda_error(e, "g4s_net_fp64_check: memset");
  k64_init<<<grid, 256, 0, s>>>(v0, vu64, acc);
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_error(e, "g4s_net_fp64_check: init");
  std::vector<double> h_dv((size_t)n);
  int first = -1;
  for (int32_t t = 0; t < steps; ++t) {
    int rc = g4s_net_run(net, 1, G4S_ALG_SKL);
    if (rc) return rc;
    const NetView &v = net_view(net);
    e = cudaMemsetAsync(cnt, 0, 2 * sizeof(int), s);  // spikes and mismatches of this step
    if (e != cudaSuccess) return cuda_error(e, "g4s_net_fp64_check: memset");
    k64_step<<<grid, 256, 0, s>>>(v, t, vu64, acc, flag, list, cnt);
    k64_deliver<<<(unsigned)sms * 8, 256, 0, s>>>(v, list, cnt, acc, cnt + 2);
    k64_compare<<<grid, 256, 0, s>>>(v, t, vu64, flag, dv, cnt + 1);
    int words[3] = {0, 0, 0};
    if ((e = cudaGetLastError()) == cudaSuccess)
      e = cudaMemcpyAsync(h_dv.data(), dv, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(words, cnt, sizeof words, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_error(e, "g4s_net_fp64_check: step");
    if (words[2]) return set_error(G4S_ERR_INVALID, "g4s_net_fp64_check: a weight of magnitude >= 2^40 or not finite");
    if (words[1] && first < 0) first = t;
    // nearest-rank percentiles: the ceil(p n)-th smallest value
    const size_t r99 = (size_t)std::ceil(0.99 * (double)n) - 1, r50 = (size_t)std::ceil(0.5 * (double)n) - 1;
    double mx = 0.0;
    for (double x : h_dv) mx = std::max(mx, x);
    std::nth_element(h_dv.begin(), h_dv.begin() + (ptrdiff_t)r99, h_dv.end());
    const double p99 = h_dv[r99];
    std::nth_element(h_dv.begin(), h_dv.begin() + (ptrdiff_t)r50, h_dv.begin() + (ptrdiff_t)r99);
    const double p50 = h_dv[r50];
    if (dv_max) dv_max[t] = mx;
    if (dv_p99) dv_p99[t] = p99;
    if (dv_median) dv_median[t] = p50;
  }
  if (first_divergent) *first_divergent = first;
  if (v64_out || u64_out) {
    std::vector<double2> h((size_t)n);
    e = cudaMemcpyAsync(h.data(), vu64, (size_t)n * sizeof(double2), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_error(e, "g4s_net_fp64_check: state");
    for (int64_t i = 0; i < n; ++i) {
      if (v64_out) v64_out[i] = h[(size_t)i].x;
      if (u64_out) u64_out[i] = h[(size_t)i].y;
    }
  }
  return G4S_OK;
}
