// g4s_types.h — types shared by the host library and the kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace g4s {

// Philox key word 1 per random stream (key word 0 is the network seed).
constexpr uint64_t kStreamConn = 1;    // target draws:   counter (row, draw block, 0)
constexpr uint64_t kStreamWeight = 2;  // weights:        counter (row, slot / 4, 0)
constexpr uint64_t kStreamParam = 3;   // parameter r:    counter (neuron, 0, 0)
constexpr uint64_t kStreamNoise = 4;   // thalamic drive: counter (neuron, step, attempt)

// Device-side error codes (the host maps them to G4S_ERR_*).
constexpr int kErrTimeoutCode = 1;   // a grid barrier waited longer than its limit
constexpr int kErrOverflowCode = 2;  // a spike did not fit the raster buffer
constexpr int kErrConnCode = 3;      // connectivity generation ran out of draws

// Grid barrier state: a monotone arrival counter and an error word (one 128 B line).
struct alignas(128) GridSync {
  unsigned count;
  int error;
  unsigned pad[30];
};

// Per-neuron spike statistics, touched only when the neuron fires (32 B, one sector).
struct alignas(32) SpikeStat {
  int nospks;     // spikes so far (the reference's Neuron::nospks)
  int last;       // step of the last spike, -1 before the first
  int nisi;       // inter-spike intervals seen
  int pad;
  long long s1;   // sum of intervals (steps)
  long long s2;   // sum of squared intervals
};

// Everything a kernel needs to step one network (passed by value).
struct NetView {
  int64_t n;        // neurons
  int64_t nexc;     // excitatory neurons: ids [0, nexc)
  int32_t nsyn;     // synapses per neuron
  int32_t stride;   // row stride of the tables, a multiple of 4 (padding: target -1)
  uint64_t seed;
  float ge, gi;     // thalamic gains (5, 2) x drive scale
  float2 *vu;       // membrane potential v, recovery u
  float4 *abcd;     // a, b, c, d
  float *rpar;      // the uniform r each neuron's a, b, c, d derive from (may be null)
  long long *acc;   // Q32.32 synaptic current, consumed and cleared by the update
  float *ilast;     // total input current of the last step of a run
  SpikeStat *sstat;
  const int *idx;   // [n][stride] targets
  const float *w;   // [n][stride] weights
  const int2 *pair;  // [n][stride] the same rows interleaved (target, weight bits): one
                     // contiguous run per segment for the team kernel (may be null)
  int *raster;      // spike ids of the current chunk, step after step
  int64_t raster_cap;
  int *counts;      // spikes per step of the current chunk
  long long *base;  // raster offset of each step of the current chunk
  unsigned long long *stamps;  // globaltimer per step: [2*lt] step start, [2*lt+1] update end
  int *status;      // device error word (kErr*Code)
};

// One network of a team-kernel launch: its arrays, the steps of this launch, and its
// team (CTAs `team`, each owning `rc` neurons).
struct TeamItem {
  NetView v;
  const uint16_t *seg;  // [n][team+1] row segment offsets (team > 1)
  unsigned long long *list;  // [4][n] tagged spike ids, by step parity: [par] beyond a rank's record
                             // lines (at its neuron offset), [2 + par] the step's dense list
  unsigned long long *rec;   // [2][team][2 x 16] tagged spike records, by step parity (zero at launch)
  int64_t t_abs0;       // absolute step of the first step of this launch
  int steps;            // steps of this launch (0: nothing to do)
  int last;             // this launch ends the run: record the input current at its last step
  int team;             // CTAs of the team
  int rc;               // neurons per CTA slice
  GridSync *sync;       // error word of the team
  int mode;             // delivery mapping of a multi-CTA team (kDeliverRun or kDeliverGroup)
  int cap;              // delivery window of a multi-CTA rank (spike ids in shared memory)
  unsigned tag0;        // record tag of step lt: tag0 + lt + 1 (never repeats for the list's words)
};

// Delivery mappings of a multi-CTA team: warps walk the concatenated segments of 32
// spikes, each synapse finding its spike by a search over the batch (kDeliverRun, for
// short segments), or groups of eight lanes walk one spike's segment each (kDeliverGroup,
// for long segments: no search); kDeliverAuto picks by the mean segment length.
constexpr int kDeliverAuto = -1;
constexpr int kDeliverRun = 0;
constexpr int kDeliverGroup = 1;
// mean synapses of a rank's segment of a row (Nsyn / team) from which kDeliverAuto takes the
// eight-lane groups (measured in the team kernel: even with the runs at ~26 synapses, 14%
// faster per step at ~66)
constexpr int kGroupMinSegment = 24;

}  // namespace g4s
