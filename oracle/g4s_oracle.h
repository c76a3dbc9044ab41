/*
 * g4s_oracle.h — CPU oracle for the GPU4SNN simulation step (test infrastructure only).
 *
 * This library is the checker, never the product: only tests, the smoke check and the
 * CPU-baseline leg of bench.py load it.  It restates, in plain C, the reference's
 * algorithm for one pulse-coupled Izhikevich network:
 *   - neuron parameters             gpu4snn.cu:286-320  (initNeuron)
 *   - the two-half-step update       gpu4snn.cu:356-414  (stateupdate)
 *   - thalamic drive gains           gpu4snn.cu:362-382
 *   - spike delivery                 gpu4snn.cu:323-331, 420-467, 554-584, 669-716
 *   - connectivity law and weights   gpu4snn.cu:862-899
 *   - N_exc = floor(4N/5)            gpu4snn.cu:744
 * The reference draws its randomness from cuRAND XORWOW (seeded with time(NULL)) and
 * glibc rand(); the library replaces both with a counter-based Philox4x64-10 stream
 * (Salmon et al., SC'11) whose layout is defined below, so that CPU and GPU produce
 * identical bits.  Currents are accumulated as Q32.32 fixed point, which makes the
 * result independent of the order of the additions.
 *
 * Two arithmetic modes:
 *   G4O_FP32  — the FP32 mirror: every float operation in the same order and rounding
 *               as the CUDA kernels; rasters, states and currents are bit-exact.
 *   G4O_FP64  — the same random draws promoted to double, dynamics in double; the
 *               synaptic currents are exact Q64.64 sums of the weights, converted to
 *               double (correctly rounded) when consumed, so they do not depend on the
 *               order of the additions; used to bound the FP32 error of the membrane
 *               potential, and the CPU twin of the library's on-device FP64 check.
 *
 * Pinning: Philox4x64-10 against numpy.random.Philox; the reference-compatible table
 * generator (glibc rand) against tables dumped by the reference's own host code.
 */
#ifndef G4S_ORACLE_H
#define G4S_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Philox stream identifiers: key = (seed, stream). */
#define G4O_STREAM_CONN 1u   /* connectivity target draws,  ctr = (row, draw block, 0, 0) */
#define G4O_STREAM_WEIGHT 2u /* connectivity weights,      ctr = (row, slot/4, 0, 0)     */
#define G4O_STREAM_PARAM 3u  /* neuron parameter r,        ctr = (neuron, 0, 0, 0)       */
#define G4O_STREAM_NOISE 4u  /* thalamic noise, Philox4x32: ctr = (neuron, step, attempt, 4) */

#define G4O_FP32 0
#define G4O_FP64 1

typedef struct g4o_desc {
  int64_t n;            /* neurons                                          */
  int32_t nsyn;         /* synapses per neuron (distinct targets)           */
  int32_t stride;       /* row stride of the tables, >= nsyn                 */
  int32_t exc_permille; /* excitatory share in 1/1000 (800 = the reference) */
  int32_t self_loops;   /* 1: a neuron may target itself (the reference)    */
  uint64_t seed;        /* master seed of the network                       */
  float drive_scale;    /* ge = 5*scale, gi = 2*scale (1.0 = balanced mode) */
  int32_t pad_;
} g4o_desc;

/* ---- random numbers ---------------------------------------------------------- */
void g4o_philox4x64_10(const uint64_t ctr[4], const uint64_t key[2], uint64_t out[4]);
void g4o_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
float g4o_logf(float x);
float g4o_normal(uint64_t seed, uint64_t neuron, uint64_t step);
float g4o_param_r(uint64_t seed, uint64_t neuron);
/* draw k of row `row` (before the distinctness test), in [0, n) */
int64_t g4o_conn_draw(uint64_t seed, int64_t n, int self_loops, int64_t row, int64_t k);

/* ---- connectivity ------------------------------------------------------------- */
/* Philox law: rows [row0, row0+nrows), written at idx/w + (row-row0)*stride.
 * Slots nsyn..stride-1 are padding (idx -1, w 0). Returns 0 or -1. */
int g4o_conn_philox(const g4o_desc *d, int64_t row0, int64_t nrows, int32_t *idx, float *w);
/* Rows sorted in the library's order: by target as unsigned (padding -1 last), equal
 * targets by weight bits.  Returns 0 or -1. */
int g4o_sort_rows(int32_t *idx, float *w, int64_t nrows, int32_t stride);
/* The reference's own law with glibc rand() after srand(seed) (gpu4snn.cu:873-898). */
int g4o_conn_glibc(unsigned seed, int32_t n, int32_t nsyn, int32_t *idx, float *w);
/* Q32.32 value of one weight */
int64_t g4o_wfix(float w);

/* ---- simulation --------------------------------------------------------------- */
typedef struct g4o_sim g4o_sim;
g4o_sim *g4o_sim_create(const g4o_desc *d, const int32_t *idx, const float *w, int mode);
void g4o_sim_destroy(g4o_sim *s);
/* advance `steps` steps with `threads` OpenMP threads (1 = serial) */
int g4o_sim_run(g4o_sim *s, int32_t steps, int32_t threads);
int64_t g4o_sim_step_index(const g4o_sim *s);
int64_t g4o_sim_raster_size(const g4o_sim *s);
/* copy the raster (step, neuron) pairs in (step, id) order */
int64_t g4o_sim_raster(const g4o_sim *s, int32_t *t, int32_t *id, int64_t cap);
/* per-step spike counts for the steps run so far */
int64_t g4o_sim_counts(const g4o_sim *s, int32_t *counts, int64_t cap);
/* state: v, u, I as float (FP64 mode rounds), params, spike counts */
void g4o_sim_state(const g4o_sim *s, float *v, float *u, float *i_last, float *a, float *b,
                   float *c, float *dd, int32_t *nospks);
void g4o_sim_state64(const g4o_sim *s, double *v, double *u);
/* raw Q32.32 current accumulator (FP32 mode) */
void g4o_sim_acc(const g4o_sim *s, int64_t *acc);
/* FP64 statistics: mean rate (Hz) and mean per-neuron ISI CV (neurons with >= 2 ISIs) */
void g4o_sim_stats(const g4o_sim *s, double *rate_hz, double *isi_cv, int64_t *total_spikes);

#ifdef __cplusplus
}
#endif
#endif
