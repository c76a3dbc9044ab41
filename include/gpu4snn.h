/*
 * gpu4snn.h — C ABI of the GB300 simulation library (libgpu4snn.so).
 *
 * The reference has no library interface: its boundary is the command line
 * `./gpu4snn N Nsyn iterations` (gpu4snn.cu:735-739, spawned by gpu4snn.py:42) plus the
 * result files it writes (gpu4snn.cu:1109-1140, 1256-1267, 1311-1327).  This ABI is what a
 * ctypes driver (or any FFI) binds in its place.  Each entry point names the reference
 * code it replaces.
 *
 * Conventions: every function returns an int status (G4S_OK = 0, negative G4S_ERR_* on
 * failure) unless stated otherwise; the message of the last failure on the calling
 * thread is g4s_last_error().  The library owns all device memory of a handle; the
 * caller owns every host buffer it passes in.  A handle is used by one thread at a time;
 * distinct handles may be used from distinct threads.  No C++ exception crosses the ABI.
 */
#ifndef GPU4SNN_H
#define GPU4SNN_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define G4S_ABI_VERSION 1

#define G4S_OK 0
#define G4S_ERR_INVALID (-1)   /* bad argument or descriptor                         */
#define G4S_ERR_CUDA (-2)      /* a CUDA runtime call failed                          */
#define G4S_ERR_NOMEM (-3)     /* device or host allocation failed                    */
#define G4S_ERR_TIMEOUT (-4)   /* a grid barrier of a persistent kernel timed out      */
#define G4S_ERR_OVERFLOW (-5)  /* raster buffer overflow                              */
#define G4S_ERR_IO (-6)        /* a result file could not be written                  */
#define G4S_ERR_BUDGET (-7)    /* request does not fit the memory budget               */
#define G4S_ERR_CANCELLED (-8) /* request cancelled                                    */
#define G4S_ERR_STATE (-9)     /* call not valid in the handle's current state        */

/* Propagation schemes; values are the reference's `dynamic` (gpu4snn.cu:1083). */
#define G4S_ALG_AP 0   /* nested fan-out: a thread group per spiking row   (gpu4snn.cu:323-331, 409) */
#define G4S_ALG_N 1    /* thread per spiking neuron                          (gpu4snn.cu:420-443)      */
#define G4S_ALG_S 2    /* thread per synapse vector, oversubscribed grid     (gpu4snn.cu:446-467)      */
#define G4S_ALG_AB 3   /* persistent grid over the synapse range             (gpu4snn.cu:554-584)      */
#define G4S_ALG_SKL 4  /* whole step loop in one cooperative kernel          (gpu4snn.cu:669-716)      */
#define G4S_ALG_AUTO 5 /* autotuner's pick                                                            */

/* Connectivity laws. */
#define G4S_CONN_PHILOX 0 /* GPU generator, counter-based Philox stream (default)              */
#define G4S_CONN_GLIBC 1  /* the reference's host generator: srand(seed), rand() (gpu4snn.cu:873-898) */

/* Network description (replaces argv N/Nsyn, gpu4snn.cu:738-744, and the hard-coded
 * 80/20 split, drive gains and self-loop behaviour). */
typedef struct g4s_net_desc {
  int64_t n;                   /* neurons                                                   */
  int32_t nsyn;                /* synapses per neuron (distinct targets)                    */
  int32_t exc_permille;        /* excitatory share x1000; 800 = floor(4N/5) as the reference  */
  int32_t self_loops;          /* 1: a neuron may target itself (the reference's tables)      */
  int32_t conn_law;            /* G4S_CONN_*                                                */
  uint64_t seed;               /* network seed (tables, parameters, drive)                  */
  float drive_scale;           /* thalamic gains (5, 2) x scale; modes 0/1/2 = 0.5/1.0/1.5  */
  int32_t record_raster;       /* 1: keep the spike raster on the host                      */
  int64_t raster_budget_bytes; /* device raster buffer per chunk (0 = default 1 GiB)        */
} g4s_net_desc;

typedef struct g4s_net g4s_net;

/* Run-time information of a handle. */
typedef struct g4s_net_info {
  int64_t n;
  int32_t nsyn;
  int32_t stride;            /* row stride of the tables (multiple of 4)                */
  int64_t steps_done;        /* absolute step counter                                   */
  int64_t total_spikes;      /* since creation or the last reset                         */
  int64_t raster_size;       /* (step, id) pairs held on the host                       */
  double last_run_ms;        /* device time of the last g4s_net_run (CUDA events)       */
  double last_run_wall_ms;   /* host wall time of the last g4s_net_run                  */
  int64_t last_run_spikes;   /* spikes of the last run                                   */
  int32_t last_algorithm;    /* scheme the last run used (AUTO resolved)                */
  int32_t persistent_blocks; /* grid of the SKL kernel                                  */
  int64_t device_bytes;      /* device memory held by the handle                        */
  double last_run_kernel_ms; /* CUDA-event time of the step kernels alone, last run     */
  int64_t last_run_launches; /* kernel launches of the last run                         */
} g4s_net_info;

int g4s_abi_version(void);
const char *g4s_last_error(void);
/* CUDA device of the calling thread for subsequent handles (the reference picks it with
 * findCudaDevice, gpu4snn.cu:818). */
int g4s_set_device(int32_t device);

/* Allocation + initNeuron + connectivity (gpu4snn.cu:750-911, 1094). */
int g4s_net_create(const g4s_net_desc *desc, g4s_net **out);
/* Same with caller-supplied host tables [n][stride] (the reference's H2D copy of its host
 * tables, gpu4snn.cu:910-911); padding slots carry target -1. */
int g4s_net_create_from_tables(const g4s_net_desc *desc, const int32_t *idx, const float *w, int32_t stride,
                               g4s_net **out);
/* Replace the tables of an existing handle from host memory (H2D). */
int g4s_net_load_tables(g4s_net *net, const int32_t *idx, const float *w, int32_t stride);
/* Neuron state, currents, statistics and raster back to step 0 (initNeuron, gpu4snn.cu:1094). */
int g4s_net_reset(g4s_net *net);
/* Advance `steps` steps with one scheme (the step loop, gpu4snn.cu:1215-1300). */
int g4s_net_run(g4s_net *net, int32_t steps, int32_t algorithm);
int g4s_net_get_info(g4s_net *net, g4s_net_info *info);
/* Spike raster (the reference's spiketimes.csv rows, gpu4snn.cu:1256-1261), ordered by
 * (step, neuron id).  Writes min(cap, size) pairs; *n receives the size. */
int g4s_net_raster(g4s_net *net, int32_t *t, int32_t *id, int64_t cap, int64_t *n);
/* Spikes per step since the last reset (computetime.csv SpksPerStep, gpu4snn.cu:1267). */
int g4s_net_counts(g4s_net *net, int32_t *counts, int64_t cap, int64_t *n);
/* Per-step device times in ms: update phase and whole step (computetime.csv columns). */
int g4s_net_step_times(g4s_net *net, float *update_ms, float *step_ms, int64_t cap, int64_t *n);
/* Neuron record (gpu4snn.cu:50-62, writeNeuronInfo :727-729); any pointer may be NULL. */
int g4s_net_state(g4s_net *net, float *v, float *u, float *i_last, float *a, float *b, float *c, float *d,
                  int32_t *nospks);
/* Raw Q32.32 synaptic currents pending for the next step. */
int g4s_net_currents(g4s_net *net, int64_t *acc);
/* Rows [row0, row0+nrows) of the tables, [nrows][stride]. */
int g4s_net_tables(g4s_net *net, int64_t row0, int64_t nrows, int32_t *idx, float *w);
/* FP64 statistics: mean rate (Hz, 1 ms steps) and mean per-neuron ISI CV. */
int g4s_net_stats(g4s_net *net, double *rate_hz, double *isi_cv, int64_t *total_spikes);
/* On-device FP64 check of the network's FP32 trajectory (no counterpart in the reference,
 * whose update, gpu4snn.cu:376-405, runs in FP32 only): from step 0 (after create or
 * reset; G4S_ERR_STATE otherwise) runs `steps` steps of the network (SKL scheme) in
 * lockstep with an FP64 twin on the GPU: the same random draws, v and u in double, the
 * synaptic currents as exact Q64.64 sums (the CPU oracle's FP64 mode, bit for bit).  Per
 * step t: dv_max[t], dv_p99[t], dv_median[t] = max, 99th and 50th nearest-rank percentile
 * of |v32 - v64| (mV) over all neurons; *first_divergent = first step whose spike sets
 * differ (-1: none); v64_out, u64_out [n] = the twin's final state.  Any output may be
 * NULL.  The network advances by `steps` steps.  Allocates ~41 bytes per neuron. */
int g4s_net_fp64_check(g4s_net *net, int32_t steps, double *dv_max, double *dv_p99, double *dv_median,
                       int32_t *first_divergent, double *v64_out, double *u64_out);
/* Grid-barrier time limit of the SKL kernel in ns (default 2 s); 0 makes every barrier
 * give up at once (used to test the timeout path). */
int g4s_net_set_barrier_timeout(g4s_net *net, uint64_t ns);
/* Geometry of the SKL kernel (the reference sizes its persistent grids from occupancy,
 * gpu4snn.cu:1066-1076): `owner_blocks` CTAs, each owning a contiguous slice of target
 * neurons whose currents stay in its shared memory (0 = automatic), and the delivery
 * mapping of a multi-CTA team (-1, the default: automatic, eight-lane groups when a rank's
 * segment of a row averages 24 synapses or more, else segment runs; 0: warps walk the
 * concatenated segments of 32 spikes; 1: eight lanes walk each spike's segment).
 * get_geometry reports the geometry in use (zeros when the network is too large for
 * shared-memory ownership, or its tables exceed the exact-accumulation bound, and the
 * global-atomic persistent kernel runs instead) and the neurons per CTA; get_delivery the
 * mapping in use (0 or 1; -1 without a multi-CTA team).  Results do not depend on either. */
int g4s_net_set_geometry(g4s_net *net, int32_t owner_blocks, int32_t delivery);
/* Threads per CTA of the SKL team kernel: 1024 (the most table reads in flight, for steps
 * with many synapses per CTA), 768 (80 registers a thread instead of 64, no spills: faster
 * for steps whose work is small) or 0 (the default: 768 when a CTA's expected share of a
 * step, from the recent firing rate, is under 32768 synapses, else 1024; 1024 in a batch).
 * Results do not depend on it; the autotuner tries both sizes.  A no-alloc run and a batch
 * of networks that disagree use 1024.  get_block_threads reports the size in use. */
int g4s_net_set_block_threads(g4s_net *net, int32_t threads);
int g4s_net_get_block_threads(g4s_net *net, int32_t *threads);
int g4s_net_get_geometry(g4s_net *net, int32_t *owner_blocks, int64_t *slice);
int g4s_net_get_delivery(g4s_net *net, int32_t *delivery);

/* Autotuner (replaces the reference's occupancy-based launch configurator,
 * gpu4snn.cu:780-838, 959-1079): times the candidate schemes (SKL with teams of 1, 2, 4, ...
 * CTAs at both CTA sizes, by segment runs and, where a team's segments average 12 synapses or
 * more, by eight-lane groups; AB, AP) on `probe_steps` steps of this network from a device
 * snapshot of its state,
 * restores the state (the simulation is unchanged), and keeps the fastest for ALG_AUTO on
 * this handle and, process-wide, for networks of the same size, fan-out and firing rate
 * (log2 buckets).  Outputs (any may be NULL): the scheme, its team size, us per step. */
int g4s_net_autotune(g4s_net *net, int32_t probe_steps, int32_t *algorithm, int32_t *team, double *us_per_step);

/* Batched execution (the reference runs one network per launch sequence; this has no
 * counterpart there beyond SKL_deliverspks, gpu4snn.cu:669-716): `count` independent
 * handles, network i advancing steps[i] further steps, all in shared persistent launches
 * of the SKL team kernel (a network that fits one CTA's shared memory runs on one CTA).
 * Results land in each handle as after g4s_net_run.  *device_ms receives the CUDA-event
 * time of the launches, *launches their number (either pointer may be NULL). */
int g4s_nets_run(g4s_net **nets, const int32_t *steps, int32_t count, double *device_ms, int64_t *launches);
int g4s_net_destroy(g4s_net *net);

/* Host-side fault injection for failure-detection tests (nothing faults the GPU):
 *   G4S_FAULT_BARRIER_STALL  the next SKL launch of `net` waits at its first barrier for
 *                            one block more than it has, so the wait runs out after the
 *                            barrier time limit and the run returns G4S_ERR_TIMEOUT;
 *   G4S_FAULT_ALLOC          the next device allocation of g4s_net_create fails
 *                            (process-wide; `net` may be NULL). */
#define G4S_FAULT_BARRIER_STALL 1
#define G4S_FAULT_ALLOC 2
int g4s_inject_fault(g4s_net *net, int32_t kind);

/* Reference result files for one run in `dir` (gpu4snn.cu:1109-1140, 1256-1267,
 * 1311-1327): neuroninfo.csv (initial record), spiketimes.csv, computetime.csv,
 * sim_overview.csv, neuroninfoafter.csv (the actual final record). */
int g4s_net_write_results(g4s_net *net, const char *dir, const float *init_state /* [9][n] or NULL */,
                          double elapsed_ms, double elapsed_with_data_ms);

/* Binary files (the reference writes its raster as text rows from a per-step host scan,
 * gpu4snn.cu:1256-1261, and regenerates its tables for every run, gpu4snn.cu:862-911).
 * Raster file "G4SRAS01" (little-endian): char[8] magic; int64 n; int64 first step;
 * int64 steps; int64 spikes; then chunks to the end of the file: int32 cs; int32
 * counts[cs]; int32 ids[sum counts], ascending within each step.
 * g4s_net_stream_raster(net, path) writes the raster of the following runs to `path`, one
 * chunk per device chunk, from a writer thread while the GPU computes the next chunk; the
 * raster is then not kept in host memory.  path = NULL (or a reset, or destroy) ends the
 * stream and completes the header.  Needs record_raster; G4S_ERR_IO if a write fails.
 * g4s_net_write_raster_file writes the host raster of every step since the reset. */
int g4s_net_stream_raster(g4s_net *net, const char *path);
int g4s_net_write_raster_file(g4s_net *net, const char *path);
/* Tables checkpoint "G4STAB01": char[8] magic; int64 n; int32 nsyn; int32 stride; uint64
 * seed; int32 conn_law; int32 self_loops; int32 exc_permille; int32 flags (1 = rows sorted
 * by target); int32 reserved[2]; int32 idx[n][stride]; float w[n][stride].
 * g4s_net_create_from_file builds a network from such a file (desc->n and desc->nsyn must
 * match it; desc->seed still seeds the neuron parameters and the drive). */
int g4s_net_save_tables(g4s_net *net, const char *path);
int g4s_net_create_from_file(const g4s_net_desc *desc, const char *path, g4s_net **out);

/* The reference's whole experiment (main, gpu4snn.cu:735-1332): for each drive mode
 * (0..2, or `mode`) and scheme (0..4, or `algorithm`), run `iterations` steps of the same
 * network and write Results/N{n}Nsyn{nsyn}Regime{mode}Alg{alg}/ under results_root. */
int g4s_run_protocol(int32_t n, int32_t nsyn, int32_t iterations, int32_t algorithm, int32_t mode, uint64_t seed,
                     int32_t conn_law, const char *results_root);

/* Serving with continuous batching (no counterpart in the reference, which runs one
 * experiment per process, gpu4snn.py:42).  A server admits submitted simulations while
 * their estimated device bytes fit `hbm_budget_bytes`, keeps them resident, and advances
 * all resident ones together in one persistent launch of the SKL team kernel per round:
 * `quantum_steps` steps in a request's first round, then as many as the median resident
 * request runs in `quantum_steps` steps, from the measured per-step times (at most
 * `quantum_steps` for a request that records its raster); requests arriving meanwhile
 * join at the next round.  The requests' device memory comes from a pool of the server's
 * that keeps what finished requests free for the next ones: the server holds its peak
 * device memory until it stops.  submit/poll/result/release/get_stats are thread-safe. */
typedef struct g4s_request {
  int64_t n;           /* neurons                                   */
  int32_t nsyn;        /* synapses per neuron                       */
  int32_t steps;       /* steps to simulate                         */
  uint64_t seed;       /* network seed                              */
  float drive_scale;   /* thalamic gains (5, 2) x scale             */
  int32_t record_raster;
} g4s_request;

typedef struct g4s_request_result {
  int64_t id;
  int32_t status;       /* 0 or G4S_ERR_*                            */
  int32_t steps_done;
  int64_t total_spikes;
  double latency_ms;    /* submit -> results on the host             */
  double queue_ms;      /* submit -> resident on the device          */
  double rate_hz;       /* FP64 statistics of the run                */
  double isi_cv;
  double create_ms;     /* network creation at admission (host wall) */
  double device_ms;     /* device time of its steps in the rounds     */
  double sm_ms;         /* the same times the CTAs of its team        */
  int32_t rounds;       /* rounds it took part in                     */
  int32_t team;         /* CTAs of its team in its last round         */
} g4s_request_result;

typedef struct g4s_server_stats {
  int64_t rounds, launches, completed, queued, resident, events;
  double busy_ms;       /* CUDA-event time of the rounds' launches   */
  double wall_ms;       /* since start                               */
  int64_t bytes_in_use, peak_bytes;
} g4s_server_stats;

typedef struct g4s_server g4s_server;
int g4s_server_start(int64_t hbm_budget_bytes, int32_t quantum_steps, g4s_server **out);
/* G4S_ERR_BUDGET if the request alone exceeds the budget; G4S_ERR_INVALID if malformed. */
int g4s_server_submit(g4s_server *s, const g4s_request *req, int64_t *id);
/* Results completed since the last poll (up to cap). */
int g4s_server_poll(g4s_server *s, g4s_request_result *out, int32_t cap, int32_t *n);
/* Raster ((step, id) order) and final v, u, spike counts of a completed request. */
int g4s_server_result(g4s_server *s, int64_t id, int32_t *t, int32_t *ids, int64_t cap, int64_t *n, float *v,
                      float *u, int32_t *nospks);
int g4s_server_release(g4s_server *s, int64_t id);
int g4s_server_get_stats(g4s_server *s, g4s_server_stats *out);
/* drain = 1: wait for every submitted request first; 0: finish the resident ones, drop
 * the queued ones. */
int g4s_server_stop(g4s_server *s, int32_t drain);

/* Device arrays of one network, owned by the caller (layouts as the library's own). */
typedef struct g4s_dev_net {
  int64_t n;          /* neurons                                                        */
  int64_t nexc;       /* excitatory neurons: ids [0, nexc)                                */
  int32_t nsyn;       /* synapses per neuron                                              */
  int32_t stride;     /* row stride of the tables: a multiple of 4, nsyn <= stride <= 16384 */
  uint64_t seed;      /* seed of the thalamic drive                                       */
  float ge, gi;       /* thalamic gains of excitatory / inhibitory neurons                 */
  void *vu;           /* float2[n]: v, u                                                   */
  void *abcd;         /* float4[n]: a, b, c, d                                             */
  int64_t *acc;       /* int64[n]: pending Q32.32 synaptic currents                        */
  float *i_last;      /* float[n]: input current of the last step of a run                 */
  void *spike_stat;   /* 32-byte records [n]: int32 nospks, last (-1 before the first
                         spike), nisi, pad; int64 sum of intervals, sum of squares          */
  const int32_t *idx; /* [n][stride] targets, every row ascending, unused slots (-1) last
                         (as g4s_net_tables returns them)                                   */
  const float *w;     /* [n][stride] weights                                                */
} g4s_dev_net;

/* The SKL team kernel on caller-owned device arrays, allocating nothing.  No counterpart
 * in the reference.  For callers that cannot allocate device memory while they step a
 * network: real-time loops that cannot take the device-wide synchronisation an allocation
 * or a free may imply, and hosts whose device memory is a capped pool this library cannot
 * draw from.  Nothing is copied from host memory either.  Advances `steps` steps from absolute
 * step t_abs0 with a team of `team` CTAs (1..8); outputs, all device memory of the caller:
 * d_counts int32[steps] spikes per step, d_base int64[steps] raster offset of each step,
 * d_raster int32[raster_cap] spike ids (ids that do not fit are not recorded), d_status
 * (may be NULL) 0 or a device error code; `last` = 1 records i_last at the last step.
 * Stream-ordered on `stream` (NULL: the default stream).  The kernel's scratch is one
 * fixed __device__ array of about 6.5 MB (held by every GPU that loads the library): at
 * most 131072 neurons and 16384 neurons per CTA; larger requests are rejected with
 * G4S_ERR_INVALID.  The first call on a device looks the array's address up (once per
 * device, with that device current) and sets the team kernel's shared-memory ceiling.  A
 * multi-CTA call rebuilds the per-row segment table of its tables every time.  All calls
 * share the array: calls that overlap on the GPU race and must not be made. */
int g4s_run_noalloc(const g4s_dev_net *net, int64_t t_abs0, int32_t steps, int32_t team, int32_t last,
                    int32_t *d_counts, int64_t *d_base, int32_t *d_raster, int64_t raster_cap, int32_t *d_status,
                    void *stream);

/* Page-locked host buffers for fast table uploads and raster downloads (the reference
 * copies from pageable malloc memory, gpu4snn.cu:863-866, 910-911). */
int g4s_pinned_alloc(uint64_t bytes, void **out);
int g4s_pinned_free(void *p);

/* The reference's host table generator with glibc rand() after srand(seed)
 * (gpu4snn.cu:873-898), into [n][stride] host buffers (padding: -1 / 0). */
int g4s_conn_glibc(uint32_t seed, int32_t n, int32_t nsyn, int32_t stride, int32_t *idx, float *w);

#ifdef __cplusplus
}
#endif
#endif
