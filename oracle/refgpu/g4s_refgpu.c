/*
 * g4s_refgpu.c — drives the reference's own CUDA kernels on a GPU (baseline and test
 * infrastructure; never part of the product, and no product code links it).
 *
 * The kernels are the reference's, compiled unmodified from gpu4snn.cu into a linked
 * cubin by `make -C oracle refcubin` (device code only, with the device runtime linked in
 * for the AP scheme's device-side launches).  This program is this project's own host
 * code: it loads that cubin with the CUDA driver API and runs the kernels the way the
 * reference's main does (gpu4snn.cu:780-1300):
 *   randgeneratorinit (gpu4snn.cu:273-283) with a FIXED seed instead of time(NULL) (:841);
 *   initNeuron (:286-320);
 *   per step stateupdate (:334-417; the AP scheme launches propagatespikes :323-331 from
 *   the device) followed by deliverspks1 (N, :420-443), deliverspks2 (S, :446-467) or a
 *   cooperative AB_deliverspks (AB, :554-584); or one cooperative SKL_deliverspks for all
 *   steps (:669-716).
 * Block sizes come from the occupancy calculator as in the reference (:785, :826, :1009,
 * :1019, :1032, :1057, :1070); the persistent grids are SMs x blocks per SM (:1062, :1074).
 *
 * Guards, so that the reference's code stays in bounds on every input this program takes:
 *   - initNeuron reads state[id] before its bound check (:289-292): the cuRAND state array
 *     is sized to the launched grid (N rounded up to the block) and zeroed;
 *   - the S, AB and SKL kernels index synapses with `int` (:460, :569, :692): runs with
 *     N x Nsyn >= 2^31 are refused;
 *   - targets are checked to lie in [0, N) before the upload;
 *   - the device runtime's pending-launch limit is raised to at least N for the AP scheme,
 *     so that no step, whatever its spikes, can exceed it (the reference keeps the default
 *     of 2048 and silently drops the launches beyond it).
 *
 * Usage:
 *   g4s_refgpu --cubin F --n N --nsyn S --idx F --w F --steps T
 *              [--schemes 0,1,2,3,4] [--modes 0,1,2] [--seeds 1,2,...] [--raster PREFIX]
 *              [--reps R]
 * idx: int32 [N][S] row-major targets; w: float32 [N][S].  For every (scheme, mode, seed)
 * it prints one JSON line: spikes (sum of the neurons' nospks), device time of the step
 * loop (CUDA events; with --raster the per-step copy of the spike flags to the host is
 * inside it, as in the reference's elapsedwithdata), launch geometry.  With --raster the
 * per-step spike flags are copied back each step (host-driven schemes) and written as
 * int32 (step, neuron) pairs to PREFIX_s{scheme}_m{mode}_r{seed}.bin.
 */
#include <cuda.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define CK(call)                                                                      \
  do {                                                                                \
    CUresult r_ = (call);                                                             \
    if (r_ != CUDA_SUCCESS) {                                                         \
      const char *s_ = NULL;                                                          \
      cuGetErrorString(r_, &s_);                                                      \
      fprintf(stderr, "g4s_refgpu: %s failed: %s (line %d)\n", #call, s_ ? s_ : "?", \
              __LINE__);                                                              \
      exit(2);                                                                        \
    }                                                                                 \
  } while (0)

/* The reference's Neuron record (gpu4snn.cu:50-62): 9 x 4 bytes. */
typedef struct {
  float v, u, a, b, c, d, I;
  int nospks, neuronid;
} RefNeuron;

/* Mangled names of the reference's kernels (their C++ signatures, gpu4snn.cu:273-716). */
static const char *K_RNG = "_Z17randgeneratorinitjP17curandStateXORWOWi";
static const char *K_INIT = "_Z10initNeuroniiP6NeuronP17curandStateXORWOW";
static const char *K_UPD = "_Z11stateupdateP6NeuronPbPfPjS2_P17curandStateXORWOWiiiiiii";
static const char *K_PROP = "_Z15propagatespikesiPfPjS_ii";
static const char *K_N = "_Z12deliverspks1P6NeuronPbPfPjS2_iiii";
static const char *K_S = "_Z12deliverspks2P6NeuronPbPfPjS2_iiii";
static const char *K_AB = "_Z14AB_deliverspksP6NeuronPbPfPjS2_iiii";
static const char *K_SKL = "_Z15SKL_deliverspksP6NeuronPbPfPjS2_iiiPiP17curandStateXORWOWii";

/* Upper bound of sizeof(curandStateXORWOW) (48 bytes with this toolkit). */
#define STATE_BYTES 64

static int parse_list(const char *s, int *out, int cap) {
  int k = 0;
  while (*s && k < cap) {
    out[k++] = atoi(s);
    const char *c = strchr(s, ',');
    if (!c) break;
    s = c + 1;
  }
  return k;
}

static void *read_file(const char *path, size_t bytes) {
  FILE *f = fopen(path, "rb");
  if (!f) {
    fprintf(stderr, "g4s_refgpu: cannot open %s\n", path);
    exit(2);
  }
  void *p = malloc(bytes ? bytes : 1);
  if (!p || fread(p, 1, bytes, f) != bytes) {
    fprintf(stderr, "g4s_refgpu: %s is shorter than %zu bytes\n", path, bytes);
    exit(2);
  }
  fclose(f);
  return p;
}

typedef struct {
  CUfunction f;
  int block, grid_per_sm;
} Kern;

static Kern kern(CUmodule m, const char *name) {
  Kern k;
  int min_grid = 0;
  CK(cuModuleGetFunction(&k.f, m, name));
  CK(cuOccupancyMaxPotentialBlockSize(&min_grid, &k.block, k.f, NULL, 0, 0));
  CK(cuOccupancyMaxActiveBlocksPerMultiprocessor(&k.grid_per_sm, k.f, k.block, 0));
  return k;
}

int main(int argc, char **argv) {
  const char *cubin = NULL, *fidx = NULL, *fw = NULL, *raster = NULL;
  long long n = 0, nsyn = 0;
  int steps = 0, reps = 1;
  int schemes[8] = {0, 1, 2, 3, 4}, nschemes = 5;
  int modes[3] = {1}, nmodes = 1;
  int seeds[64] = {1}, nseeds = 1;
  for (int i = 1; i + 1 < argc; i += 2) {
    const char *k = argv[i], *v = argv[i + 1];
    if (!strcmp(k, "--cubin")) cubin = v;
    else if (!strcmp(k, "--n")) n = atoll(v);
    else if (!strcmp(k, "--nsyn")) nsyn = atoll(v);
    else if (!strcmp(k, "--idx")) fidx = v;
    else if (!strcmp(k, "--w")) fw = v;
    else if (!strcmp(k, "--steps")) steps = atoi(v);
    else if (!strcmp(k, "--reps")) reps = atoi(v);
    else if (!strcmp(k, "--raster")) raster = v;
    else if (!strcmp(k, "--schemes")) nschemes = parse_list(v, schemes, 8);
    else if (!strcmp(k, "--modes")) nmodes = parse_list(v, modes, 3);
    else if (!strcmp(k, "--seeds")) nseeds = parse_list(v, seeds, 64);
    else {
      fprintf(stderr, "g4s_refgpu: unknown option %s\n", k);
      return 2;
    }
  }
  if (!cubin || !fidx || !fw || n < 2 || nsyn < 1 || nsyn > n || steps < 1 || reps < 1) {
    fprintf(stderr, "g4s_refgpu: need --cubin --n --nsyn --idx --w --steps (see the header)\n");
    return 2;
  }
  if (n * nsyn >= (1LL << 31)) {
    /* every scheme's synapse index or table size is an int product in the reference */
    printf("{\"error\": \"reference cannot run: N x Nsyn = %lld >= 2^31 overflows its int indices\"}\n", n * nsyn);
    return 0;
  }
  for (int i = 0; i < nschemes; ++i)
    if (schemes[i] < 0 || schemes[i] > 4) return fprintf(stderr, "g4s_refgpu: scheme out of range\n"), 2;
  for (int i = 0; i < nmodes; ++i)
    if (modes[i] < 0 || modes[i] > 2) return fprintf(stderr, "g4s_refgpu: mode out of range\n"), 2;

  const int N = (int)n, NS = (int)nsyn;
  const int N_exc = 4 * N / 5, N_inh = N / 5; /* ceil of an integer quotient (gpu4snn.cu:744-745) */
  const size_t syn = (size_t)N * (size_t)NS;
  uint32_t *h_idx = read_file(fidx, syn * 4);
  float *h_w = read_file(fw, syn * 4);
  for (size_t k = 0; k < syn; ++k)
    if (h_idx[k] >= (uint32_t)N) {
      fprintf(stderr, "g4s_refgpu: target %u at synapse %zu is out of range\n", h_idx[k], k);
      return 2;
    }

  CUdevice dev;
  CUcontext ctx;
  CUmodule mod;
  CK(cuInit(0));
  CK(cuDeviceGet(&dev, 0));
  CK(cuDevicePrimaryCtxRetain(&ctx, dev));
  CK(cuCtxSetCurrent(ctx));
  /* room for one pending device launch per neuron: a step of the AP scheme launches one
     child grid per spiking neuron */
  size_t pending = (size_t)N > 2048 ? (size_t)N : 2048;
  CUresult lim = cuCtxSetLimit(CU_LIMIT_DEV_RUNTIME_PENDING_LAUNCH_COUNT, pending);
  if (lim != CUDA_SUCCESS) pending = 0;
  CK(cuModuleLoad(&mod, cubin));
  int sms = 0;
  CK(cuDeviceGetAttribute(&sms, CU_DEVICE_ATTRIBUTE_MULTIPROCESSOR_COUNT, dev));
  char name[256] = {0};
  CK(cuDeviceGetName(name, sizeof name, dev));

  Kern k_rng = kern(mod, K_RNG), k_init = kern(mod, K_INIT), k_upd = kern(mod, K_UPD);
  Kern k_prop = kern(mod, K_PROP), k_n = kern(mod, K_N), k_s = kern(mod, K_S);
  Kern k_ab = kern(mod, K_AB), k_skl = kern(mod, K_SKL);
  /* the reference sizes randgeneratorinit with stateupdate's block (gpu4snn.cu:826-833) */
  const int bs_rng = k_upd.block, grid_rng = (N + bs_rng - 1) / bs_rng;
  const int grid_init = (N + k_init.block - 1) / k_init.block;
  const int grid_upd = (N + k_upd.block - 1) / k_upd.block;
  int grid_ps = (N + k_prop.block - 1) / k_prop.block, bs_ps = k_prop.block;
  const int grid_n = (N + k_n.block - 1) / k_n.block;
  const int grid_s = (int)((syn + (size_t)k_s.block - 1) / (size_t)k_s.block);
  const int grid_ab = sms * k_ab.grid_per_sm, grid_skl = sms * k_skl.grid_per_sm;
  int max_threads = grid_rng * bs_rng;
  if (grid_init * k_init.block > max_threads) max_threads = grid_init * k_init.block;
  if (grid_upd * k_upd.block > max_threads) max_threads = grid_upd * k_upd.block;

  CUdeviceptr d_neuron, d_spikes, d_w, d_idx, d_isyn, d_states, d_total;
  CK(cuMemAlloc(&d_neuron, (size_t)N * sizeof(RefNeuron)));
  CK(cuMemAlloc(&d_spikes, (size_t)N));
  CK(cuMemAlloc(&d_w, syn * 4));
  CK(cuMemAlloc(&d_idx, syn * 4));
  CK(cuMemAlloc(&d_isyn, (size_t)N * 4));
  CK(cuMemAlloc(&d_states, (size_t)max_threads * STATE_BYTES));
  CK(cuMemAlloc(&d_total, 4));
  CK(cuMemcpyHtoD(d_w, h_w, syn * 4));
  CK(cuMemcpyHtoD(d_idx, h_idx, syn * 4));
  free(h_w);
  free(h_idx);

  RefNeuron *h_neuron = malloc((size_t)N * sizeof(RefNeuron));
  unsigned char *h_spk = malloc((size_t)N);
  CUevent e0, e1;
  CK(cuEventCreate(&e0, CU_EVENT_DEFAULT));
  CK(cuEventCreate(&e1, CU_EVENT_DEFAULT));

  for (int is = 0; is < nschemes; ++is)
    for (int im = 0; im < nmodes; ++im)
      for (int ir = 0; ir < nseeds; ++ir)
        for (int rep = 0; rep < reps; ++rep) {
          int scheme = schemes[is], mode = modes[im];
          unsigned seed = (unsigned)seeds[ir];
          int nn = N, ne = N_exc, ni = N_inh, nsy = NS, count = steps, dyn = scheme;
          /* fresh cuRAND streams and parameters every run (the reference re-draws the
             parameters from streams that earlier runs advanced, gpu4snn.cu:1094) */
          CK(cuMemsetD8(d_states, 0, (size_t)max_threads * STATE_BYTES));
          CK(cuMemsetD8(d_isyn, 0, (size_t)N * 4));
          CK(cuMemsetD8(d_spikes, 0, (size_t)N));
          CK(cuMemsetD8(d_total, 0, 4));
          void *a_rng[] = {&seed, &d_states, &nn};
          CK(cuLaunchKernel(k_rng.f, grid_rng, 1, 1, bs_rng, 1, 1, 0, NULL, a_rng, NULL));
          void *a_init[] = {&ne, &nn, &d_neuron, &d_states};
          CK(cuLaunchKernel(k_init.f, grid_init, 1, 1, k_init.block, 1, 1, 0, NULL, a_init, NULL));
          CK(cuCtxSynchronize());

          FILE *rf = NULL;
          if (raster && scheme != 4) {
            char path[1024];
            snprintf(path, sizeof path, "%s_s%d_m%d_r%u.bin", raster, scheme, mode, seed);
            rf = fopen(path, "wb");
            if (!rf) return fprintf(stderr, "g4s_refgpu: cannot write %s\n", path), 2;
          }
          long long rec_spikes = 0;
          void *a_upd[] = {&d_neuron, &d_spikes, &d_w, &d_idx, &d_isyn, &d_states, &nn, &ne, &nsy,
                           &grid_ps, &bs_ps, &dyn, &mode};
          void *a_del[] = {&d_neuron, &d_spikes, &d_w, &d_idx, &d_isyn, &nn, &ne, &ni, &nsy};
          void *a_skl[] = {&d_neuron, &d_spikes, &d_w, &d_idx, &d_isyn, &nn, &ne, &nsy, &d_total, &d_states,
                           &mode, &count};
          CK(cuEventRecord(e0, NULL));
          if (scheme == 4) {
            CK(cuLaunchCooperativeKernel(k_skl.f, grid_skl, 1, 1, k_skl.block, 1, 1, 0, NULL, a_skl));
          } else {
            for (int t = 0; t < steps; ++t) {
              CK(cuLaunchKernel(k_upd.f, grid_upd, 1, 1, k_upd.block, 1, 1, 0, NULL, a_upd, NULL));
              if (scheme == 1)
                CK(cuLaunchKernel(k_n.f, grid_n, 1, 1, k_n.block, 1, 1, 0, NULL, a_del, NULL));
              else if (scheme == 2)
                CK(cuLaunchKernel(k_s.f, grid_s, 1, 1, k_s.block, 1, 1, 0, NULL, a_del, NULL));
              else if (scheme == 3)
                CK(cuLaunchCooperativeKernel(k_ab.f, grid_ab, 1, 1, k_ab.block, 1, 1, 0, NULL, a_del));
              if (rf) {
                CK(cuMemcpyDtoH(h_spk, d_spikes, (size_t)N));
                for (int i = 0; i < N; ++i)
                  if (h_spk[i]) {
                    int32_t pair[2] = {t, i};
                    fwrite(pair, sizeof pair, 1, rf);
                    rec_spikes++;
                  }
              }
            }
          }
          CK(cuEventRecord(e1, NULL));
          CK(cuEventSynchronize(e1));
          CK(cuCtxSynchronize());
          float ms = 0.f;
          CK(cuEventElapsedTime(&ms, e0, e1));
          const int with_data = rf != NULL;
          if (rf) fclose(rf);
          CK(cuMemcpyDtoH(h_neuron, d_neuron, (size_t)N * sizeof(RefNeuron)));
          long long spikes = 0;
          for (int i = 0; i < N; ++i) spikes += h_neuron[i].nospks;
          int total = 0;
          CK(cuMemcpyDtoH(&total, d_total, 4));
          int grid = scheme == 4 ? grid_skl : scheme == 3 ? grid_ab : scheme == 2 ? grid_s : scheme == 1 ? grid_n : grid_upd;
          int block = scheme == 4 ? k_skl.block : scheme == 3 ? k_ab.block : scheme == 2 ? k_s.block : scheme == 1 ? k_n.block : k_upd.block;
          printf("{\"scheme\": %d, \"mode\": %d, \"seed\": %u, \"rep\": %d, \"n\": %d, \"nsyn\": %d, \"steps\": %d, "
                 "\"spikes\": %lld, \"raster_spikes\": %lld, \"skl_total\": %d, \"ms\": %.6f, \"with_data\": %d, "
                 "\"grid\": %d, \"block\": %d, \"update_grid\": %d, \"update_block\": %d, \"ap_child_grid\": %d, "
                 "\"ap_child_block\": %d, \"pending_launch_limit\": %zu, \"sms\": %d, \"device\": \"%s\"}\n",
                 scheme, mode, seed, rep, N, NS, steps, spikes, rec_spikes, total, ms, with_data, grid, block, grid_upd,
                 k_upd.block, grid_ps, bs_ps, pending, sms, name);
          fflush(stdout);
        }
  cuMemFree(d_neuron);
  cuMemFree(d_spikes);
  cuMemFree(d_w);
  cuMemFree(d_idx);
  cuMemFree(d_isyn);
  cuMemFree(d_states);
  cuMemFree(d_total);
  cuModuleUnload(mod);
  cuDevicePrimaryCtxRelease(dev);
  free(h_neuron);
  free(h_spk);
  return 0;
}
