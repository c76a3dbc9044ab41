/*
 * Link-time wraps that let the reference's own host code (gpu4snn.cu:735-911) run on a
 * machine without a GPU, up to the point where it has generated its connectivity tables.
 *   time()                         -> G4S_REF_SEED, so srand() (gpu4snn.cu:873) is seeded
 *   device queries / occupancy     -> fixed plausible values (16 SMs, 1024 threads)
 *   cudaMalloc                     -> host calloc (the pointers are only passed around)
 *   cudaMemcpy host->device        -> the 1st copy (weights, gpu4snn.cu:910) and the 2nd
 *                                     (targets, :911) are written to $G4S_REF_OUT, then exit
 * Kernel launches before that point fail with "no device" and are ignored by the reference.
 */
#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

time_t __wrap_time(time_t *t) {
  const char *s = getenv("G4S_REF_SEED");
  time_t v = (time_t)strtoll(s ? s : "1", 0, 10);
  if (t) *t = v;
  return v;
}
cudaError_t __wrap_cudaGetDevice(int *d) { *d = 0; return cudaSuccess; }
cudaError_t __wrap_cudaDeviceGetAttribute(int *v, enum cudaDeviceAttr a, int dev) {
  (void)dev;
  switch (a) {
    case cudaDevAttrMaxThreadsPerBlock: *v = 1024; break;
    case cudaDevAttrMultiProcessorCount: *v = 16; break;
    case cudaDevAttrMaxThreadsPerMultiProcessor: *v = 1024; break;
    case cudaDevAttrWarpSize: *v = 32; break;
    default: *v = 65536;
  }
  return cudaSuccess;
}
cudaError_t __wrap_cudaFuncGetAttributes(struct cudaFuncAttributes *a, const void *f) {
  (void)f;
  memset(a, 0, sizeof *a);
  a->maxThreadsPerBlock = 1024;
  a->numRegs = 32;
  return cudaSuccess;
}
cudaError_t __wrap_cudaOccupancyMaxActiveBlocksPerMultiprocessorWithFlags(int *n, const void *f, int bs,
                                                                          size_t sm, unsigned fl) {
  (void)f; (void)bs; (void)sm; (void)fl;
  *n = 1;
  return cudaSuccess;
}
cudaError_t __wrap_cudaGetDeviceProperties(struct cudaDeviceProp *p, int dev) {
  (void)dev;
  memset(p, 0, sizeof *p);
  p->warpSize = 32;
  p->multiProcessorCount = 16;
  p->maxThreadsPerMultiProcessor = 1024;
  p->maxThreadsPerBlock = 1024;
  return cudaSuccess;
}
cudaError_t __wrap_cudaMalloc(void **p, size_t n) {
  *p = calloc(1, n ? n : 1);
  return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
static int ncopies = 0;
cudaError_t __wrap_cudaMemcpy(void *dst, const void *src, size_t n, enum cudaMemcpyKind k) {
  if (k != cudaMemcpyHostToDevice) {
    memset(dst, 0, n);
    return cudaSuccess;
  }
  const char *dir = getenv("G4S_REF_OUT");
  char path[4096];
  snprintf(path, sizeof path, "%s/%s", dir ? dir : ".", ncopies == 0 ? "conn_w.bin" : "conn_idx.bin");
  FILE *f = fopen(path, "wb");
  if (!f) {
    perror(path);
    exit(2);
  }
  fwrite(src, 1, n, f);
  fclose(f);
  if (++ncopies == 2) exit(0);
  return cudaSuccess;
}
