/*
 * probe.cu -- measured peak of the operation that bounds the histogram
 * updates of the counting kernels: 32-bit atomic adds to shared memory.
 *
 * The pair-counting kernels do one shared-memory atomic add per in-range
 * pair (two for weighted sums); the rate at which an SM retires such adds
 * when the 32 lanes of a warp hit 32 different banks is the denominator of
 * that part of their roofline.  No counterpart in the reference.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "fcfcg_internal.h"

#define PROBE_THREADS 256
#define PROBE_WORDS 2048

/* Every thread adds 1 to its own shared word `iters` times (lane-distinct
 * banks: no conflicts inside a warp), then checks the total, so the adds
 * cannot be dropped; a wrong total is counted in *bad. */
__global__ void __launch_bounds__(PROBE_THREADS)
k_probe_smem_atomics(int iters, unsigned *bad) {
  __shared__ unsigned h[PROBE_WORDS];
  for (int i = threadIdx.x; i < PROBE_WORDS; i += blockDim.x) h[i] = 0;
  __syncthreads();
  unsigned *p = h + threadIdx.x;
#pragma unroll 16
  for (int k = 0; k < iters; k++) atomicAdd(p, 1u);
  __syncthreads();
  if (h[threadIdx.x] != (unsigned) iters) atomicAdd(bad, 1u);
}

extern "C" int fcfcg_probe_smem_atomics(int device, double *adds_per_s) {
  if (!adds_per_s) return FCFCG_ERR_ARG;
  *adds_per_s = 0;
  cudaError_t e;
  int prev = 0;
  if ((e = cudaGetDevice(&prev))) return FCFCG_ERR_CUDA;
  const int dev = device < 0 ? prev : device;
  if ((e = cudaSetDevice(dev))) return FCFCG_ERR_CUDA;
  int nsm = 0, per_sm = 0;
  if ((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) ||
      (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
           &per_sm, (const void *) k_probe_smem_atomics, PROBE_THREADS, 0)) ||
      per_sm < 1) {
    cudaSetDevice(prev);
    return FCFCG_ERR_CUDA;
  }
  const int blocks = nsm * per_sm, iters = 1 << 14;
  unsigned *bad = NULL;
  cudaEvent_t e0 = NULL, e1 = NULL;
  cudaStream_t st = NULL;
  int rc = FCFCG_ERR_CUDA;
  unsigned hbad = 0;
  float best = 0.f;
  if (cudaMalloc((void **) &bad, sizeof(unsigned)) ||
      cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) ||
      cudaEventCreate(&e0) || cudaEventCreate(&e1) ||
      cudaMemsetAsync(bad, 0, sizeof(unsigned), st))
    goto out;
  for (int rep = 0; rep < 4; rep++) {     /* the first one warms up */
    float ms = 0.f;
    if (cudaEventRecord(e0, st)) goto out;
    k_probe_smem_atomics<<<blocks, PROBE_THREADS, 0, st>>>(iters, bad);
    if (cudaGetLastError() || cudaEventRecord(e1, st) ||
        cudaEventSynchronize(e1) || cudaEventElapsedTime(&ms, e0, e1))
      goto out;
    if (rep && (best == 0.f || ms < best)) best = ms;
  }
  if (cudaMemcpy(&hbad, bad, sizeof hbad, cudaMemcpyDeviceToHost)) goto out;
  if (hbad || best <= 0.f) {
    rc = FCFCG_ERR_DATA;
    goto out;
  }
  *adds_per_s = (double) blocks * PROBE_THREADS * iters / (best * 1e-3);
  rc = FCFCG_OK;
out:
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  if (bad) cudaFree(bad);
  cudaSetDevice(prev);
  return rc;
}
