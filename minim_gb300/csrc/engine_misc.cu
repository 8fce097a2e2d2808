// engine_misc.cu -- conversion helpers used by the host runtime.
#include <cuda_runtime.h>
#include <stddef.h>

#include "common.cuh"

// ---- small helpers used by the host runtime -------------------------------------
__global__ void k_d2f(const double* __restrict__ a, float* __restrict__ b, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}
__global__ void k_f2d(const float* __restrict__ a, double* __restrict__ b, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    b[i] = (double)a[i];
}

extern "C" int mg_convert(const void* src, void* dst, size_t n, int to_float, void* stream) {
  const int threads = 256;
  int blocks = (int)((n + threads - 1) / threads);
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (blocks < 1) blocks = 1;
  if (to_float)
    k_d2f<<<blocks, threads, 0, (cudaStream_t)stream>>>((const double*)src, (float*)dst, n);
  else
    k_f2d<<<blocks, threads, 0, (cudaStream_t)stream>>>((const float*)src, (double*)dst, n);
  return (int)cudaGetLastError();
}

// The grid barrier's bounded wait on an arrival count that nothing reaches:
// thread 0 of the one block gives up after bar->limit_ms, records the error
// in bar->err, and the kernel returns.
__global__ void k_wait_probe(mg::GridSyncState* bar) {
  if (threadIdx.x != 0) return;
  int ok = 1;
  mg::GridTeam tm{nullptr, nullptr, bar, nullptr, 0, &ok, 0u};
  tm.wait_count(0xffffffffu);
}

extern "C" int mg_wait_probe(mg::GridSyncState* bar, void* stream) {
  k_wait_probe<<<1, 32, 0, (cudaStream_t)stream>>>(bar);
  return (int)cudaGetLastError();
}
