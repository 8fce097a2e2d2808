// math_probe.cu -- test-only kernels that evaluate the engine's hand-written
// arithmetic helpers next to CUDA's own correctly rounded operations, for
// tests/test_gpu_math_helpers.py (compiled by that test; not part of the
// engine library).
//
//   rcp_nr(x)            (common.cuh)     against __frcp_rn(x)
//   df_rcp(split(x))     (common.cuh)     against 1.0 / x in FP64
//   bah_sqrt<DFn>(x)     (potentials.cuh) against sqrt(x) in FP64
//   df_split_bits(x)     (common.cuh)     against x itself
//   DF product a * b     (common.cuh)     against a * b in FP64
//   dfl_rcp(split(x))    (potentials.cuh) against 1.0 / x in FP64
//   DFl sum a + b        (potentials.cuh) against the FP64 sum of its inputs
#include <cuda_runtime.h>

#include "potentials.cuh"

using namespace mg;

__global__ void k_probe(const double* x, const double* y, double* out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double a = x[i], b = y[i];
  const float af = (float)a;
  double* o = out + 12 * (size_t)i;
  o[0] = (double)rcp_nr(af);
  o[1] = (double)__frcp_rn(af);
  const DF s = df_split_bits(a);
  o[2] = df_to(s);
  o[3] = df_to(df_rcp(s));
  o[4] = 1.0 / a;
  o[5] = (double)bah_sqrt<DFn>(DFn(s));
  o[6] = sqrt(a);
  o[7] = df_to(df_split_bits(a) * df_split_bits(b));
  const DFl la = dfl(s), lb = dfl(df_split_bits(b));
  o[8] = dfl_to(dfl_rcp(la));
  o[9] = dfl_to(la + lb);
  o[10] = dfl_to(la) + dfl_to(lb);
  o[11] = fabs(dfl_to(la)) + fabs(dfl_to(lb));
}

// out: 12 values per input (see k_probe); returns a cudaError_t
extern "C" int math_probe(const double* x, const double* y, double* out, int n) {
  double *dx = nullptr, *dy = nullptr, *dout = nullptr;
  cudaError_t e = cudaMalloc(&dx, n * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&dy, n * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&dout, 12 * (size_t)n * sizeof(double));
  if (e == cudaSuccess) e = cudaMemcpy(dx, x, n * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dy, y, n * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_probe<<<(n + 255) / 256, 256>>>(dx, dy, dout, n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(out, dout, 12 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost);
  cudaFree(dx);
  cudaFree(dy);
  cudaFree(dout);
  return (int)e;
}
