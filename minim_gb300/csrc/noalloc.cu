// noalloc.cu -- allocation-free minimisation of one Lennard-Jones cluster.
//
// Some callers cannot allocate device memory: a program embedded in another
// runtime that has already reserved the GPU's memory for its own caching
// allocator (cudaMalloc would fail or fragment that pool), or a latency-
// critical loop that must not enter the driver's allocator.  For them this
// file provides minim_gpu_lj_minimise_noalloc(): the caller supplies the
// coordinates in device memory (read as the start, overwritten with the
// minimum) and a stream; every other byte the minimiser needs -- its
// coordinate copies, gradients, L-BFGS history or FIRE velocity and its
// state -- lives in the fixed array below, which every GPU that loads this
// library holds until the process exits.
//
//   * capacity: kMaxDof degrees of freedom (1024 particles in 3-D) with an
//     L-BFGS history of up to 16 pairs, in kScratchBytes (1 MiB);
//   * every call uses the same array: calls whose work overlaps on the GPU
//     (two streams, two host threads) race and corrupt each other -- the
//     caller must serialise them;
//   * the host does not know the array's device address; it is looked up
//     with cudaGetSymbolAddress on the first call on each device (with that
//     device current), together with the kernel's per-device opt-in to its
//     shared-memory size;
//   * the state record at the start of the array is reset on every call; the
//     kernel writes every vector before reading it.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "kernels.cuh"
#include "minim_gpu.h"

namespace {

constexpr size_t kScratchBytes = 1u << 20;
constexpr int kMaxDof = 3072;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_setup_mu;
void* g_scratch_addr[128];
bool g_scratch_ready[128];
// the kernel's opt-in to more than 48 KB of shared memory is a per-device
// function attribute: set once on each device, with the address lookup
bool g_smem_ready[128];

size_t up256(size_t v) { return (v + 255) & ~(size_t)255; }

}  // namespace

namespace mg {

__global__ void __launch_bounds__(256, 2) noalloc_lj_kernel(InstDesc d, int slice, int lj_tile) {
  __shared__ SharedScalars<> S;
  __shared__ __align__(16) InstDesc s_in;
  extern __shared__ __align__(16) unsigned char dyn[];
  if (threadIdx.x == 0) s_in = d;
  __syncthreads();
  CtaTeam tm{S.red, S.wide};
  Runner<CtaTeam, K_LJ> R{tm, s_in, dyn, lj_tile};
  setup_runner(R, S, s_in);
  R.load(*s_in.st);
  R.run(slice);
  R.store(*s_in.st);
}

}  // namespace mg

extern "C" void mg_set_last_error(const char* msg);

extern "C" int minim_gpu_lj_minimise_noalloc(const minim_gpu_lj_params* p, double* x_dev, size_t ndof,
                                             const minim_gpu_minimiser_params* mp, minim_gpu_result* res,
                                             void* stream) {
  using namespace mg;
  if (!p || !x_dev || !mp || !res) {
    mg_set_last_error("minim_gpu_lj_minimise_noalloc: null argument");
    return MINIM_GPU_ERR_INVALID;
  }
  if (p->ndim < 2 || p->ndim > 3 || ndof == 0 || ndof % p->ndim) {
    mg_set_last_error("LjNd: Length of coords must be a multiple of the number of dimensions.");
    return MINIM_GPU_ERR_INVALID;
  }
  if (p->cutoff != 0) {
    mg_set_last_error("minim_gpu_lj_minimise_noalloc: evaluates every pair (cutoff must be 0)");
    return MINIM_GPU_ERR_INVALID;
  }
  if (ndof > (size_t)kMaxDof) {
    mg_set_last_error("minim_gpu_lj_minimise_noalloc: at most 3072 degrees of freedom "
                      "(1024 particles in 3-D) fit the fixed scratch array");
    return MINIM_GPU_ERR_INVALID;
  }
  if (mp->method < 0 || mp->method > 2 || (mp->method == MINIM_LBFGS && (mp->m < 1 || mp->m > MINIM_MAXM)) ||
      mp->precision < 0 || mp->precision > 2 ||
      (mp->linesearch != MINIM_LS_BACKTRACKING && mp->linesearch != MINIM_LS_NONE)) {
    mg_set_last_error("minim_gpu_lj_minimise_noalloc: invalid minimiser parameters");
    return MINIM_GPU_ERR_INVALID;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 128) {
    mg_set_last_error("minim_gpu_lj_minimise_noalloc: no current CUDA device");
    return MINIM_GPU_ERR_NO_DEVICE;
  }
  int major = 0, minor = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  if (major != 10 || minor != 3) {
    mg_set_last_error("minim_gpu_lj_minimise_noalloc: the kernels are built for sm_103a");
    return MINIM_GPU_ERR_NO_DEVICE;
  }
  const int lj_tile = 1536;  // the batch kernels' shared memory (48 KB)
  const size_t smem = (size_t)lj_tile * sizeof(D4);
  unsigned char* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_smem_ready[dev]) {
      // static plus dynamic shared memory is above the 48 KB default
      const cudaError_t e = cudaFuncSetAttribute((const void*)noalloc_lj_kernel,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) {
        mg_set_last_error(cudaGetErrorString(e));
        return MINIM_GPU_ERR_CUDA;
      }
      g_smem_ready[dev] = true;
    }
    if (!g_scratch_ready[dev]) {
      void* a = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&a, g_noalloc_scratch);
      if (e != cudaSuccess || a == nullptr) {
        mg_set_last_error(cudaGetErrorString(e));
        return MINIM_GPU_ERR_CUDA;
      }
      g_scratch_addr[dev] = a;
      g_scratch_ready[dev] = true;
    }
    base = static_cast<unsigned char*>(g_scratch_addr[dev]);
  }
  // carve the scratch array: state record, then the minimiser's vectors
  const size_t n = ndof;
  const size_t hs = (n + 63) & ~(size_t)63;
  const bool fp64 = mp->precision != MINIM_PREC_FP32;
  const int nS = mp->method == MINIM_LBFGS ? mp->m + 1 : (mp->method == MINIM_FIRE ? 1 : 0);
  const int nY = mp->method == MINIM_LBFGS ? mp->m + 1 : 0;
  size_t off = 0;
  auto take = [&](size_t bytes) { const size_t r = off; off += up256(bytes); return base + r; };
  InstDesc d;
  std::memset(&d, 0, sizeof d);
  d.kind = K_LJ;
  d.ndof = (int)n;
  d.lj.ndim = p->ndim;
  d.lj.np = (int)(n / p->ndim);
  d.lj.s6 = std::pow(p->sigma, 6);
  d.lj.eps = p->epsilon;
  d.st = reinterpret_cast<MinScalars*>(take(sizeof(MinScalars)));
  for (int k = 0; k < 2; k++) d.X32[k] = reinterpret_cast<float*>(take(n * 4));
  for (int k = 0; k < 2; k++) d.X64[k] = fp64 ? reinterpret_cast<double*>(take(n * 8)) : nullptr;
  for (int k = 0; k < 2; k++) d.G[k] = reinterpret_cast<float*>(take(n * 4));
  d.hstride = (int)hs;
  d.Sb = nS ? reinterpret_cast<float*>(take((size_t)nS * hs * 4)) : nullptr;
  d.Yb = nY ? reinterpret_cast<float*>(take((size_t)nY * hs * 4)) : nullptr;
  d.V = mp->method == MINIM_FIRE ? reinterpret_cast<float*>(take(n * 4)) : nullptr;
  if (off > kScratchBytes) {
    mg_set_last_error("minim_gpu_lj_minimise_noalloc: workspace exceeds the fixed scratch array");
    return MINIM_GPU_ERR_INVALID;
  }
  d.xres = x_dev;
  d.mp.method = mp->method;
  d.mp.linesearch = mp->linesearch;
  d.mp.max_iter = mp->max_iter;
  d.mp.m = mp->method == MINIM_LBFGS ? mp->m : 0;
  d.mp.precision = mp->precision;
  d.mp.tol = mp->tol >= 0 ? mp->tol : 1e-6;
  d.mp.max_step = mp->max_step;
  d.mp.init_step = mp->init_step;
  d.mp.dt_max = mp->dt_max;
  d.mp.alpha = mp->alpha;
  // the state record starts fresh on every call
  MinScalars s;
  std::memset(&s, 0, sizeof s);
  s.status = ST_RUNNING;
  s.pend = -1;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemcpyAsync(d.st, &s, sizeof s, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    noalloc_lj_kernel<<<1, 256, smem, st>>>(d, 0x7fffffff, lj_tile);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&s, d.st, sizeof s, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    mg_set_last_error(cudaGetErrorString(e));
    return MINIM_GPU_ERR_CUDA;
  }
  std::memset(res, 0, sizeof *res);
  res->status = s.status;
  res->iter = s.iter;
  res->fp64_iters = s.fp64_iters;
  res->evals = s.evals;
  res->energy = s.E;
  res->rms = std::sqrt(s.gg / (double)n);
  res->dt_max = s.dtmax;
  return MINIM_GPU_OK;
}
