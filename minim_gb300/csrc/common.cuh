// common.cuh -- device-side building blocks shared by every kernel.
//
// A "team" is the set of threads that cooperate on one minimisation:
//   CtaTeam  : one thread block (batched path: one instance per CTA),
//   GridTeam : every block of a cooperative launch (one large instance).
// Both expose the same interface, so the potentials and the minimiser are
// written once.  Reductions are deterministic: fixed-order warp butterflies,
// then a fixed-order sum over warps / blocks, all in FP64, and every thread
// of the team receives bitwise the same result (uniform control flow).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "engine.h"

#define MINIM_MAXRED 8    // values reduced together in one team reduction

namespace mg {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Accumulates a stream of FP32 terms: short runs are summed in FP32 and
// flushed into an FP64 total (the FP64 pipe is a scarce resource on GB300;
// the FP32 run length bounds the FP32 rounding).
struct Acc {
  double d;
  float f;
  int n;
  __device__ __forceinline__ Acc() : d(0.0), f(0.f), n(0) {}
  __device__ __forceinline__ void add(float v) {
    f += v;
    if (++n == 8) { d += (double)f; f = 0.f; n = 0; }
  }
  __device__ __forceinline__ void add(double v) { d += v; }
  __device__ __forceinline__ double total() const { return d + (double)f; }
};

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// ---------------------------------------------------------------------------
// Team = one CTA
// ---------------------------------------------------------------------------
struct CtaTeam {
  int tid, nthr;
  double* red;  // shared scratch, >= (32 + 1) * MINIM_MAXRED doubles
  static constexpr bool kGrid = false;
  __device__ __forceinline__ void sync() { __syncthreads(); }
  __device__ __forceinline__ bool ok() const { return true; }
  __device__ __forceinline__ bool block0() const { return true; }

  template <int K>
  __device__ void reduce(double (&v)[K]) {
    static_assert(K <= MINIM_MAXRED, "too many values");
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < K; k++) v[k] = warp_sum(v[k]);
    if (lane == 0) {
#pragma unroll
      for (int k = 0; k < K; k++) red[w * MINIM_MAXRED + k] = v[k];
    }
    __syncthreads();
    if (threadIdx.x < K) {
      double s = 0.0;
      for (int i = 0; i < nw; i++) s += red[i * MINIM_MAXRED + threadIdx.x];
      red[32 * MINIM_MAXRED + threadIdx.x] = s;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; k++) v[k] = red[32 * MINIM_MAXRED + k];
    __syncthreads();
  }
};

// ---------------------------------------------------------------------------
// Team = whole grid (cooperative launch), with a bounded software barrier
// ---------------------------------------------------------------------------
struct GridTeam {
  int tid, nthr;
  double* red;            // shared scratch as in CtaTeam
  GridSyncState* bar;     // global
  double* partials;       // global, 2 * gridDim.x * MINIM_MAXRED doubles
  int buf;                // partials double buffer index
  int* s_ok;              // shared flag
  static constexpr bool kGrid = true;
  static constexpr unsigned long long kWaitLimitNs = 5000000000ull;  // 5 s

  __device__ __forceinline__ bool block0() const { return blockIdx.x == 0; }
  __device__ __forceinline__ bool ok() const { return *s_ok != 0; }

  // Sense-counting barrier over all blocks.  Every wait is bounded: after
  // kWaitLimitNs the block records an error and leaves; blocks arriving
  // later see the error flag and leave too, so the kernel always returns.
  __device__ void sync() {
    __syncthreads();
    if (threadIdx.x == 0) {
      int okv = *s_ok;
      if (okv) {
        volatile unsigned int* vgen = &bar->gen;
        volatile int* verr = &bar->err;
        unsigned int g = *vgen;
        __threadfence();
        unsigned int arrived = atomicAdd(&bar->count, 1u);
        if (arrived == gridDim.x - 1) {
          atomicExch(&bar->count, 0u);
          __threadfence();
          atomicAdd(&bar->gen, 1u);
        } else {
          unsigned long long t0 = globaltimer_ns();
          while (*vgen == g) {
            if (*verr) { okv = 0; break; }
            if (globaltimer_ns() - t0 > kWaitLimitNs) {
              atomicExch(&bar->err, 1);
              okv = 0;
              break;
            }
            __nanosleep(64);
          }
        }
        __threadfence();
        if (*verr) okv = 0;
      }
      *s_ok = okv;
    }
    __syncthreads();
  }

  template <int K>
  __device__ void reduce(double (&v)[K]) {
    static_assert(K <= MINIM_MAXRED, "too many values");
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < K; k++) v[k] = warp_sum(v[k]);
    if (lane == 0) {
#pragma unroll
      for (int k = 0; k < K; k++) red[w * MINIM_MAXRED + k] = v[k];
    }
    __syncthreads();
    double* P = partials + (size_t)buf * gridDim.x * MINIM_MAXRED;
    if (threadIdx.x < K) {
      double s = 0.0;
      for (int i = 0; i < nw; i++) s += red[i * MINIM_MAXRED + threadIdx.x];
      P[blockIdx.x * MINIM_MAXRED + threadIdx.x] = s;
    }
    sync();
    if (w == 0) {
      for (int k = 0; k < K; k++) {
        double s = 0.0;
        for (int b = lane; b < (int)gridDim.x; b += 32) s += __ldcg(&P[b * MINIM_MAXRED + k]);
        s = warp_sum(s);
        if (lane == 0) red[32 * MINIM_MAXRED + k] = s;
      }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; k++) v[k] = red[32 * MINIM_MAXRED + k];
    __syncthreads();
    buf ^= 1;
  }
};

}  // namespace mg
