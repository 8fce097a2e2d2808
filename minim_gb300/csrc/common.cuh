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
#define MINIM_WIDE 64     // values reduced together in one wide reduction

namespace mg {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Warp reduce-scatter of 32 values: on entry every lane holds v[0..31]; on
// exit lane l holds, in v[0], the sum over the warp of v[l].  31 shuffles per
// lane instead of 5 per value.
__device__ __forceinline__ float warp_reduce_scatter32(float* v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int s = 16; s >= 1; s >>= 1) {
    const bool up = (lane & s) != 0;
#pragma unroll
    for (int j = 0; j < s; j++) {
      const float send = up ? v[j] : v[j + s];
      const float keep = up ? v[j + s] : v[j];
      v[j] = keep + __shfl_xor_sync(0xffffffffu, send, s);
    }
  }
  return v[0];
}

// Wide reductions are assembled in three steps: every warp zeroes its row of
// the shared `wide` table (wide_clear), adds groups of 32 per-thread partials
// -- 4 dot products x 8 slots -- to it (wide_store32, value index
// dot * 16 + k0 + slot), then the team combines the rows (wide_combine).
__device__ __forceinline__ void wide_clear_row(double* wide) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  wide[w * MINIM_WIDE + lane] = 0.0;
  wide[w * MINIM_WIDE + 32 + lane] = 0.0;
  __syncwarp();
}
__device__ __forceinline__ void wide_store_row(float (&v)[32], int k0, double* wide) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const float a = warp_reduce_scatter32(v);
  wide[w * MINIM_WIDE + (lane >> 3) * 16 + k0 + (lane & 7)] = (double)a;
  __syncwarp();
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

// aligned 4-wide access to FP32 vectors (element 4*i4 .. 4*i4+3)
__device__ __forceinline__ float4 ld4(const float* p, int i4) {
  return reinterpret_cast<const float4*>(p)[i4];
}
__device__ __forceinline__ void st4(float* p, int i4, float4 v) { reinterpret_cast<float4*>(p)[i4] = v; }
__device__ __forceinline__ float dot4(float4 a, float4 b) {
  return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w;
}
__device__ __forceinline__ float4 axpy4(float a, float4 x, float4 y) {  // a*x + y
  return make_float4(fmaf(a, x.x, y.x), fmaf(a, x.y, y.y), fmaf(a, x.z, y.z), fmaf(a, x.w, y.w));
}

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
  double* wide; // shared scratch, >= (8 + 1) * MINIM_WIDE doubles
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

  __device__ __forceinline__ void wide_clear() { wide_clear_row(wide); }
  __device__ __forceinline__ void wide_store32(float (&v)[32], int k0) { wide_store_row(v, k0, wide); }
  // Combines the warps' rows: FP64 totals of values 0..K-1 in out (shared).
  __device__ void wide_combine(int K, double* out) {
    const int nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
      double s = 0.0;
      for (int i = 0; i < nw; i++) s += wide[i * MINIM_WIDE + k];
      out[k] = s;
    }
    __syncthreads();
  }
};

// ---------------------------------------------------------------------------
// Team = whole grid (cooperative launch), with a bounded software barrier
// ---------------------------------------------------------------------------
struct GridTeam {
  int tid, nthr;
  double* red;            // shared scratch as in CtaTeam
  double* wide;           // shared scratch as in CtaTeam
  GridSyncState* bar;     // global
  double* partials;       // global: 2 * gridDim.x * MINIM_WIDE partials, 2 * MINIM_WIDE
                          // totals, then gridDim.x unsigned flags
  int buf;                // partials double buffer index
  int* s_ok;              // shared flag
  unsigned int epoch;     // barriers passed in this launch (uniform)
  static constexpr bool kGrid = true;
  static constexpr unsigned long long kWaitLimitNs = 5000000000ull;  // 5 s

  __device__ __forceinline__ bool block0() const { return blockIdx.x == 0; }
  __device__ __forceinline__ bool ok() const { return *s_ok != 0; }

  // Bounded wait until *p reaches `want` (or an error was recorded).
  __device__ bool wait_value(volatile unsigned int* p, unsigned int want) {
    volatile int* verr = &bar->err;
    unsigned long long t0 = 0;
    while (*p < want) {
      if (*verr) return false;
      const unsigned long long t = globaltimer_ns();
      if (t0 == 0) {
        t0 = t;
      } else if (t - t0 > kWaitLimitNs) {
        atomicExch(&bar->err, 1);
        return false;
      }
      __nanosleep(32);
    }
    return true;
  }

  // Flag barrier with an optional reduction.  Every block publishes the
  // barrier's epoch in its own flag (no contended atomics); block 0 waits for
  // all flags in parallel, sums the blocks' K partials in a fixed order into
  // the published totals, then releases the others by publishing the epoch.
  // Every wait is bounded (kWaitLimitNs): a block that gives up records an
  // error; later barriers see it and return at once, so the kernel always
  // finishes (status TIMEOUT).
  __device__ void arrive_release(int K, double* out) {
    unsigned int* flags =
        reinterpret_cast<unsigned int*>(partials + (size_t)2 * gridDim.x * MINIM_WIDE + 2 * MINIM_WIDE);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    double* P = partials + (size_t)buf * gridDim.x * MINIM_WIDE;
    double* Rz = partials + (size_t)2 * gridDim.x * MINIM_WIDE + (size_t)buf * MINIM_WIDE;
    const unsigned int ep = ++epoch;
    __syncthreads();
    const bool okb = *s_ok != 0;
    __syncthreads();
    if (okb) {
      if (threadIdx.x == 0) {
        __threadfence();
        *(volatile unsigned int*)&flags[blockIdx.x] = ep;
      }
      if (blockIdx.x == 0) {
        bool okv = true;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
          okv = wait_value((volatile unsigned int*)&flags[b], ep) && okv;
        if (!okv) *s_ok = 0;
        __threadfence();
        __syncthreads();
        if (*s_ok) {
          for (int k = w; k < K; k += nw) {
            double s = 0.0;
            for (int b = lane; b < (int)gridDim.x; b += 32) s += __ldcg(&P[b * MINIM_WIDE + k]);
            s = warp_sum(s);
            if (lane == 0) Rz[k] = s;
          }
          __syncthreads();
          if (threadIdx.x == 0) {
            __threadfence();
            *(volatile unsigned int*)&bar->gen = ep;
          }
        }
      } else if (threadIdx.x == 0) {
        if (!wait_value((volatile unsigned int*)&bar->gen, ep)) *s_ok = 0;
        __threadfence();
      }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < K; k += blockDim.x) out[k] = __ldcg(&Rz[k]);
    __syncthreads();
    buf ^= 1;
  }

  __device__ void sync() { arrive_release(0, nullptr); }

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
    double* P = partials + (size_t)buf * gridDim.x * MINIM_WIDE;
    if (threadIdx.x < K) {
      double s = 0.0;
      for (int i = 0; i < nw; i++) s += red[i * MINIM_MAXRED + threadIdx.x];
      P[blockIdx.x * MINIM_WIDE + threadIdx.x] = s;
    }
    arrive_release(K, red + 32 * MINIM_MAXRED);
#pragma unroll
    for (int k = 0; k < K; k++) v[k] = red[32 * MINIM_MAXRED + k];
    __syncthreads();
  }

  __device__ __forceinline__ void wide_clear() { wide_clear_row(wide); }
  __device__ __forceinline__ void wide_store32(float (&v)[32], int k0) { wide_store_row(v, k0, wide); }
  __device__ void wide_combine(int K, double* out) {
    const int nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    double* P = partials + (size_t)buf * gridDim.x * MINIM_WIDE;
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
      double s = 0.0;
      for (int i = 0; i < nw; i++) s += wide[i * MINIM_WIDE + k];
      P[blockIdx.x * MINIM_WIDE + k] = s;
    }
    arrive_release(K, out);
  }
};

}  // namespace mg
