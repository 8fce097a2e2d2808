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
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "engine.h"

#define MINIM_MAXRED 8    // values reduced together in one team reduction
#define MINIM_NSTAGE 4    // shared-memory stages of a staged vector pass

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

// Accumulates a stream of FP32 terms with compensated (TwoSum) FP32
// arithmetic: the sum and its running rounding error together carry about
// 48 bits, and no per-term work touches the FP64 pipe, which on GB300 runs at
// 1/64 of the FP32 rate.  The order of additions is fixed, so results are
// deterministic.
struct Acc {
  float s, c;  // running sum and its rounding error (Neumaier / TwoSum, all FP32)
  double d;    // FP64 terms
  __device__ __forceinline__ Acc() : s(0.f), c(0.f), d(0.0) {}
  __device__ __forceinline__ void add(float v) {
    const float t = __fadd_rn(s, v);
    const float bp = __fsub_rn(t, s);
    c = __fadd_rn(c, __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(v, bp)));
    s = t;
  }
  __device__ __forceinline__ void add(double v) { d += v; }
  __device__ __forceinline__ double total() const { return d + ((double)s + (double)c); }
};

// Double-float numbers: an unevaluated sum hi + lo of two FP32 values with
// |lo| <= ulp(hi)/2, about 48 significant bits with the FP32 exponent range.
// Built on the error-free transformations of Knuth (TwoSum) and Dekker
// (Fast2Sum), with the product's error taken from one fused multiply-add;
// every operation is a handful of FP32 instructions instead of the FP64 pipe,
// which runs at 1/64 of the FP32 rate on GB300.  Compile-time rounding is
// explicit (__fadd_rn etc.) so that no contraction breaks the transformations.
struct DF {
  float hi, lo;
};
__device__ __forceinline__ DF df_fast2sum(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return DF{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ DF df_2sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return DF{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ DF df_from(double x) {
  const float hi = (float)x;
  return DF{hi, (float)(x - (double)hi)};
}
__device__ __forceinline__ DF df_from(float x) { return DF{x, 0.f}; }
__device__ __forceinline__ double df_to(DF a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ DF operator+(DF a, DF b) {
  const DF s = df_2sum(a.hi, b.hi);
  const DF t = df_2sum(a.lo, b.lo);
  const DF u = df_fast2sum(s.hi, __fadd_rn(s.lo, t.hi));
  return df_fast2sum(u.hi, __fadd_rn(u.lo, t.lo));
}
// The plain double-float sum: TwoSum of the high parts with the low parts
// added to its error -- error within a few units of 2^-46 of the operands'
// magnitudes (an FP64 sum's is within 2^-53 of its operands'), 11 FP32
// instructions against the cancellation-safe sum's 20.
__device__ __forceinline__ DF df_add_plain(DF a, DF b) {
  const DF s = df_2sum(a.hi, b.hi);
  return df_fast2sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ DF operator-(DF a) { return DF{-a.hi, -a.lo}; }
__device__ __forceinline__ DF operator-(DF a, DF b) { return a + (-b); }
__device__ __forceinline__ DF operator*(DF a, DF b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return df_fast2sum(p, e);
}
// 1 / x in FP32: the hardware approximation refined by one Newton-Raphson
// step, r' = r + r (1 - x r) (within an ulp or so; the correctly rounded
// reciprocal costs several times more)
__device__ __forceinline__ float rcp_nr(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return __fmaf_rn(r, __fmaf_rn(-x, r, 1.f), r);
}

// 1 / b: the FP32 reciprocal refined by one Newton step in double-float
__device__ __forceinline__ DF df_rcp(DF b) {
  const float y = rcp_nr(b.hi);
  const DF r = DF{1.f, 0.f} - b * DF{y, 0.f};  // residual 1 - b y
  return DF{y, 0.f} + DF{y, 0.f} * r;
}
// Split of a double into double-float by its bits (integer and FP32
// instructions only; the FP64 conversions it replaces run at the FP64 rate):
// hi is x with its mantissa cut to 24 bits, lo the remainder (29 bits) to
// FP32 rounding, about 47 bits in all.  Magnitudes outside [2^-70, 2^127)
// (and zero) take the converting split.
__device__ __forceinline__ DF df_split_bits(double x) {
  const long long b = __double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7ff);
  if (e < 1023 - 70 || e > 1023 + 126) return df_from(x);
  const unsigned long long m = (unsigned long long)b & 0xFFFFFFFFFFFFFULL;
  const unsigned sign = (unsigned)((unsigned long long)b >> 63) << 31;
  const float hi = __int_as_float((int)(sign | ((unsigned)(e - 1023 + 127) << 23) | (unsigned)(m >> 29)));
  const float scale = __int_as_float((int)((unsigned)(e - 1075 + 127) << 23));  // 2^(e - 1075)
  const float lo = __fmul_rn(__uint2float_rn((unsigned)(m & 0x1FFFFFFFULL)), scale);
  return DF{hi, sign ? -lo : lo};
}

// Double-float as a number type, for code written once for float / double /
// double-float arithmetic (the PhaseField and BarAndHinge FP64-stage
// sweeps): sums are the plain double-float sum, products the FMA product,
// division goes through the refined reciprocal; comparisons use the sign of
// the difference.
struct DFn {
  float hi, lo;
  DFn() = default;
  __device__ __forceinline__ DFn(DF a) : hi(a.hi), lo(a.lo) {}
  __device__ __forceinline__ DFn(float a) : hi(a), lo(0.f) {}
  __device__ __forceinline__ DFn(int a) : hi((float)a), lo(0.f) {}  // |a| < 2^24
  __device__ __forceinline__ DFn(double a) {
    const DF d = df_from(a);
    hi = d.hi;
    lo = d.lo;
  }
  __device__ __forceinline__ DF df() const { return DF{hi, lo}; }
  __device__ __forceinline__ explicit operator double() const { return (double)hi + (double)lo; }
  __device__ __forceinline__ explicit operator float() const { return __fadd_rn(hi, lo); }
};
__device__ __forceinline__ DFn operator+(DFn a, DFn b) { return DFn(df_add_plain(a.df(), b.df())); }
__device__ __forceinline__ DFn operator-(DFn a, DFn b) { return DFn(df_add_plain(a.df(), -b.df())); }
__device__ __forceinline__ DFn operator-(DFn a) { return DFn(DF{-a.hi, -a.lo}); }
__device__ __forceinline__ DFn operator*(DFn a, DFn b) { return DFn(a.df() * b.df()); }
__device__ __forceinline__ DF df_rcp(DF b);
__device__ __forceinline__ DFn operator/(DFn a, DFn b) { return DFn(a.df() * df_rcp(b.df())); }
__device__ __forceinline__ DFn& operator+=(DFn& a, DFn b) { return a = a + b; }
__device__ __forceinline__ DFn& operator-=(DFn& a, DFn b) { return a = a - b; }
__device__ __forceinline__ DFn& operator*=(DFn& a, DFn b) { return a = a * b; }
__device__ __forceinline__ bool operator<(DFn a, DFn b) { return (a - b).hi < 0.f; }
__device__ __forceinline__ bool operator>(DFn a, DFn b) { return (a - b).hi > 0.f; }
__device__ __forceinline__ bool operator<=(DFn a, DFn b) { return (a - b).hi <= 0.f; }
__device__ __forceinline__ bool operator>=(DFn a, DFn b) { return (a - b).hi >= 0.f; }
__device__ __forceinline__ bool operator==(DFn a, DFn b) { return (a - b).hi == 0.f; }
__device__ __forceinline__ bool operator!=(DFn a, DFn b) { return (a - b).hi != 0.f; }

__device__ __forceinline__ DF df_shfl(DF a, int src) {
  return DF{__shfl_sync(0xffffffffu, a.hi, src), __shfl_sync(0xffffffffu, a.lo, src)};
}

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

// L2 prefetch of the 128-byte line that holds float4 element i4 of p.  One
// lane in eight issues it (eight consecutive float4 share a line; callers
// keep i4 of lane 0 of each group a multiple of 8).  A prefetch holds no
// register, so the passes keep more bytes in flight than their loads alone.
__device__ __forceinline__ void prefetch_line(const float* p, int i4) {
  if ((threadIdx.x & 7) == 0) asm volatile("prefetch.global.L2 [%0];" ::"l"(p + 4 * (size_t)i4));
}

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// ---- compact-form L-BFGS algebra on one warp -----------------------------------
// Every lane of the calling warp takes part; lane k < mt holds pair k in age
// order (oldest first) with sg = s_k.g and yg = y_k.g.  Solves
//   R u = S^T g,   R^T w = (D + gamma Y^T Y) u - gamma Y^T g,
// R the upper triangle of S^T Y and D its diagonal, for the coefficients of
// P = -(gamma g + S w - gamma Y u): the direction the reference's two-loop
// recursion forms (src/minimisers/Lbfgs.cpp:60-105), in compact form.
// sy(a, b) = s_a.y_b and yy(a, b) = y_a.y_b in age order.  The triangular
// solves go column by column: once lane b holds its unknown it is broadcast
// and every lane still open subtracts its term, so the dependent chain per
// pair is one multiply and one FMA (FP64 runs at 1/64 of the FP32 rate on
// this GPU, with a long latency per dependent operation) instead of a row's
// dot product and a division; 1 / R[k][k] is formed once per lane.
template <class SYf, class YYf>
__device__ __forceinline__ void lbfgs_compact_warp(int mt, double gamma, double sg, double yg, SYf sy, YYf yy,
                                                   double& u_out, double& w_out) {
  const int lane = (threadIdx.y * blockDim.x + threadIdx.x) & 31;
  const bool on = lane < mt;
  const double r = on ? 1.0 / sy(lane, lane) : 0.0;
  double t = on ? sg : 0.0, u = 0.0;
  for (int b = mt - 1; b >= 0; b--) {
    const double ub = __shfl_sync(0xffffffffu, t * r, b);
    if (lane == b) u = ub;
    else if (lane < b) t -= sy(lane, b) * ub;
  }
  double v = on ? sy(lane, lane) * u - gamma * yg : 0.0;
  for (int b = 0; b < mt; b++) {
    const double ub = __shfl_sync(0xffffffffu, u, b);
    if (on) v += gamma * yy(lane, b) * ub;
  }
  double w = 0.0;
  t = v;
  for (int b = 0; b < mt; b++) {
    const double wb = __shfl_sync(0xffffffffu, t * r, b);
    if (lane == b) w = wb;
    else if (on && lane > b) t -= sy(b, lane) * wb;
  }
  u_out = u;
  w_out = w;
}

// slot of pair k (age order) of the m-slot ring whose next slot is c, with
// mt pairs stored: (c - mt + k) mod m
__device__ __forceinline__ int ring_slot(int c, int mt, int k, int m) {
  const int s = c - mt + k;
  return s < 0 ? s + m : s;
}

// ---- bulk copies into shared memory (cp.async.bulk + mbarrier) -----------------
// A stage is a shared buffer with an mbarrier.  One thread announces the
// bytes the stage will receive (arrive.expect_tx) and issues the copies; the
// mbarrier's phase completes when all bytes have landed, and every thread
// waits on that phase before reading.  Addresses and sizes are multiples of
// 16 bytes.
__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void proxy_async_fence() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// The spin itself carries no memory clobber (nothing the compiler holds in
// registers is reloaded per poll); a compiler fence after the loop keeps the
// reads of the landed data below the wait, whose acquire makes them visible.
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity));
  return ok != 0;
}
// Bounded wait for the given phase parity (false after `limit_ns`).
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity,
                                          unsigned long long limit_ns) {
  bool ok = true;
  if (!mbar_try_wait(bar, parity)) {
    const unsigned long long t0 = globaltimer_ns();
    while (!mbar_try_wait(bar, parity)) {
      if (globaltimer_ns() - t0 > limit_ns) {
        ok = false;
        break;
      }
    }
  }
  asm volatile("" ::: "memory");
  return ok;
}

// A ring of MINIM_NSTAGE shared stages streaming chunks of nv vectors into a
// block: each stage has a "full" mbarrier (the chunk's bytes have landed)
// and an "empty" one (every warp is done with it).  The block's chunks are
// cidx = blockIdx.x + j * gridDim.x; a chunk holds `ch` floats of each
// vector.  Thread 0 fills the ring ahead; warp 0, after releasing chunk j,
// waits until all warps have, and refills that stage with chunk j +
// MINIM_NSTAGE, so warps never wait on one another except through the data.
// Uses are numbered per launch (sq), which fixes the barriers' phase
// parities.  All state lives in registers (no member access through memory).
struct StageRing {
  char* base;                 // shared: MINIM_NSTAGE stages of stage_bytes
  unsigned long long* full;   // shared mbarriers
  unsigned long long* empty;
  int* err;                   // shared: a wait gave up
  int stage_bytes, n, ch, nv, mine, j, issued;
  unsigned sq;

  __device__ __forceinline__ float* buf(int s) const {
    return reinterpret_cast<float*>(base + (size_t)s * stage_bytes);
  }
  template <class VecFn>
  __device__ __forceinline__ void issue(int s, int cidx, VecFn vec) const {
    const int i0 = cidx * ch;
    const int cnt = min(ch, n - i0);
    const unsigned bytes = (unsigned)((cnt * 4 + 15) & ~15);
    float* dst = buf(s);
    proxy_async_fence();
    mbar_expect_tx(&full[s], bytes * (unsigned)nv);
    for (int v = 0; v < nv; v++) bulk_g2s(dst + (size_t)v * ch, vec(v) + i0, bytes, &full[s]);
  }
  // all threads; `ok` false skips the sweep
  template <class VecFn>
  __device__ __forceinline__ void begin(bool ok, VecFn vec) {
    const int nch = (n + ch - 1) / ch;
    mine = ok && (int)blockIdx.x < nch ? (nch - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    j = 0;
    issued = 0;
    if (threadIdx.x == 0) {
      *err = 0;
      for (; issued < min(MINIM_NSTAGE, mine); issued++)
        issue((sq + issued) % MINIM_NSTAGE, blockIdx.x + issued * gridDim.x, vec);
    }
    __syncthreads();
  }
  __device__ __forceinline__ int i0() const { return ((int)blockIdx.x + j * (int)gridDim.x) * ch; }
  __device__ __forceinline__ int count() const { return min(ch, n - i0()); }
  // wait for chunk j; null if the block must stop
  __device__ __forceinline__ const float* acquire() {
    const unsigned u = sq + (unsigned)j;
    if (*(volatile int*)err) return nullptr;
    if (!mbar_wait(&full[u % MINIM_NSTAGE], (u / MINIM_NSTAGE) & 1u, 5000000000ull)) {
      *(volatile int*)err = 1;
      return nullptr;
    }
    return buf(u % MINIM_NSTAGE);
  }
  template <class VecFn>
  __device__ __forceinline__ void release(VecFn vec) {
    const unsigned u = sq + (unsigned)j;
    const int s = u % MINIM_NSTAGE;
    __syncwarp();
    if ((threadIdx.x & 31) == 0) mbar_arrive(&empty[s]);
    if (threadIdx.x < 32 && j + MINIM_NSTAGE < mine) {
      const bool ok = mbar_wait(&empty[s], (u / MINIM_NSTAGE) & 1u, 5000000000ull);
      if (threadIdx.x == 0) {
        if (ok) {
          issue(s, blockIdx.x + (j + MINIM_NSTAGE) * gridDim.x, vec);
          issued++;
        } else {
          *(volatile int*)err = 1;
        }
      }
      __syncwarp();
    }
    j++;
  }
  // all threads, after the loop; false if a wait gave up (the copies still
  // in flight have been given bounded time to land)
  __device__ __forceinline__ bool end() {
    __syncthreads();
    const bool bad = *(volatile int*)err != 0;
    if (bad && threadIdx.x == 0)
      for (int k = 0; k < issued; k++) {
        const unsigned u = sq + (unsigned)k;
        mbar_wait(&full[u % MINIM_NSTAGE], (u / MINIM_NSTAGE) & 1u, 5000000000ull);
      }
    sq += (unsigned)mine;
    return !bad;
  }
};

// ---------------------------------------------------------------------------
// Team = one CTA
// ---------------------------------------------------------------------------
// Sum of two compensated FP32 partial sums (s, c): TwoSum of the running
// sums, errors added (the combination Acc::add uses).  Symmetric in its
// arguments, so both lanes of a butterfly exchange get the same result.
__device__ __forceinline__ void pair_add(float& s, float& c, float s2, float c2) {
  const float t = __fadd_rn(s, s2);
  const float bp = __fsub_rn(t, s);
  const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(s2, bp));
  c = __fadd_rn(__fadd_rn(c, c2), err);
  s = t;
}
__device__ __forceinline__ void warp_pair_sum(float& s, float& c) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const float s2 = __shfl_xor_sync(0xffffffffu, s, off), c2 = __shfl_xor_sync(0xffffffffu, c, off);
    pair_add(s, c, s2, c2);
  }
}
// A double as such a pair (exact for the sum of an Acc's two floats)
__device__ __forceinline__ void to_pair(double v, float& s, float& c) {
  s = (float)v;
  c = (float)(v - (double)s);
}
struct NoPost {
  __device__ void operator()(double*) const {}
};

// Anneal's random numbers: SplitMix64's output mix (Steele, Lea and Flood
// 2014) applied twice to a counter of (iteration, coordinate index), keyed by
// the seed; the top 53 bits give u in [0, 1).  Stateless, so every thread
// draws its own coordinates' numbers in any order.
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}
__device__ __forceinline__ double anneal_unit(unsigned long long seed, int iter, unsigned idx) {
  const unsigned long long h = mix64(seed ^ mix64(((unsigned long long)(unsigned)iter << 32) | idx));
  return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

struct CtaTeam {
  // thread index and count come from special registers, never from memory
  __device__ __forceinline__ int tid() const { return threadIdx.x; }
  __device__ __forceinline__ int nthr() const { return blockDim.x; }
  double* red;  // shared scratch, >= (32 + 1) * MINIM_MAXRED doubles
  double* wide; // shared scratch, one row of MINIM_WIDE doubles per warp
  static constexpr bool kGrid = false;
  static constexpr bool kCluster = false;
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

  // The team sums of K compensated FP32 partials (s[k], c[k]) with FP32
  // butterflies inside the warps; warp 0 alone forms the FP64 totals over the
  // warps (fixed order), and its thread 0 runs post(totals) to append D
  // derived values (e.g. square roots), so that no other warp issues an FP64
  // instruction.  out[0..K+D) receives totals and derived values.
  template <int K, int D = 0, class Post = NoPost>
  __device__ void reduce_pairs(float (&s)[K], float (&c)[K], double (&out)[K + D], Post post = Post{}) {
    static_assert(K + D <= MINIM_MAXRED, "too many values");
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    float* rf = reinterpret_cast<float*>(red);  // [warp][2K] floats, before the totals
    double* tot = red + 32 * MINIM_MAXRED;
#pragma unroll
    for (int k = 0; k < K; k++) warp_pair_sum(s[k], c[k]);
    if (lane == 0) {
#pragma unroll
      for (int k = 0; k < K; k++) {
        rf[w * 2 * MINIM_MAXRED + 2 * k] = s[k];
        rf[w * 2 * MINIM_MAXRED + 2 * k + 1] = c[k];
      }
    }
    __syncthreads();
    if (threadIdx.x < 32) {
      if (lane < K) {
        double t = 0.0;
        for (int i = 0; i < nw; i++)
          t += (double)rf[i * 2 * MINIM_MAXRED + 2 * lane] + (double)rf[i * 2 * MINIM_MAXRED + 2 * lane + 1];
        tot[lane] = t;
      }
      __syncwarp();
      if (lane == 0) post(tot);
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K + D; k++) out[k] = tot[k];
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

struct D4q {
  double x, y, z, w;
};

// Sums column k < K (<= 64) of G rows of MINIM_WIDE doubles (row b at
// P + b * MINIM_WIDE) in row order into out[k], with every thread of the
// block: one double4 load per (row, 4 columns) spread over the threads (all
// issued at once), butterflies across the lanes that share a column, then a
// fixed-order sum over warps through `wide` (8 * MINIM_WIDE doubles of
// scratch).  Deterministic: the order depends only on G, K and blockDim.
__device__ inline void sum_rows_fixed(const double* P, int G, int K, double* out, double* wide) {
  const int nq = (K + 3) >> 2;  // double4 columns
  // linear thread index (the block may be 2-D; it holds whole warps)
  const int tl = threadIdx.y * blockDim.x + threadIdx.x, nt = blockDim.x * blockDim.y;
  const int lane = tl & 31, w = tl >> 5, nw = (nt + 31) >> 5;
  const int nqp = nq <= 1 ? 1 : nq <= 2 ? 2 : nq <= 4 ? 4 : nq <= 8 ? 8 : 16;
  const int q = tl & (nqp - 1);
  const int r0 = tl / nqp, rs = nt / nqp;
  // four consecutive partials of row b (L2, 2 x 16-byte loads)
  auto ld = [&](int b) {
    const double2* r = reinterpret_cast<const double2*>(P + (size_t)b * MINIM_WIDE) + 2 * q;
    const double2 lo = __ldcg(r), hi = __ldcg(r + 1);
    return D4q{lo.x, lo.y, hi.x, hi.y};
  };
  D4q acc{0.0, 0.0, 0.0, 0.0};
  if (q < nq) {
    // four rows per step, all loads issued before the adds (rows past G
    // read as zero), so that up to 4 * rs rows cost one L2 round trip
    const D4q z{0.0, 0.0, 0.0, 0.0};
    for (int b = r0; b < G; b += 4 * rs) {
      const D4q v0 = ld(b);
      const D4q v1 = b + rs < G ? ld(b + rs) : z;
      const D4q v2 = b + 2 * rs < G ? ld(b + 2 * rs) : z;
      const D4q v3 = b + 3 * rs < G ? ld(b + 3 * rs) : z;
      acc.x += v0.x; acc.y += v0.y; acc.z += v0.z; acc.w += v0.w;
      acc.x += v1.x; acc.y += v1.y; acc.z += v1.z; acc.w += v1.w;
      acc.x += v2.x; acc.y += v2.y; acc.z += v2.z; acc.w += v2.w;
      acc.x += v3.x; acc.y += v3.y; acc.z += v3.z; acc.w += v3.w;
    }
  }
  for (int off = 16; off >= nqp; off >>= 1) {
    acc.x += __shfl_xor_sync(0xffffffffu, acc.x, off);
    acc.y += __shfl_xor_sync(0xffffffffu, acc.y, off);
    acc.z += __shfl_xor_sync(0xffffffffu, acc.z, off);
    acc.w += __shfl_xor_sync(0xffffffffu, acc.w, off);
  }
  // columns of warp w: lanes 0 .. min(nqp, 32) - 1 (nqp <= 16)
  if (lane < nqp && q < nq) {
    double* d = wide + (size_t)w * MINIM_WIDE + 4 * q;
    d[0] = acc.x; d[1] = acc.y; d[2] = acc.z; d[3] = acc.w;
  }
  __syncthreads();
  for (int k = tl; k < K; k += nt) {
    if (nw <= 8) {  // the warps' sums as a pairwise tree (short FP64 add chain)
      double t[8];
#pragma unroll
      for (int i = 0; i < 8; i++) t[i] = i < nw ? wide[i * MINIM_WIDE + k] : 0.0;
      out[k] = ((t[0] + t[1]) + (t[2] + t[3])) + ((t[4] + t[5]) + (t[6] + t[7]));
    } else {
      double t = 0.0;
      for (int i = 0; i < nw; i++) t += wide[i * MINIM_WIDE + k];
      out[k] = t;
    }
  }
}

// ---------------------------------------------------------------------------
// Team = whole grid (cooperative launch), with a bounded software barrier
// ---------------------------------------------------------------------------
struct GridTeam {
  __device__ __forceinline__ int tid() const { return blockIdx.x * blockDim.x + threadIdx.x; }
  __device__ __forceinline__ int nthr() const { return gridDim.x * blockDim.x; }
  double* red;            // shared scratch as in CtaTeam
  double* wide;           // shared scratch as in CtaTeam
  GridSyncState* bar;     // global
  double* partials;       // global: 2 * gridDim.x * MINIM_WIDE partials (double-buffered rows)
  int buf;                // partials double buffer index
  int* s_ok;              // shared flag
  unsigned int epoch;     // barriers passed in this launch (uniform)
  static constexpr bool kGrid = true;
  static constexpr bool kCluster = false;
  static constexpr unsigned long long kWaitLimitNs = 5000000000ull;  // 5 s

  __device__ __forceinline__ bool block0() const { return blockIdx.x == 0; }
  __device__ __forceinline__ bool ok() const { return *s_ok != 0; }
  __device__ __forceinline__ unsigned long long wait_limit_ns() const {
    const unsigned int ms = bar->limit_ms;
    return ms ? (unsigned long long)ms * 1000000ull : kWaitLimitNs;
  }
  // records a failed wait: this block stops, the others stop at their next
  // barrier (status TIMEOUT)
  __device__ void fail() {
    if (threadIdx.x == 0) {
      atomicExch(&bar->err, 1);
      *s_ok = 0;
    }
  }

  // Bounded wait until the arrival counter reaches `want` (or an error was
  // recorded by any block).
  __device__ bool wait_count(unsigned int want) {
    unsigned long long t0 = 0;
    for (;;) {
      unsigned int c;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(c) : "l"(&bar->count) : "memory");
      if (c >= want) return true;
      if (*(volatile int*)&bar->err) return false;
      const unsigned long long t = globaltimer_ns();
      if (t0 == 0) {
        t0 = t;
      } else if (t - t0 > wait_limit_ns()) {
        atomicExch(&bar->err, 1);
        return false;
      }
      __nanosleep(20);
    }
  }

  // Every block sums the K (<= 64) partials of all blocks' rows in block
  // order (sum_rows_fixed), so all blocks hold bitwise the same totals
  // without a second round trip; `wide` is free during barriers.
  __device__ void sum_rows(const double* P, int K, double* out) { sum_rows_fixed(P, gridDim.x, K, out, wide); }

  // Counter barrier with an optional reduction.  Every block adds 1 to the
  // launch's arrival counter after its partials are written (fence, then a
  // fire-and-forget atomic), waits until all blocks have arrived at this
  // barrier (epoch * gridDim.x arrivals), and then sums every block's K
  // partials itself.  Every wait is bounded (kWaitLimitNs): a block that
  // gives up records an error; later barriers see it and return at once, so
  // the kernel always finishes (status TIMEOUT).
  __device__ void arrive_release(int K, double* out) {
    const double* P = partials + (size_t)buf * gridDim.x * MINIM_WIDE;
    const unsigned int ep = ++epoch;
    __syncthreads();
    if (threadIdx.x == 0 && *s_ok) {
      __threadfence();
      atomicAdd(&bar->count, 1u);
      if (!wait_count(ep * gridDim.x)) *s_ok = 0;
      __threadfence();
    }
    __syncthreads();
    if (*s_ok && K > 0) sum_rows(P, K, out);
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

  // As CtaTeam::reduce_pairs: the block's sums from FP32 butterflies and warp
  // 0, the grid's from every block's partial row (fixed order), then post in
  // thread 0 of every block (all blocks hold the same totals).
  template <int K, int D = 0, class Post = NoPost>
  __device__ void reduce_pairs(float (&s)[K], float (&c)[K], double (&out)[K + D], Post post = Post{}) {
    static_assert(K + D <= MINIM_MAXRED, "too many values");
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    float* rf = reinterpret_cast<float*>(red);
    double* tot = red + 32 * MINIM_MAXRED;
#pragma unroll
    for (int k = 0; k < K; k++) warp_pair_sum(s[k], c[k]);
    if (lane == 0) {
#pragma unroll
      for (int k = 0; k < K; k++) {
        rf[w * 2 * MINIM_MAXRED + 2 * k] = s[k];
        rf[w * 2 * MINIM_MAXRED + 2 * k + 1] = c[k];
      }
    }
    __syncthreads();
    double* P = partials + (size_t)buf * gridDim.x * MINIM_WIDE;
    if (threadIdx.x < K) {
      double t = 0.0;
      for (int i = 0; i < nw; i++)
        t += (double)rf[i * 2 * MINIM_MAXRED + 2 * threadIdx.x] + (double)rf[i * 2 * MINIM_MAXRED + 2 * threadIdx.x + 1];
      P[blockIdx.x * MINIM_WIDE + threadIdx.x] = t;
    }
    arrive_release(K, tot);
    if (threadIdx.x == 0) post(tot);
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K + D; k++) out[k] = tot[k];
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

// ---------------------------------------------------------------------------
// Team = a thread-block cluster (one instance on several SMs of the batch
// path).  Barriers are the cluster's hardware barrier (every thread of every
// CTA, release / acquire at cluster scope); a reduction writes each CTA's
// totals to its own shared-memory row and every CTA then reads all rows
// through distributed shared memory in rank order, so every CTA holds
// bitwise the same totals and takes the same branches.  Rows are
// double-buffered: a CTA writes a row again only after the next barrier,
// which every reader of the previous use has passed.
// ---------------------------------------------------------------------------
struct ClusterTeam {
  double* red;   // per-CTA shared scratch as in CtaTeam
  double* wide;  // per-CTA shared scratch as in CtaTeam
  double* xch;   // per-CTA shared exchange rows: 2 x MINIM_WIDE doubles
  int buf;       // exchange row in use
  static constexpr bool kGrid = true;      // a multi-CTA team: team-generic kernels
  static constexpr bool kCluster = true;
  __device__ __forceinline__ int rank() const { return (int)cooperative_groups::this_cluster().block_rank(); }
  __device__ __forceinline__ int csize() const { return (int)cooperative_groups::this_cluster().num_blocks(); }
  __device__ __forceinline__ int tid() const { return rank() * blockDim.x + threadIdx.x; }
  __device__ __forceinline__ int nthr() const { return csize() * blockDim.x; }
  __device__ __forceinline__ void sync() { cooperative_groups::this_cluster().sync(); }
  __device__ __forceinline__ bool ok() const { return true; }
  __device__ __forceinline__ bool block0() const { return rank() == 0; }
  __device__ __forceinline__ void fail() {}

  // this CTA's K totals are in xch row `buf`: the cluster's totals (rank
  // order) into out (this CTA's shared memory)
  __device__ void exchange(int K, double* out) {
    auto cl = cooperative_groups::this_cluster();
    cl.sync();
    const int nc = (int)cl.num_blocks();
    double* row = xch + buf * MINIM_WIDE;
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
      double s = 0.0;
      for (int r = 0; r < nc; r++) s += cl.map_shared_rank(row, r)[k];
      out[k] = s;
    }
    buf ^= 1;
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
    if (threadIdx.x < K) {
      double s = 0.0;
      for (int i = 0; i < nw; i++) s += red[i * MINIM_MAXRED + threadIdx.x];
      xch[buf * MINIM_WIDE + threadIdx.x] = s;
    }
    exchange(K, red + 32 * MINIM_MAXRED);
#pragma unroll
    for (int k = 0; k < K; k++) v[k] = red[32 * MINIM_MAXRED + k];
    __syncthreads();
  }

  // As CtaTeam::reduce_pairs within each CTA, then the CTAs' FP64 totals
  // summed in rank order; post in thread 0 of every CTA.
  template <int K, int D = 0, class Post = NoPost>
  __device__ void reduce_pairs(float (&s)[K], float (&c)[K], double (&out)[K + D], Post post = Post{}) {
    static_assert(K + D <= MINIM_MAXRED, "too many values");
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    float* rf = reinterpret_cast<float*>(red);
    double* tot = red + 32 * MINIM_MAXRED;
#pragma unroll
    for (int k = 0; k < K; k++) warp_pair_sum(s[k], c[k]);
    if (lane == 0) {
#pragma unroll
      for (int k = 0; k < K; k++) {
        rf[w * 2 * MINIM_MAXRED + 2 * k] = s[k];
        rf[w * 2 * MINIM_MAXRED + 2 * k + 1] = c[k];
      }
    }
    __syncthreads();
    if (threadIdx.x < K) {
      double t = 0.0;
      for (int i = 0; i < nw; i++)
        t += (double)rf[i * 2 * MINIM_MAXRED + 2 * threadIdx.x] + (double)rf[i * 2 * MINIM_MAXRED + 2 * threadIdx.x + 1];
      xch[buf * MINIM_WIDE + threadIdx.x] = t;
    }
    exchange(K, tot);
    if (threadIdx.x == 0) post(tot);
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K + D; k++) out[k] = tot[k];
    __syncthreads();
  }

  __device__ __forceinline__ void wide_clear() { wide_clear_row(wide); }
  __device__ __forceinline__ void wide_store32(float (&v)[32], int k0) { wide_store_row(v, k0, wide); }
  __device__ void wide_combine(int K, double* out) {
    const int nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
      double s = 0.0;
      for (int i = 0; i < nw; i++) s += wide[i * MINIM_WIDE + k];
      xch[buf * MINIM_WIDE + k] = s;
    }
    exchange(K, out);
  }
};

}  // namespace mg
