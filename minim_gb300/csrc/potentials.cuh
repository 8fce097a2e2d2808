// potentials.cuh -- device energy/gradient of LjNd, PhaseField and BarAndHinge.
//
// Each evaluator is a template over the coordinate type T (float for the FP32
// stage, double for the FP64 stage and the FP64 API call) and the team.  The
// coordinates are read through a CView (x + t*p, so line-search trial points
// are never materialised), optionally written out (the accepted point), and
// the gradient is handed DOF by DOF to an Emit functor exactly once per DOF.
// The return value is the calling thread's share of the energy.
#pragma once
#include "common.cuh"

namespace mg {

// coordinates x + t * p (p may be NULL); one rounding, the same everywhere
template <typename T>
struct CView {
  const T* x;
  const float* p;
  T t;
  __device__ __forceinline__ T operator()(int i) const;
};
template <>
__device__ __forceinline__ float CView<float>::operator()(int i) const {
  return p ? __fadd_rn(x[i], __fmul_rn(t, p[i])) : x[i];
}
template <>
__device__ __forceinline__ double CView<double>::operator()(int i) const {
  return p ? __dadd_rn(x[i], __dmul_rn(t, (double)p[i])) : x[i];
}

template <typename T> struct EAcc;
template <> struct EAcc<float> {
  Acc a;
  __device__ __forceinline__ void add(float v) { a.add(v); }
  __device__ __forceinline__ double total() const { return a.total(); }
};
template <> struct EAcc<double> {
  double d = 0.0;
  __device__ __forceinline__ void add(double v) { d += v; }
  __device__ __forceinline__ double total() const { return d; }
};
template <> struct EAcc<DFn> {
  DFn s = DFn(0);
  __device__ __forceinline__ void add(DFn v) { s += v; }
  __device__ __forceinline__ double total() const { return (double)s; }
};

struct NoEmit {
  template <typename T>
  __device__ __forceinline__ void operator()(int, T) {}
};

// ===========================================================================
// LjNd: all i<j pairs (src/potentials/LjNd.cpp:12-53).  Each thread owns
// particles i and sums the force from every j (no scatter, deterministic);
// the energy counts each pair once (j > i).  Coordinates are staged through
// shared memory in tiles.
// ===========================================================================
struct alignas(16) F4 { float x, y, z, w; };
struct alignas(16) D4 { double x, y, z, w; };

// Double-float for the Lennard-Jones pair terms: the DF representation with
// the cheaper operations that suffice there.  A sum is TwoSum of the high
// parts with the low parts added to its error (11 FP32 instructions instead
// of the cancellation-safe form's 20); its error is bounded by a few units
// of 2^-46 of the operands' magnitudes, as an FP64 sum's is by 2^-53 of
// theirs, and every force and energy the pair code sums is compared with
// operands of its own size.  The reciprocal takes its Newton residual
// 1 - b y from one fused multiply-add (b.hi y is within 2^-22 of 1, so the
// residual is formed to FP32 relative accuracy) and the low part's product.
struct DFl {
  float hi, lo;
};
__device__ __forceinline__ DFl dfl(DF a) { return DFl{a.hi, a.lo}; }
__device__ __forceinline__ DFl operator+(DFl a, DFl b) { return dfl(df_add_plain(DF{a.hi, a.lo}, DF{b.hi, b.lo})); }
__device__ __forceinline__ DFl operator-(DFl a) { return DFl{-a.hi, -a.lo}; }
__device__ __forceinline__ DFl operator-(DFl a, DFl b) { return a + (-b); }
__device__ __forceinline__ DFl operator*(DFl a, DFl b) { return dfl(DF{a.hi, a.lo} * DF{b.hi, b.lo}); }
__device__ __forceinline__ DFl dfl_rcp(DFl b) {
  const float y = rcp_nr(b.hi);
  const float r = __fmaf_rn(-b.lo, y, __fmaf_rn(-b.hi, y, 1.f));  // 1 - b y
  const DF q = df_fast2sum(y, __fmul_rn(y, r));
  return DFl{q.hi, q.lo};
}
__device__ __forceinline__ double dfl_to(DFl a) { return (double)a.hi + (double)a.lo; }

// Pair arithmetic type: FP32 in the FP32 stage; double-float (DFl, about 46
// bits) in the FP64 stage and the FP64 API evaluation -- the O(N^2) pair
// terms stay off the FP64 pipe.  A pair closer than r^2 = 1e-5 sigma^2 (where
// FP32's exponent range could overflow lj12) is computed in double.
template <typename T> struct LjC;
template <> struct LjC<float> {
  using C = float;
  __device__ static C from(float x) { return x; }
  __device__ static double to(C x) { return (double)x; }
  __device__ static float scaled(double c, C x) { return (float)c * x; }  // no FP64 per DOF
};
template <> struct LjC<double> {
  using C = DFl;
  __device__ static C from(double x) { return dfl(df_from(x)); }
  __device__ static double to(C x) { return dfl_to(x); }
  __device__ static double scaled(double c, C x) { return c * dfl_to(x); }
};
template <typename C> struct CV3 { C x, y, z; };

__device__ __forceinline__ float lj_shfl(float a, int src) { return __shfl_sync(0xffffffffu, a, src); }
__device__ __forceinline__ DFl lj_shfl(DFl a, int src) { return dfl(df_shfl(DF{a.hi, a.lo}, src)); }

// lj6 = s6 / r^6, lj12 = lj6^2 and the force factor f = (2 lj12 - lj6) / r^2
// of one pair separated by (dx, dy, dz)
__device__ __forceinline__ void lj_pair(float dx, float dy, float dz, float s6, float& lj6, float& lj12,
                                        float& f) {
  const float inv = rcp_nr(dx * dx + dy * dy + dz * dz);
  lj6 = s6 * inv * inv * inv;
  lj12 = lj6 * lj6;
  f = (lj12 + lj12 - lj6) * inv;
}
__device__ __forceinline__ void lj_pair(DFl dx, DFl dy, DFl dz, DFl s6, DFl& lj6, DFl& lj12, DFl& f) {
  const DFl r2 = dx * dx + dy * dy + dz * dz;
  if (r2.hi >= 1e-5f) {
    const DFl inv = dfl_rcp(r2);
    const DFl inv3 = inv * inv * inv;
    lj6 = s6 * inv3;
    lj12 = lj6 * lj6;
    // 2 lj12 exactly (both parts doubled)
    f = (DFl{2.f * lj12.hi, 2.f * lj12.lo} - lj6) * inv;
  } else {
    const double ddx = dfl_to(dx), ddy = dfl_to(dy), ddz = dfl_to(dz);
    const double inv = 1.0 / (ddx * ddx + ddy * ddy + ddz * ddz);
    const double l6 = dfl_to(s6) * inv * inv * inv, l12 = l6 * l6;
    lj6 = dfl(df_from(l6));
    lj12 = dfl(df_from(l12));
    f = dfl(df_from((2 * l12 - l6) * inv));
  }
}

// energy accumulator of the pair type
template <typename C> struct LjAcc;
template <> struct LjAcc<float> {
  Acc a;
  __device__ __forceinline__ void add(float v) { a.add(v); }
  __device__ __forceinline__ double total() const { return a.total(); }
};
template <> struct LjAcc<DFl> {
  DFl s{0.f, 0.f};
  __device__ __forceinline__ void add(DFl v) { s = s + v; }
  __device__ __forceinline__ double total() const { return dfl_to(s); }
};

template <typename T, class Team, class Emit>
__device__ __noinline__ double lj_eval(Team& tm, const PotLJ& P, CView<T> cv, T* xw, Emit* emp,
                                       bool want_e, bool want_g, void* smem, int tile) {
  using L = LjC<T>;
  using C = typename L::C;
  Emit emit = *emp;
  CV3<C>* sx = reinterpret_cast<CV3<C>*>(smem);
  const int N = P.np, nd = P.ndim;
  const C s6 = L::from((T)P.s6);
  const C zero = L::from((T)0);
  if (xw) {
    for (int i = tm.tid(); i < N * nd; i += tm.nthr()) xw[i] = cv(i);
  }
  LjAcc<C> e4[4];
  const int step = tm.nthr();
  // every thread of every block runs the same number of outer rounds
  const int rounds = (N + step - 1) / step;
  for (int r = 0; r < rounds; r++) {
    const int i = r * step + tm.tid();
    const bool act = i < N;
    C xi = zero, yi = zero, zi = zero;
    if (act) {
      xi = L::from(cv(nd * i));
      yi = L::from(cv(nd * i + 1));
      zi = (nd == 3) ? L::from(cv(nd * i + 2)) : zero;
    }
    C fx = zero, fy = zero, fz = zero;
    for (int j0 = 0; j0 < N; j0 += tile) {
      const int nt = min(tile, N - j0);
      __syncthreads();
      for (int j = threadIdx.x; j < nt; j += blockDim.x) {
        const int jj = j0 + j;
        CV3<C> v;
        v.x = L::from(cv(nd * jj));
        v.y = L::from(cv(nd * jj + 1));
        v.z = (nd == 3) ? L::from(cv(nd * jj + 2)) : zero;
        sx[j] = v;
      }
      __syncthreads();
      if (act) {
        // pair energies go to four compensated accumulators in turn (four
        // short dependent chains instead of one long one)
        if (want_g) {
#pragma unroll 4
          for (int j = 0; j < nt; j++) {
            if (j0 + j == i) continue;
            const CV3<C> b = sx[j];
            const C dx = xi - b.x, dy = yi - b.y, dz = zi - b.z;
            C lj6, lj12, f;
            lj_pair(dx, dy, dz, s6, lj6, lj12, f);
            fx = fx + dx * f;
            fy = fy + dy * f;
            fz = fz + dz * f;
            if (want_e && (j0 + j > i)) e4[j & 3].add(lj12 - lj6);
          }
        } else if (want_e) {
#pragma unroll 4
          for (int j = max(0, i + 1 - j0); j < nt; j++) {
            const CV3<C> b = sx[j];
            const C dx = xi - b.x, dy = yi - b.y, dz = zi - b.z;
            C lj6, lj12, f;
            lj_pair(dx, dy, dz, s6, lj6, lj12, f);
            e4[j & 3].add(lj12 - lj6);
          }
        }
      }
    }
    if (act && want_g) {
      const double c = -24.0 * P.eps;
      emit(nd * i, L::scaled(c, fx));
      emit(nd * i + 1, L::scaled(c, fy));
      if (nd == 3) emit(nd * i + 2, L::scaled(c, fz));
    }
  }
  __syncthreads();
  *emp = emit;
  return 4.0 * P.eps * ((e4[0].total() + e4[1].total()) + (e4[2].total() + e4[3].total()));
}

}  // namespace mg
#include "ljcells.cuh"
namespace mg {

// Energy only, for one CTA (the batched path's line-search trials): each
// unordered pair once, 32x32 tile pairs (I <= J) dealt to the warps in turn
// -- no forces, so no rounds and no barriers, and every warp gets the same
// number of pairs whatever N (a thread per particle over j > i leaves the
// first threads with N pairs and the last with none).  Diagonal tiles count
// every pair twice at half weight; pairs with padding particles are skipped.
template <typename T>
__device__ __noinline__ double lj_energy_sym(CtaTeam& tm, const PotLJ& P, CView<T> cv, void* smem) {
  using L = LjC<T>;
  using C = typename L::C;
  const int N = P.np, nd = P.ndim;
  const int nt = (N + 31) >> 5;
  CV3<C>* sx = reinterpret_cast<CV3<C>*>(smem);
  const C s6 = L::from((T)P.s6);
  const C zero = L::from((T)0);
  const C half = L::from((T)0.5);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int j = threadIdx.x; j < 32 * nt; j += blockDim.x) {
    CV3<C> v;
    if (j < N) {
      v.x = L::from(cv(nd * j));
      v.y = L::from(cv(nd * j + 1));
      v.z = (nd == 3) ? L::from(cv(nd * j + 2)) : zero;
    } else {
      v.x = L::from((T)(1e6 * (double)(j + 1)));
      v.y = zero;
      v.z = zero;
    }
    sx[j] = v;
  }
  __syncthreads();
  LjAcc<C> e;
  const int npairs = nt * (nt + 1) / 2;
  for (int p = w; p < npairs; p += nw) {
    // (I, J), I <= J, row by row of the upper triangle
    int I = 0, rem = p;
    while (rem >= nt - I) {
      rem -= nt - I;
      I++;
    }
    const int J = I + rem;
    const int i = 32 * I + lane;
    const CV3<C> a = sx[i];
    C ee = zero;
    if (I == J) {
#pragma unroll 4
      for (int s = 1; s < 32; s++) {
        const int j = 32 * I + ((lane + s) & 31);
        const CV3<C> b = sx[j];
        const C dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
        C lj6, lj12, f;
        lj_pair(dx, dy, dz, s6, lj6, lj12, f);
        if (j < N) ee = ee + (lj12 - lj6);
      }
      if (i < N) e.add(ee * half);
    } else {
#pragma unroll 4
      for (int s = 0; s < 32; s++) {
        const int j = 32 * J + ((lane + s) & 31);
        const CV3<C> b = sx[j];
        const C dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
        C lj6, lj12, f;
        lj_pair(dx, dy, dz, s6, lj6, lj12, f);
        if (j < N) ee = ee + (lj12 - lj6);
      }
      if (i < N) e.add(ee);
    }
  }
  __syncthreads();
  return 4.0 * P.eps * e.total();
}

// FP32 energy and gradient for one CTA without rounds: each unordered pair
// once, the tile pairs (I <= J) dealt to the warps in turn as in
// lj_energy_sym, every warp adding its pairs' forces to its own
// shared-memory accumulators (no two warps write one accumulator, so no
// barrier between tile pairs and no warp idles while others finish a round),
// then one fixed-order sum over the warps per particle.  Within a tile pair
// the j tile's positions and forces rotate through the lanes with shuffles,
// as in lj_eval_sym.  Shared memory: 32 nt positions (4 floats) and nw x 3 x
// 32 nt accumulators (lj_dealt_bytes).
template <class Emit>
__device__ __noinline__ double lj_eval_dealt(CtaTeam& tm, const PotLJ& P, CView<float> cv, float* xw, Emit* emp,
                                             bool want_e, void* smem) {
  Emit emit = *emp;
  const int N = P.np, nd = P.ndim;
  const int nt = (N + 31) >> 5, npad = 32 * nt;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  // positions as 16-byte records (one conflict-free vector load per lane)
  float4* sx = reinterpret_cast<float4*>(smem);
  float* acc = reinterpret_cast<float*>(sx + npad);  // [warp][dim][particle]
  const float s6 = (float)P.s6;
  for (int j = threadIdx.x; j < npad; j += blockDim.x) {
    float4 v;
    v.w = 0.f;
    if (j < N) {
      v.x = cv(nd * j);
      v.y = cv(nd * j + 1);
      v.z = (nd == 3) ? cv(nd * j + 2) : 0.f;
      if (xw) {
        xw[nd * j] = v.x;
        xw[nd * j + 1] = v.y;
        if (nd == 3) xw[nd * j + 2] = v.z;
      }
    } else {
      v.x = (float)(1e6 * (double)(j + 1));
      v.y = 0.f;
      v.z = 0.f;
    }
    sx[j] = v;
  }
  for (int k = threadIdx.x; k < 3 * nw * npad; k += blockDim.x) acc[k] = 0.f;
  __syncthreads();
  float* mine = acc + (size_t)w * 3 * npad;
  LjAcc<float> e;
  const int npairs = nt * (nt + 1) / 2;
  for (int p = w; p < npairs; p += nw) {
    int I = 0, rem = p;
    while (rem >= nt - I) {
      rem -= nt - I;
      I++;
    }
    const int J = I + rem;
    const int i = 32 * I + lane;
    const float4 a = sx[i];
    float fx = 0.f, fy = 0.f, fz = 0.f, ee = 0.f;
    if (I == J) {
      // each lane with the 31 others of its tile (every pair twice, half the
      // energy each), force on the own particle only
#pragma unroll 4
      for (int s = 1; s < 32; s++) {
        const float4 b = sx[32 * I + ((lane + s) & 31)];
        const float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
        float lj6, lj12, f;
        lj_pair(dx, dy, dz, s6, lj6, lj12, f);
        fx += dx * f; fy += dy * f; fz += dz * f;
        ee += lj12 - lj6;
      }
      mine[i] += fx; mine[npad + i] += fy; mine[2 * npad + i] += fz;
      if (want_e && i < N) e.add(0.5f * ee);
    } else {
      float4 b = sx[32 * J + lane];
      float gx = 0.f, gy = 0.f, gz = 0.f;
      const int src = (lane + 1) & 31;
#pragma unroll 4
      for (int s = 0; s < 32; s++) {
        const float4 bc = b;
        b.x = __shfl_sync(0xffffffffu, b.x, src);
        b.y = __shfl_sync(0xffffffffu, b.y, src);
        b.z = __shfl_sync(0xffffffffu, b.z, src);
        const float dx = a.x - bc.x, dy = a.y - bc.y, dz = a.z - bc.z;
        float lj6, lj12, f;
        lj_pair(dx, dy, dz, s6, lj6, lj12, f);
        const float ex = dx * f, ey = dy * f, ez = dz * f;
        fx += ex; fy += ey; fz += ez;
        gx = __shfl_sync(0xffffffffu, gx - ex, src);
        gy = __shfl_sync(0xffffffffu, gy - ey, src);
        gz = __shfl_sync(0xffffffffu, gz - ez, src);
        ee += lj12 - lj6;
      }
      const int j = 32 * J + lane;
      mine[i] += fx; mine[npad + i] += fy; mine[2 * npad + i] += fz;
      mine[j] += gx; mine[npad + j] += gy; mine[2 * npad + j] += gz;
      if (want_e) e.add(ee);
    }
  }
  __syncthreads();
  const double c = -24.0 * P.eps;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    float f[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      float t = 0.f;
      for (int k = 0; k < nw; k++) t += acc[((size_t)k * 3 + d) * npad + i];
      f[d] = t;
    }
    emit(nd * i, (float)c * f[0]);
    emit(nd * i + 1, (float)c * f[1]);
    if (nd == 3) emit(nd * i + 2, (float)c * f[2]);
  }
  __syncthreads();
  *emp = emit;
  return 4.0 * P.eps * e.total();
}

// Symmetric all-pairs evaluation for one CTA (the batched path): each
// unordered pair is computed once.  Particles are grouped in tiles of 32;
// tile pairs are scheduled round-robin (circle method) so that within a
// round every tile belongs to one warp.  The warp keeps its i tile in lanes
// and rotates the j tile's positions and forces through the lanes with
// shuffles (32 steps return them home), then adds both tiles' forces to
// shared-memory accumulators -- no atomics, and the summation order per
// particle is fixed by the round order, so results are deterministic.  Tiles
// are padded with particles 1e6 sigma apart, which contribute nothing
// measurable.  Shared memory: positions and forces (3 values each) per
// particle, in the pair arithmetic type.
template <typename T, class Emit>
__device__ __noinline__ double lj_eval_sym(CtaTeam& tm, const PotLJ& P, CView<T> cv, T* xw, Emit* emp,
                                           bool want_e, void* smem) {
  using L = LjC<T>;
  using C = typename L::C;
  Emit emit = *emp;
  const int N = P.np, nd = P.ndim;
  const int nt = (N + 31) >> 5;            // tiles
  const int ntp = nt + (nt & 1);           // even count for the schedule (last may be empty)
  CV3<C>* sx = reinterpret_cast<CV3<C>*>(smem);
  C* sf = reinterpret_cast<C*>(sx + 32 * ntp);  // 3 per particle
  const C s6 = L::from((T)P.s6);
  const C zero = L::from((T)0);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int j = threadIdx.x; j < 32 * ntp; j += blockDim.x) {
    CV3<C> v;
    if (j < N) {
      const T px = cv(nd * j), py = cv(nd * j + 1), pz = (nd == 3) ? cv(nd * j + 2) : (T)0;
      v.x = L::from(px);
      v.y = L::from(py);
      v.z = L::from(pz);
      if (xw) {
        xw[nd * j] = px;
        xw[nd * j + 1] = py;
        if (nd == 3) xw[nd * j + 2] = pz;
      }
    } else {
      v.x = L::from((T)(1e6 * (double)(j + 1)));
      v.y = zero;
      v.z = zero;
    }
    sx[j] = v;
    sf[3 * j] = zero;
    sf[3 * j + 1] = zero;
    sf[3 * j + 2] = zero;
  }
  __syncthreads();
  LjAcc<C> e;
  // diagonal tiles: each lane pairs with the 31 others of its tile (every
  // pair twice, half the energy each), force on the own particle only
  for (int t = w; t < nt; t += nw) {
    const int i = 32 * t + lane;
    const CV3<C> a = sx[i];
    C fx = zero, fy = zero, fz = zero, ee = zero;
#pragma unroll 4
    for (int s = 1; s < 32; s++) {
      const CV3<C> b = sx[32 * t + ((lane + s) & 31)];
      const C dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
      C lj6, lj12, f;
      lj_pair(dx, dy, dz, s6, lj6, lj12, f);
      fx = fx + dx * f; fy = fy + dy * f; fz = fz + dz * f;
      ee = ee + (lj12 - lj6);
    }
    sf[3 * i] = sf[3 * i] + fx; sf[3 * i + 1] = sf[3 * i + 1] + fy; sf[3 * i + 2] = sf[3 * i + 2] + fz;
    if (want_e && i < N) e.add(ee * L::from((T)0.5));
  }
  __syncthreads();
  // off-diagonal tile pairs, circle-method rounds
  const int half = ntp >> 1;
  for (int r = 0; r < ntp - 1; r++) {
    for (int k = w; k < half; k += nw) {
      int I, J;
      if (k == 0) { I = ntp - 1; J = r; }
      else { I = (r + k) % (ntp - 1); J = (r - k + (ntp - 1)) % (ntp - 1); }
      if (I >= nt || J >= nt) continue;   // the empty padding tile
      const int i = 32 * I + lane;
      const CV3<C> a = sx[i];
      CV3<C> b = sx[32 * J + lane];
      C fx = zero, fy = zero, fz = zero, gx = zero, gy = zero, gz = zero, ee = zero;
      const int src = (lane + 1) & 31;
      // the next step's j position is fetched first: only the force rotation
      // (an add and a shuffle) chains one step to the next, so the pair
      // arithmetic of consecutive steps overlaps
#pragma unroll 4
      for (int s = 0; s < 32; s++) {
        const CV3<C> bc = b;
        b.x = lj_shfl(b.x, src);
        b.y = lj_shfl(b.y, src);
        b.z = lj_shfl(b.z, src);
        const C dx = a.x - bc.x, dy = a.y - bc.y, dz = a.z - bc.z;
        C lj6, lj12, f;
        lj_pair(dx, dy, dz, s6, lj6, lj12, f);
        const C ex = dx * f, ey = dy * f, ez = dz * f;
        fx = fx + ex; fy = fy + ey; fz = fz + ez;
        gx = lj_shfl(gx - ex, src);
        gy = lj_shfl(gy - ey, src);
        gz = lj_shfl(gz - ez, src);
        ee = ee + (lj12 - lj6);
      }
      const int j = 32 * J + lane;
      sf[3 * i] = sf[3 * i] + fx; sf[3 * i + 1] = sf[3 * i + 1] + fy; sf[3 * i + 2] = sf[3 * i + 2] + fz;
      sf[3 * j] = sf[3 * j] + gx; sf[3 * j + 1] = sf[3 * j + 1] + gy; sf[3 * j + 2] = sf[3 * j + 2] + gz;
      if (want_e) e.add(ee);
    }
    __syncthreads();
  }
  const double c = -24.0 * P.eps;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    emit(nd * i, L::scaled(c, sf[3 * i]));
    emit(nd * i + 1, L::scaled(c, sf[3 * i + 1]));
    if (nd == 3) emit(nd * i + 2, L::scaled(c, sf[3 * i + 2]));
  }
  __syncthreads();
  *emp = emit;
  return 4.0 * P.eps * e.total();
}

// ===========================================================================
// PhaseField (MODEL_BASIC), gather form of PhaseField::energyGradient
// (src/potentials/PhaseField.cpp:238-288, 365-393, 432-537) followed by the
// node-local parts of specialisedConstraints (fixFluid, hard density, lines
// 580-612).  Each node computes its own bulk and gradient terms and collects
// the contributions that the reference scatters into it from its two
// neighbours in every direction, so every DOF is written exactly once.
//
// With PF_UNSTR the same sweep evaluates PhaseFieldUnstructured's energy
// elements (src/potentials/PhaseFieldUnstructured.cpp:158-236, 518-692):
// solid nodes carry no elements, pressure acts on fixed fluids too, the soft
// density element reads the first three fluids; PF_NALL is its
// fluidEnergyAll (DENSITY_FIXED) and PF_UVOL its blockEnergyGradient volume
// penalty (lines 280-308), whose volumes are summed over the team first.
// ===========================================================================
__device__ __forceinline__ int pf_type1(const PotPF& P, int node) {  // type + 1
  return P.aux ? (int)(P.aux[node] & 15u) : 1;
}

template <typename T, typename A, class Src, class Team, class Emit>
__device__ __forceinline__ double pf_eval_impl(Team& tm, const PotPF& P, const Src& src, CView<T> cv, T* xw,
                                               Emit* emp, bool want_e, bool want_g) {
  constexpr int NFMAX = MINIM_MAXF;
  Emit emit = *emp;
  const int nf = P.nfluid;
  const int nx = P.n[0], ny = P.n[1], nz = P.n[2];
  const int ng = P.ngrid;
  const unsigned fl = P.flags;
  const A res2 = (A)P.res2;
  EAcc<A> e;
  // the parameters in the arithmetic type, converted once
  A volA[9], kapA[NFMAX], kPA[NFMAX];
#pragma unroll
  for (int t = 0; t < 9; t++) volA[t] = (A)P.vol_of_type[t];
#pragma unroll
  for (int f = 0; f < NFMAX; f++) {
    kapA[f] = (A)P.kappa[f];
    kPA[f] = (A)P.kappaP[f];
  }
  // PF_UVOL: volume differences at these coordinates, every thread
  double dvol[NFMAX];
#pragma unroll
  for (int f = 0; f < NFMAX; f++) dvol[f] = 0.0;
  if (fl & PF_UVOL) {
    for (int iG = tm.tid(); iG < ng; iG += tm.nthr()) {
      const double V = P.vol_of_type[pf_type1(P, iG)];
#pragma unroll
      for (int f = 0; f < NFMAX; f++) {
        if (f < nf) {
          const double cf = (double)cv(iG * nf + f);
          dvol[f] += (nf == 1) ? 0.5 * (cf + 1) * V : cf * V;
        }
      }
    }
    tm.reduce(dvol);
#pragma unroll
    for (int f = 0; f < NFMAX; f++) {
      if (f < nf) {
        dvol[f] -= P.vol_target[f];
        if (want_e && tm.tid() == 0) e.add((A)(P.vol_coef * dvol[f] * dvol[f]));
      }
    }
  }
  const bool unstr = (fl & PF_UNSTR) != 0;
  const bool nall = (fl & PF_NALL) != 0;
  for (int iG = tm.tid(); iG < ng; iG += tm.nthr()) {
    const int z = iG % nz, y = (iG / nz) % ny, x = iG / (ny * nz);
    int nb[6];
    nb[0] = ((x == 0 ? nx - 1 : x - 1) * ny + y) * nz + z;
    nb[1] = ((x == nx - 1 ? 0 : x + 1) * ny + y) * nz + z;
    nb[2] = (x * ny + (y == 0 ? ny - 1 : y - 1)) * nz + z;
    nb[3] = (x * ny + (y == ny - 1 ? 0 : y + 1)) * nz + z;
    nb[4] = (x * ny + y) * nz + (z == 0 ? nz - 1 : z - 1);
    nb[5] = (x * ny + y) * nz + (z == nz - 1 ? 0 : z + 1);
    const unsigned aux_i = P.aux ? P.aux[iG] : 1u;
    const int t1 = (int)(aux_i & 15u);
    const bool solid_i = (t1 == 0);
    const unsigned mask_i = aux_i >> 4;
    const A V = volA[t1];
    unsigned aux_nb[6];
#pragma unroll
    for (int k = 0; k < 6; k++) aux_nb[k] = P.aux ? P.aux[nb[k]] : 1u;

    A c[NFMAX], g[NFMAX];
#pragma unroll
    for (int f = 0; f < NFMAX; f++) {
      if (f < nf) {
        c[f] = src(iG * nf + f);
        if (xw) xw[iG * nf + f] = cv(iG * nf + f);
        g[f] = 0;
      }
    }
    // solid nodes carry no elements in the element form
    const bool node_terms = !(unstr && solid_i);
    A rd = -1;  // soft density: sum c - 1 (element form: the first three fluids)
    if (fl & PF_SOFT) {
      if (unstr) {
        rd = c[0] + c[1] + c[2] - 1;
      } else {
#pragma unroll
        for (int f = 0; f < NFMAX; f++)
          if (f < nf) rd += c[f];
      }
    }
    // PF_NALL: the last fluid's term (fluidEnergyAll), whose gradient every
    // other fluid receives with the opposite sign.  Its local indices are all
    // distinct, so a solid neighbour (replaced by the node itself) enters as
    // a zero difference, and its factor has no 1/res^2.
    A gnall = 0;
    if (nall && node_terms) {
      A cN[7];
#pragma unroll
      for (int k = 0; k < 7; k++) cN[k] = 1;
#pragma unroll
      for (int f = 0; f < NFMAX - 1; f++) {
        if (f < nf - 1) {
          cN[0] -= c[f];
#pragma unroll
          for (int k = 0; k < 6; k++) cN[k + 1] -= src((((mask_i >> k) & 1u) ? iG : nb[k]) * nf + f);
        }
      }
      const A bN = (A)0.5 * kapA[nf - 1] * V;
      const A gfN = (A)0.5 * kPA[nf - 1] * V;
      const A a = cN[0] * (cN[0] - 1);
      if (want_e) e.add(bN * a * a);
      gnall = bN * 2 * cN[0] * (cN[0] - 1) * (2 * cN[0] - 1);
      A eg = 0;
#pragma unroll
      for (int d = 0; d < 3; d++) {
        const A gm = cN[0] - cN[1 + 2 * d], gp = cN[0] - cN[2 + 2 * d];
        eg += (A)0.5 * (gm * gm + gp * gp);
        gnall += gfN * (gm + gp);
        // the elements of the non-solid neighbours, whose slot toward this
        // node holds this node
#pragma unroll
        for (int sd = 0; sd < 2; sd++) {
          const int k = 2 * d + sd;
          if (((mask_i >> k) & 1u) || !want_g) continue;
          const A Vj = volA[aux_nb[k] & 15u];
          gnall -= (A)0.5 * kPA[nf - 1] * Vj * (cN[1 + k] - cN[0]);
        }
      }
      if (want_e) e.add(gfN * eg);
    }
    bool force_e_done = false;  // energy-only semantics of forceEnergy
#pragma unroll
    for (int f = 0; f < NFMAX; f++) {
      if (f >= nf) break;
      const int dof = iG * nf + f;
      const A cc = c[f];
      const A kap = (fl & PF_NODE_KAPPA) ? (A)P.kappa_node[dof] : kapA[f];
      const A kP = (fl & PF_NODE_KAPPA) ? (A)P.kappaP_node[dof] : kPA[f];
      A gv = 0;
      if (nall && f < nf - 1) gv -= gnall;
      // bulk (with PF_NALL the last fluid has none of its own)
      if (nall && f == nf - 1) {
        // nothing: its concentration is 1 minus the others'
      } else if (nf == 1) {
        const A fac = kap / 16 * V;
        const A a = (cc + 1) * (cc - 1);
        if (want_e) e.add(fac * a * a);
        gv += fac * 4 * cc * (cc * cc - 1);
      } else {
        const A fac = (A)0.5 * kap * V;
        const A a = cc * (cc - 1);
        if (want_e) e.add(fac * a * a);
        gv += fac * 2 * cc * (cc - 1) * (2 * cc - 1);
      }
      // gradient energy
      const A coefk = ((nf == 1) ? (A)0.25 : (A)0.5) / res2;
      const A Fi = coefk * kP * V;
      A eg = 0;
      const bool own_grad = !(nall && f == nf - 1);
#pragma unroll
      for (int d = 0; d < 3; d++) {
        if (P.n[d] == 1 || !own_grad) continue;
        const int im = nb[2 * d], ip = nb[2 * d + 1];
        const A cm = src(im * nf + f), cp = src(ip * nf + f);
        const bool sm = (mask_i >> (2 * d)) & 1u, sp = (mask_i >> (2 * d + 1)) & 1u;
        const A gm = cc - cm, gp = cc - cp;
        if (!sm && !sp) {
          eg += (A)0.5 * (gm * gm + gp * gp);
          gv += Fi * (gm + gp);
        } else if (!sp) {
          eg += gp * gp;
          gv += Fi * 2 * gp;
        } else if (!sm) {
          eg += gm * gm;
          gv += Fi * 2 * gm;
        }
        if (!solid_i && want_g) {  // gradient only: energy-only sweeps skip the gathers
          if (!sp) {  // term of node p whose minus neighbour is this node
            const unsigned ap = aux_nb[2 * d + 1];
            const A Vp = volA[ap & 15u];
            const A kPp = (fl & PF_NODE_KAPPA) ? (A)P.kappaP_node[ip * nf + f] : kP;
            const A Fp = coefk * kPp * Vp;
            const bool pp_solid = ((ap >> 4) >> (2 * d + 1)) & 1u;
            gv -= (pp_solid ? (A)2 : (A)1) * Fp * (cp - cc);
          }
          if (!sm) {  // term of node m whose plus neighbour is this node
            const unsigned am = aux_nb[2 * d];
            const A Vm = volA[am & 15u];
            const A kPm = (fl & PF_NODE_KAPPA) ? (A)P.kappaP_node[im * nf + f] : kP;
            const A Fm = coefk * kPm * Vm;
            const bool mm_solid = ((am >> 4) >> (2 * d)) & 1u;
            gv -= (mm_solid ? (A)2 : (A)1) * Fm * (cm - cc);
          }
        }
      }
      if (want_e) e.add(Fi * eg);
      // surface (binary only)
      if ((fl & PF_CONTACT) && nf == 1) {
        const A w = (A)P.wet[iG];
        if (w != 0) {
          if (want_e) e.add(w * (cc * cc * cc / 3 - cc - (A)(2.0 / 3)));
          gv += w * (cc * cc - 1);
        }
      }
      // pressure (the element form has it on fixed fluids too)
      if ((fl & PF_PRESSURE) && P.pressure[f] != 0 && node_terms && (unstr || !((P.fix_mask >> f) & 1u))) {
        const A pr = (A)P.pressure[f];
        if (nf == 1) {
          if (want_e) e.add(-pr * ((A)0.5 * (cc + 1) * V));
          gv -= (A)0.5 * pr * V;
        } else {
          if (want_e) e.add(-pr * (cc * V));
          gv -= pr * V;
        }
      }
      // soft density
      if ((fl & PF_SOFT) && nf > 1 && node_terms && (!unstr || f < 3)) {
        const A sc = (A)P.soft_coef;
        if (want_e && f == 0) e.add(sc * rd * rd);
        gv += 2 * sc * rd;
      }
      // body force
      if ((fl & PF_FORCE) && !solid_i && P.fmag[f] != 0) {
        const A cf = (nf == 1) ? (A)0.5 * (1 + cc) : cc;
        if (cf >= (A)0.01) {
          const A co0 = (A)(x - (nx - 1) / 2.0), co1 = (A)(y - (ny - 1) / 2.0),
                  co2 = (A)(z - (nz - 1) / 2.0);
          const A h = -(co0 * (A)P.fnorm[f][0] + co1 * (A)P.fnorm[f][1] + co2 * (A)P.fnorm[f][2]) *
                      (A)P.res;
          const A epc = V * (A)P.fmag[f] * h;
          // PhaseField::forceEnergy returns after the first fluid when no
          // gradient is asked for; the element form counts every fluid
          if (want_e && (unstr || !force_e_done)) e.add(cf * epc);
          force_e_done = true;
          gv += (nf == 1) ? (A)0.5 * epc : epc;
        }
      }
      // diffuse-solid confinement
      if ((fl & PF_CONFINE) && P.confine_coef[f] != 0 && node_terms) {
        const A c0 = (A)P.ff_init[dof];
        if ((c0 - (A)0.5) * (cc - (A)0.5) < 0) {
          const A coef = (A)P.confine_coef[f];
          if (want_e) e.add(coef * (cc - (A)0.5) * (cc - (A)0.5));
          gv += coef * 2 * (cc - (A)0.5);
        }
      }
      // element form's fixed volume: the penalty's force on interface nodes
      if (fl & PF_UVOL) {
        A w = 4 * cc * (1 - cc);
        if (w < 0) w = 0;
        gv += (A)(P.vol_coef * dvol[f]) * V * w;
      }
      g[f] = gv;
    }
    if (want_g) {
      // node-local constraints: fixed fluids, then the hard density projection
      if (fl & PF_FIXFLUID) {
#pragma unroll
        for (int f = 0; f < NFMAX; f++)
          if (f < nf && ((P.fix_mask >> f) & 1u)) g[f] = 0;
      }
      if ((fl & PF_HARD) && nf > 1) {
        A comp = 0;
#pragma unroll
        for (int f = 0; f < NFMAX; f++)
          if (f < nf && !((P.fix_mask >> f) & 1u)) comp += g[f];
        comp *= (A)1 / (A)P.nvar;
#pragma unroll
        for (int f = 0; f < NFMAX; f++)
          if (f < nf && !((P.fix_mask >> f) & 1u)) g[f] -= comp;
      }
#pragma unroll
      for (int f = 0; f < NFMAX; f++)
        if (f < nf) emit(iG * nf + f, g[f]);
    }
  }
  *emp = emit;
  return e.total();
}


template <typename T>
struct CvSrc {
  CView<T> cv;
  __device__ __forceinline__ T operator()(int i) const { return cv(i); }
};
struct DfSrc {
  const float* hi;
  const float* lo;
  __device__ __forceinline__ DFn operator()(int i) const { return DFn(DF{hi[i], lo[i]}); }
};

template <typename T, class Team, class Emit>
__device__ __noinline__ double pf_eval(Team& tm, const PotPF& P, CView<T> cv, T* xw, Emit* emp,
                                       bool want_e, bool want_g) {
  return pf_eval_impl<T, T>(tm, P, CvSrc<T>{cv}, cv, xw, emp, want_e, want_g);
}

// The FP64-coordinate evaluation in double-float arithmetic (about 47 bits;
// FP64 runs at 1/64 of the FP32 rate on GB300): the field at the evaluated
// point is split once into hi/lo float arrays (two FP32 scratch vectors of
// ndof) -- by bits, and a line-search trial point formed in double-float --
// then the same sweep runs on DFn.  The caller's next team-wide
// reduction orders this evaluation's reads of the scratch before the next
// one's writes.
template <class Team, class Emit>
__device__ __noinline__ double pf_eval_df(Team& tm, const PotPF& P, CView<double> cv, double* xw, Emit* emp,
                                          bool want_e, bool want_g, float* hi, float* lo) {
  const int n = P.ngrid * P.nfluid;
  if (xw || !cv.p) {
    // the point is stored (or is the stored one): split the FP64 value
    for (int i = tm.tid(); i < n; i += tm.nthr()) {
      const double v = cv(i);
      if (xw) xw[i] = v;
      const DF d = df_split_bits(v);
      hi[i] = d.hi;
      lo[i] = d.lo;
    }
  } else {
    // a line-search trial x + t p, formed in double-float
    const DFn t = DFn(cv.t);
    for (int i = tm.tid(); i < n; i += tm.nthr()) {
      const DFn d = DFn(df_split_bits(cv.x[i])) + t * DFn(cv.p[i]);
      hi[i] = d.hi;
      lo[i] = d.lo;
    }
  }
  tm.sync();
  return pf_eval_impl<double, DFn>(tm, P, DfSrc{hi, lo}, cv, (double*)nullptr, emp, want_e, want_g);
}

// Four consecutive values of a coordinate view (aligned: element 4*i4).
template <typename T> struct Quad { T v[4]; };
__device__ __forceinline__ Quad<float> cv4(const CView<float>& cv, int i4) {
  const float4 x = ld4(cv.x, i4);
  Quad<float> q{{x.x, x.y, x.z, x.w}};
  if (cv.p) {
    const float4 p = ld4(cv.p, i4);
    q.v[0] = __fadd_rn(x.x, __fmul_rn(cv.t, p.x));
    q.v[1] = __fadd_rn(x.y, __fmul_rn(cv.t, p.y));
    q.v[2] = __fadd_rn(x.z, __fmul_rn(cv.t, p.z));
    q.v[3] = __fadd_rn(x.w, __fmul_rn(cv.t, p.w));
  }
  return q;
}
__device__ __forceinline__ Quad<double> cv4(const CView<double>& cv, int i4) {
  const double2 a = reinterpret_cast<const double2*>(cv.x)[2 * i4];
  const double2 b = reinterpret_cast<const double2*>(cv.x)[2 * i4 + 1];
  Quad<double> q{{a.x, a.y, b.x, b.y}};
  if (cv.p) {
    const float4 p = ld4(cv.p, i4);
    q.v[0] = __dadd_rn(a.x, __dmul_rn(cv.t, (double)p.x));
    q.v[1] = __dadd_rn(a.y, __dmul_rn(cv.t, (double)p.y));
    q.v[2] = __dadd_rn(b.x, __dmul_rn(cv.t, (double)p.z));
    q.v[3] = __dadd_rn(b.y, __dmul_rn(cv.t, (double)p.w));
  }
  return q;
}
__device__ __forceinline__ void st_quad(float* x, int i4, const Quad<float>& q) {
  st4(x, i4, make_float4(q.v[0], q.v[1], q.v[2], q.v[3]));
}
__device__ __forceinline__ void st_quad(double* x, int i4, const Quad<double>& q) {
  reinterpret_cast<double2*>(x)[2 * i4] = make_double2(q.v[0], q.v[1]);
  reinterpret_cast<double2*>(x)[2 * i4 + 1] = make_double2(q.v[2], q.v[3]);
}
// Loads an emitter needs for four values (issued with the stencil's loads),
// and hands four gradient values to it (vector store when it has one).
struct NoPre {};
template <class Emit>
__device__ __forceinline__ auto emit_pre(const Emit& em, int i4, bool want_g) {
  if constexpr (requires { em.pre4(i4); }) {
    return want_g ? em.pre4(i4) : decltype(em.pre4(i4)){};
  } else {
    return NoPre{};
  }
}
template <class Emit, typename T, class Pre>
__device__ __forceinline__ void emit_quad(Emit& em, int i4, const T (&g)[4], const Pre& pre) {
  if constexpr (requires { em.emit4(i4, float4{}, pre); }) {
    em.emit4(i4, make_float4((float)g[0], (float)g[1], (float)g[2], (float)g[3]), pre);
  } else {
#pragma unroll
    for (int k = 0; k < 4; k++) em(4 * i4 + k, g[k]);
  }
}

// Binary fluid on a grid whose innermost size is a multiple of 4: each thread
// evaluates four consecutive cells along z with 16-byte loads of the cell and
// of its x and y neighbour lines, plus two scalar loads for the z ends.
template <typename T, class Team, class Emit>
__device__ __noinline__ double pf1_eval_quad(Team& tm, const PotPF& P, CView<T> cv, T* xw, Emit* emp,
                                             bool want_e, bool want_g) {
  Emit emit = *emp;
  const int nx = P.n[0], ny = P.n[1], nz = P.n[2];
  const int nq = P.ngrid >> 2;
  const T V = (T)P.vol_of_type[1];
  const T fb = (T)P.kappa[0] / 16 * V;
  const T Fi = (T)0.25 / (T)P.res2 * (T)P.kappaP[0] * V;
  const T pr = (P.flags & PF_PRESSURE) ? (T)P.pressure[0] : (T)0;
  const bool dx_on = nx > 1, dy_on = ny > 1;
  EAcc<T> e;
  for (int q = tm.tid(); q < nq; q += tm.nthr()) {
    {  // next sweep step: fetch its lines into L2 now (its neighbour lines are
       // other threads' own lines in the same window)
      const int qn = q + P.pf_dist * tm.nthr();
      if (P.pf_dist > 0 && qn < nq) {
        const float* xf = reinterpret_cast<const float*>(cv.x);
        if (sizeof(T) == 8) {  // 8 quads of doubles span two lines
          prefetch_line(xf, 2 * qn);
          prefetch_line(xf, 2 * qn + 8);
        } else {
          prefetch_line(xf, qn);
        }
        if (cv.p) prefetch_line(cv.p, qn);
        if constexpr (requires { emit.prefetch4(qn); }) {
          if (want_g) emit.prefetch4(qn);
        }
      }
    }
    const int iG = 4 * q;
    const int z0 = iG % nz, line = iG / nz;
    const int y = line % ny, x = line / ny;
    // every load of the iteration is issued before any is used (one memory
    // round trip); a dimension of size 1 reads its own line and adds nothing
    const int ym = y == 0 ? ny - 1 : y - 1, yp = y == ny - 1 ? 0 : y + 1;
    const int xm = x == 0 ? nx - 1 : x - 1, xp = x == nx - 1 ? 0 : x + 1;
    const Quad<T> c = cv4(cv, q);
    const T zm = cv(z0 == 0 ? iG + nz - 1 : iG - 1);
    const T zp = cv(z0 + 4 == nz ? iG - z0 : iG + 4);
    const Quad<T> cym = cv4(cv, ((x * ny + ym) * nz + z0) >> 2);
    const Quad<T> cyp = cv4(cv, ((x * ny + yp) * nz + z0) >> 2);
    const Quad<T> cxm = cv4(cv, ((xm * ny + y) * nz + z0) >> 2);
    const Quad<T> cxp = cv4(cv, ((xp * ny + y) * nz + z0) >> 2);
    auto pre = emit_pre(emit, q, want_g);
    if (xw) st_quad(xw, q, c);
    T lap[4], eg[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {  // z: neighbours inside the quad, plus one scalar at each end
      const T cm = (k == 0) ? zm : c.v[k - 1];
      const T cp = (k == 3) ? zp : c.v[k + 1];
      const T gm = c.v[k] - cm, gp = c.v[k] - cp;
      lap[k] = gm + gp;
      eg[k] = (T)0.5 * (gm * gm + gp * gp);
    }
    if (dy_on) {
#pragma unroll
      for (int k = 0; k < 4; k++) {
        const T gm = c.v[k] - cym.v[k], gp = c.v[k] - cyp.v[k];
        lap[k] += gm + gp;
        eg[k] += (T)0.5 * (gm * gm + gp * gp);
      }
    }
    if (dx_on) {
#pragma unroll
      for (int k = 0; k < 4; k++) {
        const T gm = c.v[k] - cxm.v[k], gp = c.v[k] - cxp.v[k];
        lap[k] += gm + gp;
        eg[k] += (T)0.5 * (gm * gm + gp * gp);
      }
    }
    T g[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const T cc = c.v[k];
      const T a = (cc + 1) * (cc - 1);
      g[k] = fb * 4 * cc * (cc * cc - 1) + 2 * Fi * lap[k];
      if (want_e) {
        e.add(fb * a * a);
        e.add(Fi * eg[k]);
      }
      if (pr != 0) {
        if (want_e) e.add(-pr * ((T)0.5 * (cc + 1) * V));
        g[k] -= (T)0.5 * pr * V;
      }
    }
    if (want_g) emit_quad(emit, q, g, pre);
  }
  *emp = emit;
  return e.total();
}

// Binary fluid (nFluid == 1) without solid, contact angle, force or
// confinement: the 7-point stencil of the bulk and gradient terms plus the
// optional pressure term.  Same arithmetic as pf_eval for this case.
template <typename T, class Team, class Emit>
__device__ __noinline__ double pf1_eval(Team& tm, const PotPF& P, CView<T> cv, T* xw, Emit* emp,
                                        bool want_e, bool want_g) {
  Emit emit = *emp;
  const int nx = P.n[0], ny = P.n[1], nz = P.n[2];
  const int ng = P.ngrid;
  const T V = (T)P.vol_of_type[1];
  const T kap = (T)P.kappa[0];
  const T fb = kap / 16 * V;                      // bulk factor
  const T Fi = (T)0.25 / (T)P.res2 * (T)P.kappaP[0] * V;  // gradient factor
  const T pr = (P.flags & PF_PRESSURE) ? (T)P.pressure[0] : (T)0;
  const bool dx_on = nx > 1, dy_on = ny > 1, dz_on = nz > 1;
  EAcc<T> e;
  for (int iG = tm.tid(); iG < ng; iG += tm.nthr()) {
    const int z = iG % nz, y = (iG / nz) % ny, x = iG / (ny * nz);
    const T c = cv(iG);
    if (xw) xw[iG] = c;
    const T a = (c + 1) * (c - 1);
    T g = fb * 4 * c * (c * c - 1);
    T eg = 0, lap = 0;
    if (dx_on) {
      const T cm = cv(((x == 0 ? nx - 1 : x - 1) * ny + y) * nz + z);
      const T cp = cv(((x == nx - 1 ? 0 : x + 1) * ny + y) * nz + z);
      const T gm = c - cm, gp = c - cp;
      eg += (T)0.5 * (gm * gm + gp * gp);
      lap += gm + gp;
    }
    if (dy_on) {
      const T cm = cv((x * ny + (y == 0 ? ny - 1 : y - 1)) * nz + z);
      const T cp = cv((x * ny + (y == ny - 1 ? 0 : y + 1)) * nz + z);
      const T gm = c - cm, gp = c - cp;
      eg += (T)0.5 * (gm * gm + gp * gp);
      lap += gm + gp;
    }
    if (dz_on) {
      const T cm = cv(iG - z + (z == 0 ? nz - 1 : z - 1));
      const T cp = cv(iG - z + (z == nz - 1 ? 0 : z + 1));
      const T gm = c - cm, gp = c - cp;
      eg += (T)0.5 * (gm * gm + gp * gp);
      lap += gm + gp;
    }
    // own term F*(gm+gp) plus the two neighbours' terms, which contribute
    // the same amount again when nothing is solid
    g += 2 * Fi * lap;
    if (want_e) {
      e.add(fb * a * a);
      e.add(Fi * eg);
    }
    if (pr != 0) {
      if (want_e) e.add(-pr * ((T)0.5 * (c + 1) * V));
      g -= (T)0.5 * pr * V;
    }
    if (want_g) emit(iG, g);
  }
  *emp = emit;
  return e.total();
}

// PhaseField node-local constraints on an arbitrary vector (a step):
// fixFluid zeroing and the hard density projection.
template <typename T, class Team>
__device__ void pf_local_constrain(Team& tm, const PotPF& P, T* v) {
  const int nf = P.nfluid;
  for (int iG = tm.tid(); iG < P.ngrid; iG += tm.nthr()) {
    T* w = v + (size_t)iG * nf;
    if (P.flags & PF_FIXFLUID)
      for (int f = 0; f < nf; f++)
        if ((P.fix_mask >> f) & 1u) w[f] = 0;
    if ((P.flags & PF_HARD) && nf > 1) {
      T comp = 0;
      for (int f = 0; f < nf; f++)
        if (!((P.fix_mask >> f) & 1u)) comp += w[f];
      comp *= (T)1 / (T)P.nvar;
      for (int f = 0; f < nf; f++)
        if (!((P.fix_mask >> f) & 1u)) w[f] -= comp;
    }
  }
}

// Fixed-volume projection (specialisedConstraints lines 614-658):
// per variable fluid, remove the component along the (density-orthogonal)
// node-volume vector.  One reduction over the grid.
//
// FP32 vectors (the minimiser's gradients and directions): every per-element
// operation in FP32, the dot products as compensated FP32 pairs reduced with
// FP64 totals in one warp -- the FP64 form below spent the FP64 pipe (1/64 of
// the FP32 rate on GB300) on two divisions per element and was the busiest
// unit of a ternary grid's iteration.
template <class Team>
__device__ void pf_volume_project_f32(Team& tm, const PotPF& P, float* v) {
  const int nf = P.nfluid;
  const bool hard = (P.flags & PF_HARD) != 0;
  const float inv_nvar = 1.f / (float)P.nvar;
  float vf[9];
#pragma unroll
  for (int t = 0; t < 9; t++) vf[t] = (float)P.vol_of_type[t];
  Acc part[MINIM_MAXF];
  for (int iG = tm.tid(); iG < P.ngrid; iG += tm.nthr()) {
    const float V = vf[pf_type1(P, iG)];
    const float* w = v + (size_t)iG * nf;
    float sv = 0.f;
    if (hard)
      for (int f = 0; f < nf; f++)
        if (!((P.fix_mask >> f) & 1u)) sv += w[f];
#pragma unroll
    for (int f = 0; f < MINIM_MAXF; f++) {
      if (f < nf && !((P.fix_mask >> f) & 1u))
        part[f].add((w[f] - (hard ? sv * inv_nvar : 0.f)) * V);
    }
  }
  float ps[MINIM_MAXF], pc[MINIM_MAXF];
  double tot[2 * MINIM_MAXF];
#pragma unroll
  for (int f = 0; f < MINIM_MAXF; f++) {
    ps[f] = part[f].s;
    pc[f] = part[f].c;
  }
  // the components tot / totalVolume2, divided once per team (the FP64
  // divisions of a uniform value in every thread kept the FP64 pipe busy)
  const double tv2 = P.total_volume2;
  tm.template reduce_pairs<MINIM_MAXF, MINIM_MAXF>(ps, pc, tot, [tv2](double* o) {
#pragma unroll
    for (int f = 0; f < MINIM_MAXF; f++) o[MINIM_MAXF + f] = o[f] / tv2;
  });
  float comp[MINIM_MAXF], csum = 0.f;
#pragma unroll
  for (int f = 0; f < MINIM_MAXF; f++) {
    comp[f] = (f < nf && !((P.fix_mask >> f) & 1u)) ? (float)tot[MINIM_MAXF + f] : 0.f;
    csum += comp[f];
  }
  for (int iG = tm.tid(); iG < P.ngrid; iG += tm.nthr()) {
    const float V = vf[pf_type1(P, iG)];
    float* w = v + (size_t)iG * nf;
    for (int f = 0; f < nf; f++) {
      if ((P.fix_mask >> f) & 1u) continue;
      float d = comp[f] * V;
      if (hard) d -= csum * V * inv_nvar;
      w[f] -= d;
    }
  }
  tm.sync();
}

template <typename T, class Team>
__device__ void pf_volume_project(Team& tm, const PotPF& P, T* v) {
  if constexpr (std::is_same_v<T, float>) {
    pf_volume_project_f32(tm, P, v);
    return;
  }
  const int nf = P.nfluid;
  const bool hard = (P.flags & PF_HARD) != 0;
  double part[MINIM_MAXF];
#pragma unroll
  for (int f = 0; f < MINIM_MAXF; f++) part[f] = 0.0;
  for (int iG = tm.tid(); iG < P.ngrid; iG += tm.nthr()) {
    const double V = P.vol_of_type[pf_type1(P, iG)];
    const T* w = v + (size_t)iG * nf;
    double sv = 0.0;
    if (hard)
      for (int f = 0; f < nf; f++)
        if (!((P.fix_mask >> f) & 1u)) sv += (double)w[f];
#pragma unroll
    for (int f = 0; f < MINIM_MAXF; f++) {
      if (f < nf && !((P.fix_mask >> f) & 1u))
        part[f] += ((double)w[f] - (hard ? sv / P.nvar : 0.0)) * V;
    }
  }
  tm.reduce(part);
  double comp[MINIM_MAXF], csum = 0.0;
#pragma unroll
  for (int f = 0; f < MINIM_MAXF; f++) {
    comp[f] = (f < nf && !((P.fix_mask >> f) & 1u)) ? part[f] / P.total_volume2 : 0.0;
    csum += comp[f];
  }
  for (int iG = tm.tid(); iG < P.ngrid; iG += tm.nthr()) {
    const double V = P.vol_of_type[pf_type1(P, iG)];
    T* w = v + (size_t)iG * nf;
    for (int f = 0; f < nf; f++) {
      if ((P.fix_mask >> f) & 1u) continue;
      double d = comp[f] * V;
      if (hard) d -= csum * V / P.nvar;
      w[f] = (T)((double)w[f] - d);
    }
  }
  tm.sync();
}

// ===========================================================================
// BarAndHinge (src/potentials/BarAndHinge.cpp:269-387).  Bars and hinges are
// pre-sorted into colours (no two elements of a colour share a vertex), so
// each colour scatters into the FP64 accumulator without atomics and the
// result is deterministic.  The dihedral angle uses the atan2 form of the
// reference's acos expression (same angle, accurate near 0 and pi).
// ===========================================================================
template <typename T>
__device__ __forceinline__ T bah_atan2(T y, T x);
template <>
__device__ __forceinline__ float bah_atan2<float>(float y, float x) { return atan2f(y, x); }
template <>
__device__ __forceinline__ double bah_atan2<double>(double y, double x) { return atan2(y, x); }
template <typename T>
__device__ __forceinline__ T bah_fmod(T a, T b);
template <>
__device__ __forceinline__ float bah_fmod<float>(float a, float b) { return fmodf(a, b); }
template <>
__device__ __forceinline__ double bah_fmod<double>(double a, double b) { return fmod(a, b); }
template <typename T>
__device__ __forceinline__ T bah_sqrt(T a);
template <>
__device__ __forceinline__ float bah_sqrt<float>(float a) { return sqrtf(a); }
template <>
__device__ __forceinline__ double bah_sqrt<double>(double a) { return sqrt(a); }
// double-float square root: the FP32 root refined by one Newton step
template <>
__device__ __forceinline__ DFn bah_sqrt<DFn>(DFn a) {
  if (a.hi <= 0.f) return DFn(0);
  const float y = sqrtf(a.hi);
  const float p = __fmul_rn(y, y);
  const float ep = __fmaf_rn(y, y, -p);
  // residual a - y^2, then y + r / (2 y)
  const float r = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, p), ep), a.lo);
  return DFn(df_fast2sum(y, __fdividef(r, 2.f * y)));
}

// The wrapped dihedral difference of bending(): theta from the atan2 form
// (2 pi - theta when n1.b3 < 0), then fmod(theta - theta0 + pi, 2 pi) - pi.
// The double-float evaluation takes the angle and its wrap in FP64 from the
// two double-float arguments.
template <typename A>
__device__ __forceinline__ A bah_dtheta(A y, A x, bool neg, double theta0) {
  const A twopi = (A)(2.0 * 3.14159265358979323846);
  const A pi = (A)3.14159265358979323846;
  A th = bah_atan2<A>(y, x);
  if (neg) th = twopi - th;
  A dth = th - (A)theta0;
  return bah_fmod<A>(dth + pi, twopi) - pi;
}
template <>
__device__ __forceinline__ DFn bah_dtheta<DFn>(DFn y, DFn x, bool neg, double theta0) {
  return DFn(bah_dtheta<double>((double)y, (double)x, neg, theta0));
}

template <typename T, class Src>
__device__ __forceinline__ void bah_bar(const PotBAH& P, const Src& cv, int b, T& e, T* gl, T* gr,
                                        bool want_g) {
  const int2 nd = P.bars[b];
  const double2 pr = P.bar_par[b];
  const T dx = cv(3 * nd.x) - cv(3 * nd.y);
  const T dy = cv(3 * nd.x + 1) - cv(3 * nd.y + 1);
  const T dz = cv(3 * nd.x + 2) - cv(3 * nd.y + 2);
  const T l = bah_sqrt<T>(dx * dx + dy * dy + dz * dz);
  const T dl = l - (T)pr.y;
  const T k = (T)pr.x;
  e = (T)0.5 * k * dl * dl;
  if (want_g) {
    const T gf = 2 * k * dl / l;  // the reference's factor of 2
    gl[0] = gf * dx; gl[1] = gf * dy; gl[2] = gf * dz;
    gr[0] = -gl[0]; gr[1] = -gl[1]; gr[2] = -gl[2];
  }
}

template <typename T, class Src>
__device__ __forceinline__ void bah_hinge(const PotBAH& P, const Src& cv, int h, T& e, T (*gq)[3],
                                          bool want_g) {
  const int4 nd = P.hinges[h];
  const double2 pr = P.hinge_par[h];
  T x1[3], x2[3], x3[3], x4[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    x1[d] = cv(3 * nd.x + d); x2[d] = cv(3 * nd.y + d);
    x3[d] = cv(3 * nd.z + d); x4[d] = cv(3 * nd.w + d);
  }
  T b1[3], b2[3], b3[3];
#pragma unroll
  for (int d = 0; d < 3; d++) { b1[d] = x2[d] - x1[d]; b2[d] = x3[d] - x2[d]; b3[d] = x4[d] - x3[d]; }
  const T b2sq = b2[0] * b2[0] + b2[1] * b2[1] + b2[2] * b2[2];
  const T b2m = bah_sqrt<T>(b2sq);
  const T n1[3] = {b1[1] * b2[2] - b1[2] * b2[1], b1[2] * b2[0] - b1[0] * b2[2], b1[0] * b2[1] - b1[1] * b2[0]};
  const T n2[3] = {b2[1] * b3[2] - b2[2] * b3[1], b2[2] * b3[0] - b2[0] * b3[2], b2[0] * b3[1] - b2[1] * b3[0]};
  const T n1sq = n1[0] * n1[0] + n1[1] * n1[1] + n1[2] * n1[2];
  const T n2sq = n2[0] * n2[0] + n2[1] * n2[1] + n2[2] * n2[2];
  const T n1n2 = n1[0] * n2[0] + n1[1] * n2[1] + n1[2] * n2[2];
  const T n1b3 = n1[0] * b3[0] + n1[1] * b3[1] + n1[2] * b3[2];
  // acos(n1.n2/|n1||n2|) = atan2(|n1 x n2|, n1.n2) and |n1 x n2| = |b2| |n1.b3|
  const T dth = bah_dtheta<T>(b2m * (n1b3 >= 0 ? n1b3 : -n1b3), n1n2, n1b3 < 0, pr.y);
  const T k = (T)pr.x;
  e = (T)0.5 * k * dth * dth;
  if (want_g) {
    const T gf = k * dth;
    const T s1 = b2m / n1sq, s2 = b2m / n2sq;
    const T sk1 = -(b1[0] * b2[0] + b1[1] * b2[1] + b1[2] * b2[2]) / b2sq;
    const T sk2 = -(b3[0] * b2[0] + b3[1] * b2[1] + b3[2] * b2[2]) / b2sq;
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const T a1 = s1 * n1[d], a2 = s2 * n2[d];
      gq[0][d] = -gf * a1;
      gq[1][d] = gf * ((1 - sk1) * a1 - sk2 * a2);
      gq[2][d] = -gf * ((1 - sk2) * a2 - sk1 * a1);
      gq[3][d] = gf * a2;
    }
  }
}

// Per-vertex external force and substrate wall (lines 359-387); returns the
// energy and the z-gradient of vertex v.
template <typename T, class Src>
__device__ __forceinline__ void bah_vertex(const PotBAH& P, const Src& cv, int v, T& e, T& gz) {
  e = 0; gz = 0;
  if (!P.node_el[v]) return;
  double fz = 0;
  if (P.nforce == 3) fz = P.force[2];
  else if (P.nforce > 0) fz = P.force[3 * v + 2];
  const T z = cv(3 * v + 2);
  e -= (T)fz * z;
  gz -= (T)fz;
  if (P.wall_on) {
    if (!P.wall_adh && z > 0) return;
    const double sig = P.wall_sig;
    const T r0 = (T)(0.858374218932559 * sig);
    T h = z + r0;
    if (h < r0 / 2) h = r0 / 2;
    const T q = (T)sig / h;
    const T q3 = q * q * q;
    const T lj9 = (T)(2.0 / 15) * q3 * q3 * q3;
    const T lj3 = q3;
    const double s3 = sig * sig * sig;
    const T lj9_0 = (T)(0.5270462766947298 * s3 * s3 * s3);
    const T lj3_0 = (T)(1.5811388300841895 * s3);
    e += (T)P.wall_eps * ((lj9 - lj9_0) - (lj3 - lj3_0));
    gz -= (T)P.wall_eps * (9 * lj9 - 3 * lj3) / h;
  }
}

// Gradient accumulators of the colour scatter: FP64, or double-float pairs in
// the same 8 bytes per DOF
struct GaF64 {
  double* g;
  template <typename A>
  __device__ __forceinline__ void set(int j, A v) { g[j] = (double)v; }
  template <typename A>
  __device__ __forceinline__ void add(int j, A v) { g[j] += (double)v; }
  __device__ __forceinline__ double get(int j) const { return g[j]; }
};
struct GaDF {
  DF* g;
  __device__ __forceinline__ void set(int j, DFn v) { g[j] = v.df(); }
  __device__ __forceinline__ void add(int j, DFn v) { g[j] = (DFn(g[j]) + v).df(); }
  __device__ __forceinline__ DFn get(int j) const { return DFn(g[j]); }
};

template <typename T, typename A, class Src, class Ga, class Team, class Emit>
__device__ __forceinline__ double bah_eval_impl(Team& tm, const PotBAH& P, const Src& src, CView<T> cv, T* xw,
                                                Ga ga, Emit* emp, bool want_e, bool want_g) {
  Emit emit = *emp;
  EAcc<A> e;
  const int nv = P.nvert;
  for (int v = tm.tid(); v < nv; v += tm.nthr()) {
    if (xw) {
      xw[3 * v] = cv(3 * v); xw[3 * v + 1] = cv(3 * v + 1); xw[3 * v + 2] = cv(3 * v + 2);
    }
    A ev, gz;
    bah_vertex<A>(P, src, v, ev, gz);
    if (want_e) e.add(ev);
    if (want_g) {
      ga.set(3 * v, A(0)); ga.set(3 * v + 1, A(0)); ga.set(3 * v + 2, gz);
    }
  }
  if (!want_g) {
    for (int b = tm.tid(); b < P.nbar; b += tm.nthr()) {
      A eb; bah_bar<A>(P, src, b, eb, (A*)nullptr, (A*)nullptr, false);
      e.add(eb);
    }
    for (int h = tm.tid(); h < P.nhinge; h += tm.nthr()) {
      A eh; bah_hinge<A>(P, src, h, eh, (A(*)[3])nullptr, false);
      e.add(eh);
    }
    *emp = emit;
    return e.total();
  }
  tm.sync();
  for (int c = 0; c < P.nbar_colors; c++) {
    const int b0 = P.bar_color_off[c], b1 = P.bar_color_off[c + 1];
    for (int b = b0 + tm.tid(); b < b1; b += tm.nthr()) {
      A eb, gl[3], gr[3];
      bah_bar<A>(P, src, b, eb, gl, gr, true);
      if (want_e) e.add(eb);
      const int2 nd = P.bars[b];
#pragma unroll
      for (int d = 0; d < 3; d++) {
        ga.add(3 * nd.x + d, gl[d]);
        ga.add(3 * nd.y + d, gr[d]);
      }
    }
    tm.sync();
  }
  for (int c = 0; c < P.nhinge_colors; c++) {
    const int h0 = P.hinge_color_off[c], h1 = P.hinge_color_off[c + 1];
    for (int h = h0 + tm.tid(); h < h1; h += tm.nthr()) {
      A eh, gq[4][3];
      bah_hinge<A>(P, src, h, eh, gq, true);
      if (want_e) e.add(eh);
      const int4 nd = P.hinges[h];
      const int vs[4] = {nd.x, nd.y, nd.z, nd.w};
#pragma unroll
      for (int q = 0; q < 4; q++)
#pragma unroll
        for (int d = 0; d < 3; d++) ga.add(3 * vs[q] + d, gq[q][d]);
    }
    tm.sync();
  }
  for (int i = tm.tid(); i < 3 * nv; i += tm.nthr()) emit(i, (A)ga.get(i));
  *emp = emit;
  return e.total();
}


template <typename T, class Team, class Emit>
__device__ __noinline__ double bah_eval(Team& tm, const PotBAH& P, CView<T> cv, T* xw, double* GA,
                                        Emit* emp, bool want_e, bool want_g) {
  return bah_eval_impl<T, T>(tm, P, CvSrc<T>{cv}, cv, xw, GaF64{GA}, emp, want_e, want_g);
}

// The FP64-coordinate evaluation in double-float (as pf_eval_df): the
// coordinates split once into the hi/lo scratch, bars and hinges in
// double-float (the dihedral angle and its wrap in FP64), the colour scatter
// into double-float pairs held in the FP64 accumulator's memory.
template <class Team, class Emit>
__device__ __noinline__ double bah_eval_df(Team& tm, const PotBAH& P, CView<double> cv, double* xw, double* GA,
                                           Emit* emp, bool want_e, bool want_g, float* hi, float* lo) {
  const int n = 3 * P.nvert;
  if (xw || !cv.p) {
    for (int i = tm.tid(); i < n; i += tm.nthr()) {
      const double v = cv(i);
      if (xw) xw[i] = v;
      const DF d = df_split_bits(v);
      hi[i] = d.hi;
      lo[i] = d.lo;
    }
  } else {
    const DFn t = DFn(cv.t);
    for (int i = tm.tid(); i < n; i += tm.nthr()) {
      const DFn d = DFn(df_split_bits(cv.x[i])) + t * DFn(cv.p[i]);
      hi[i] = d.hi;
      lo[i] = d.lo;
    }
  }
  tm.sync();
  return bah_eval_impl<double, DFn>(tm, P, DfSrc{hi, lo}, cv, (double*)nullptr,
                                    GaDF{reinterpret_cast<DF*>(GA)}, emp, want_e, want_g);
}

}  // namespace mg
