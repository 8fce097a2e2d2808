// ljcells.cuh -- Lennard-Jones with a cutoff, through a hashed cell list.
//
// No counterpart in the reference: LjNd sums every pair i < j
// (src/potentials/LjNd.cpp:12-26, 29-53) and stays the default here.  With a
// cutoff rc (LjNd::setCutoff) a pair contributes only when r^2 < rc^2, with
// the reference's pair terms otherwise unchanged (plain truncation).
//
// The pair set is defined by one FP64 criterion: r^2 = (dx^2 + dy^2) + dz^2
// in FP64, each operation rounded once (no fused multiply-add), of the
// coordinates the evaluation sees (FP32 values in the FP32 stage, FP64 in
// the FP64 stage) -- the same arithmetic as a plain CPU loop, so a CPU
// enumeration finds bitwise the same pairs.  The FP32 stage decides with an
// FP32 r^2 first and takes the FP64 test only inside a band of 1e-5 r_c^2
// around the cutoff (far wider than the FP32 rounding of r^2), so the FP64
// pipe (1/64 of the FP32 rate) is almost never used.
//
// Cells have side rc (1 + 1e-3); a particle's cell is floor(x / side) per
// dimension, computed in FP64 and clamped to +-2^20 (clamping never moves
// two particles apart, so no pair within rc is missed).  Cells are hashed
// into H = 2^hbits buckets (H >= 2N): no bounding box, no reduction.
// Build, every evaluation, on the team: each particle's bucket and cell key;
// bucket counts (atomics), a scan, a scatter, and each bucket sorted by
// particle index (so the order of every sum is fixed: results are
// deterministic).  Evaluation: one thread per particle, threads taking the
// particles in bucket order (neighbouring threads share neighbour cells);
// each of the 3^d neighbour cells is looked up by its hash and its bucket's
// particles are filtered by their cell key, so hash collisions cost time but
// never change the result.  Every pair is evaluated from both sides (no
// scatter of forces: each thread owns its particle's force); the energy
// counts the pair from its lower index.  A particle with a NaN coordinate
// makes the energy and its gradient NaN, as its pairs would in the
// all-pairs sum.
#pragma once

namespace mg {

constexpr int kCellBias = 1 << 20;

__device__ __forceinline__ int lj_cell_coord(double x, double inv_cs) {
  const double c = floor(x * inv_cs);
  // NaN and out-of-range values clamp to the ends
  if (!(c >= -(double)kCellBias)) return 0;
  if (c > (double)(kCellBias - 1)) return 2 * kCellBias - 1;
  return (int)c + kCellBias;
}
__device__ __forceinline__ unsigned long long lj_cell_key(int cx, int cy, int cz) {
  return ((unsigned long long)cx << 42) | ((unsigned long long)cy << 21) | (unsigned long long)cz;
}
__device__ __forceinline__ int lj_cell_hash(unsigned long long key, int hbits) {
  return (int)((key * 0x9E3779B97F4A7C15ull) >> (64 - hbits));
}

// the FP64 pair criterion's r^2 (one rounding per operation)
template <typename T>
__device__ __forceinline__ double lj_r2_fp64(T xi, T yi, T zi, T xj, T yj, T zj, bool three) {
  const double dx = __dsub_rn((double)xi, (double)xj), dy = __dsub_rn((double)yi, (double)yj);
  double r2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
  if (three) {
    const double dz = __dsub_rn((double)zi, (double)zj);
    r2 = __dadd_rn(r2, __dmul_rn(dz, dz));
  }
  return r2;
}

// The scratch's arrays: bucket starts (H + 1), cursors (H), the particles
// in bucket order (N), each particle's bucket (N), one int of padding, the
// 64-bit cell keys (N; P.cells is 256-byte aligned, the keys start on an
// even int offset)
__device__ __forceinline__ unsigned long long* lj_cell_keys(const PotLJ& P) {
  const int H = 1 << P.hbits;
  return reinterpret_cast<unsigned long long*>(P.cells + 2 * (size_t)H + 2 * (size_t)P.np + 2);
}

// Builds the cell list of the positions cv on the team (see above).
template <typename T, class Team>
__device__ void lj_cells_build(Team& tm, const PotLJ& P, CView<T> cv) {
  const int N = P.np, nd = P.ndim, H = 1 << P.hbits;
  int* start = P.cells;
  int* cursor = start + H + 1;
  int* order = cursor + H;
  int* bucket = order + N;
  unsigned long long* key = lj_cell_keys(P);
  for (int b = tm.tid(); b <= H; b += tm.nthr()) start[b] = 0;
  tm.sync();
  for (int i = tm.tid(); i < N; i += tm.nthr()) {
    const int cx = lj_cell_coord((double)cv(nd * i), P.inv_cs);
    const int cy = lj_cell_coord((double)cv(nd * i + 1), P.inv_cs);
    const int cz = nd == 3 ? lj_cell_coord((double)cv(nd * i + 2), P.inv_cs) : kCellBias;
    const unsigned long long k = lj_cell_key(cx, cy, cz);
    const int h = lj_cell_hash(k, P.hbits);
    key[i] = k;
    bucket[i] = h;
    atomicAdd(&start[h + 1], 1);
  }
  tm.sync();
  // inclusive scan of the counts start[1..H] by the first block: a chunk per
  // thread, the chunk totals scanned by warp shuffles, then the warps' totals
  if (tm.block0()) {
    __shared__ int wsum[32];
    const int nt = blockDim.x, t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int chunk = (H + nt - 1) / nt, b0 = 1 + t * chunk, b1 = min(H + 1, b0 + chunk);
    int s = 0;
    for (int b = b0; b < b1; b++) s += start[b];
    int incl = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    if (lane == 31 || t == nt - 1) wsum[w] = incl;
    __syncthreads();
    int before = incl - s;
    for (int k = 0; k < w; k++) before += wsum[k];
    for (int b = b0; b < b1; b++) {
      before += start[b];
      start[b] = before;
    }
    __syncthreads();
  }
  tm.sync();
  for (int b = tm.tid(); b < H; b += tm.nthr()) cursor[b] = start[b];
  tm.sync();
  for (int i = tm.tid(); i < N; i += tm.nthr()) order[atomicAdd(&cursor[bucket[i]], 1)] = i;
  tm.sync();
  // each bucket in particle order (buckets hold a few particles)
  for (int b = tm.tid(); b < H; b += tm.nthr()) {
    const int s0 = start[b], s1 = start[b + 1];
    for (int a = s0 + 1; a < s1; a++) {
      const int v = order[a];
      int c = a - 1;
      while (c >= s0 && order[c] > v) {
        order[c + 1] = order[c];
        c--;
      }
      order[c + 1] = v;
    }
  }
  tm.sync();
}

// Energy (pairs counted once) and, with want_g, the gradient of LjNd with a
// cutoff at the positions cv, through the cell list built above.  With
// pairs != NULL, the pairs i < j inside the cutoff are written instead
// (counter *npairs, at most cap; no energy or gradient).
template <typename T, class Team, class Emit>
__device__ __noinline__ double lj_cells_eval(Team& tm, const PotLJ& P, CView<T> cv, T* xw, Emit* emp,
                                             bool want_e, bool want_g, int2* pairs, int* npairs, int cap) {
  using L = LjC<T>;
  using C = typename L::C;
  Emit emit = *emp;
  const int N = P.np, nd = P.ndim, H = 1 << P.hbits;
  const bool three = nd == 3;
  if (xw) {
    for (int i = tm.tid(); i < N * nd; i += tm.nthr()) xw[i] = cv(i);
  }
  lj_cells_build<T>(tm, P, cv);
  const int* start = P.cells;
  const int* order = start + 2 * H + 1;
  const unsigned long long* key = lj_cell_keys(P);
  const C s6 = L::from((T)P.s6);
  const C zero = L::from((T)0);
  // the FP32 decision band around rc^2
  const float lo = (float)(P.rc2 * (1.0 - 1e-5)), hi = (float)(P.rc2 * (1.0 + 1e-5));
  LjAcc<C> e;
  bool bad = false;
  for (int t = tm.tid(); t < N; t += tm.nthr()) {
    const int i = order[t];
    const T xi = cv(nd * i), yi = cv(nd * i + 1), zi = three ? cv(nd * i + 2) : (T)0;
    const bool nan_i = isnan((double)xi) || isnan((double)yi) || isnan((double)zi);
    bad |= nan_i;
    const unsigned long long ki = key[i];
    const int cx = (int)(ki >> 42), cy = (int)((ki >> 21) & 0x1fffff), cz = (int)(ki & 0x1fffff);
    const C cxi = L::from(xi), cyi = L::from(yi), czi = L::from(zi);
    C fx = zero, fy = zero, fz = zero;
    for (int a = -1; a <= 1; a++) {
      if (cx + a < 0 || cx + a >= 2 * kCellBias) continue;
      for (int b = -1; b <= 1; b++) {
        if (cy + b < 0 || cy + b >= 2 * kCellBias) continue;
        for (int c = (three ? -1 : 0); c <= (three ? 1 : 0); c++) {
          if (cz + c < 0 || cz + c >= 2 * kCellBias) continue;
          const unsigned long long kn = lj_cell_key(cx + a, cy + b, cz + c);
          const int h = lj_cell_hash(kn, P.hbits);
          const int s1 = start[h + 1];
          for (int q = start[h]; q < s1; q++) {
            const int j = order[q];
            if (j == i || key[j] != kn) continue;
            const T xj = cv(nd * j), yj = cv(nd * j + 1), zj = three ? cv(nd * j + 2) : (T)0;
            bool in;
            if constexpr (std::is_same_v<T, float>) {
              const float dx = xi - xj, dy = yi - yj, dz = zi - zj;
              const float r2f = dx * dx + dy * dy + dz * dz;
              if (r2f < lo) in = true;
              else if (r2f > hi) in = false;
              else in = !(lj_r2_fp64<T>(xi, yi, zi, xj, yj, zj, three) >= P.rc2);
            } else {
              in = !(lj_r2_fp64<T>(xi, yi, zi, xj, yj, zj, three) >= P.rc2);
            }
            if (!in) continue;
            if (pairs) {
              if (j > i) {
                const int k = atomicAdd(npairs, 1);
                if (k < cap) pairs[k] = make_int2(i, j);
              }
              continue;
            }
            const C dx = cxi - L::from(xj), dy = cyi - L::from(yj), dz = czi - L::from(zj);
            C lj6, lj12, f;
            lj_pair(dx, dy, dz, s6, lj6, lj12, f);
            if (want_g) {
              fx = fx + dx * f;
              fy = fy + dy * f;
              fz = fz + dz * f;
            }
            if (want_e && j > i) e.add(lj12 - lj6);
          }
        }
      }
    }
    if (want_g && !pairs) {
      const double c = -24.0 * P.eps;
      if (nan_i) {
        emit(nd * i, (T)NAN);
        emit(nd * i + 1, (T)NAN);
        if (three) emit(nd * i + 2, (T)NAN);
      } else {
        emit(nd * i, L::scaled(c, fx));
        emit(nd * i + 1, L::scaled(c, fy));
        if (three) emit(nd * i + 2, L::scaled(c, fz));
      }
    }
  }
  tm.sync();
  *emp = emit;
  const double en = 4.0 * P.eps * e.total();
  return bad ? (double)NAN : en;
}

}  // namespace mg
