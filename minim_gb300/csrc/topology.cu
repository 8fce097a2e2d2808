// topology.cu -- BarAndHinge set-up on the device: the bond and hinge lists
// of a triangulation in the reference's order (BarAndHinge::computeBondList /
// computeHingeList, src/potentials/BarAndHinge.cpp:54-147), the element
// parameters (computeBondParams / computeHingeParams and the initial lengths
// and angles, src/potentials/BarAndHinge.cpp:150-248), and the vertex-
// disjoint colouring and ordering the evaluation kernels need.
//
// Bonds are the distinct vertex pairs of the triangles, sorted by (lower,
// higher) vertex; a bond's adjacent-triangle vertices follow in triangle
// order.  Hinges are the pairs of triangles (t1 < t2) that share exactly two
// vertices, sorted by (t1, t2).  Both orders come from bucketing by the
// lower index (count, scan, scatter) and sorting each small bucket, so no
// global sort is needed.  The colouring is the greedy pass in element order
// (on the host, one 64-bit mask per vertex), after which the device orders
// the elements by colour.  Every step is deterministic.
//
// Triangulations outside what this builder handles (out-of-range or repeated
// vertices in a triangle, more than 4 triangles on an edge, a vertex on more
// than 256 edge records, a colour beyond 63) are reported to the caller,
// which then uses the host builder (setup.cpp).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "topology.h"

namespace mg {
namespace {

constexpr int kMaxTriPerEdge = 4;
constexpr int kMaxThird = 4;
constexpr int kMaxBucket = 256;
constexpr int kT = 256;  // threads per block of the element kernels

enum Flag : int {
  F_RANGE = 1,      // a vertex index out of range
  F_DEGEN = 2,      // a triangle with a repeated vertex
  F_BUCKET = 4,     // a vertex bucket larger than kMaxBucket
  F_EDGE = 8,       // more than kMaxTriPerEdge triangles (or thirds) on an edge
  F_NOBOND = 16,    // a hinge without its bond (thickness rigidities)
  F_COLOURS = 32,   // more than 64 colours
};

struct EdgeRec {
  int lo, hi, t, c;  // edge (lo < hi) of triangle t, whose third vertex is c
};

inline int nblk(long long n, int t = kT) { return (int)((n + t - 1) / t); }

// ---- exclusive scan (one block walks the array in chunks of 4096) ------------
// out[0..n] with out[n] = total; one block keeps the order fixed.
__global__ void __launch_bounds__(1024) k_scan(const int* __restrict__ in, int* __restrict__ out, int n) {
  __shared__ int wsum[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int carry = 0;
  for (int base = 0; base < n; base += 4096) {
    const int i0 = base + 4 * (int)threadIdx.x;
    int v[4], s = 0;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      v[j] = i0 + j < n ? in[i0 + j] : 0;
      s += v[j];
    }
    int x = s;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, off);
      if (lane >= off) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    if (w == 0) {
      int ws = wsum[lane];
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, ws, off);
        if (lane >= off) ws += y;
      }
      wsum[lane] = ws;
    }
    __syncthreads();
    int ex = carry + (x - s) + (w ? wsum[w - 1] : 0);
#pragma unroll
    for (int j = 0; j < 4; j++) {
      if (i0 + j < n) out[i0 + j] = ex;
      ex += v[j];
    }
    carry += wsum[31];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[n] = carry;
}

// ---- bonds -------------------------------------------------------------------
__global__ void k_edges(const int* __restrict__ tris, int ntri, int nvert, EdgeRec* __restrict__ rec,
                        int* __restrict__ cnt, int* flags) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntri) return;
  const int v[3] = {tris[3 * t], tris[3 * t + 1], tris[3 * t + 2]};
  bool bad = false;
  for (int k = 0; k < 3; k++)
    if (v[k] < 0 || v[k] >= nvert) {
      atomicOr(flags, F_RANGE);
      bad = true;
    }
  if (!bad && (v[0] == v[1] || v[1] == v[2] || v[0] == v[2])) {
    atomicOr(flags, F_DEGEN);
    bad = true;
  }
  for (int k = 0; k < 3; k++) {
    EdgeRec r{-1, -1, t, -1};
    if (!bad) {
      const int a = v[k], b = v[(k + 1) % 3];
      r.lo = min(a, b);
      r.hi = max(a, b);
      r.c = v[(k + 2) % 3];
      atomicAdd(&cnt[r.lo], 1);
    }
    rec[3 * t + k] = r;
  }
}

__global__ void k_scatter_edges(const EdgeRec* __restrict__ rec, int nrec, const int* __restrict__ off,
                                int* __restrict__ cur, EdgeRec* __restrict__ bucket) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrec) return;
  const EdgeRec r = rec[i];
  if (r.lo < 0) return;
  bucket[off[r.lo] + atomicAdd(&cur[r.lo], 1)] = r;
}

__device__ __forceinline__ bool edge_less(const EdgeRec& a, const EdgeRec& b) {
  return a.hi != b.hi ? a.hi < b.hi : (a.t != b.t ? a.t < b.t : a.c < b.c);
}

// sorts vertex v's bucket by (hi, t, c) and counts its distinct bonds
__global__ void k_sort_edges(EdgeRec* __restrict__ bucket, const int* __restrict__ off, int nvert,
                             int* __restrict__ nbv, int* flags) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nvert) return;
  const int b = off[v], e = off[v + 1];
  if (e - b > kMaxBucket) {
    atomicOr(flags, F_BUCKET);
    nbv[v] = 0;
    return;
  }
  for (int i = b + 1; i < e; i++) {
    const EdgeRec x = bucket[i];
    int j = i - 1;
    while (j >= b && edge_less(x, bucket[j])) {
      bucket[j + 1] = bucket[j];
      j--;
    }
    bucket[j + 1] = x;
  }
  int n = 0;
  for (int i = b; i < e; i++)
    if (i == b || bucket[i].hi != bucket[i - 1].hi) n++;
  nbv[v] = n;
}

// bonds of vertex v (boff[v] ..): the pair, its adjacent-triangle vertices in
// triangle order, and its triangles
__global__ void k_bonds(const EdgeRec* __restrict__ bucket, const int* __restrict__ off, const int* __restrict__ boff,
                        int nvert, int2* __restrict__ bab, int* __restrict__ third, int* __restrict__ nthird,
                        int* __restrict__ btri, int* __restrict__ nbtri, int* flags) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nvert) return;
  const int b = off[v], e = off[v + 1];
  if (e - b > kMaxBucket) return;
  int idx = boff[v] - 1;
  for (int i = b; i < e; i++) {
    const EdgeRec r = bucket[i];
    if (i == b || r.hi != bucket[i - 1].hi) {
      idx++;
      bab[idx] = make_int2(v, r.hi);
      nthird[idx] = 0;
      nbtri[idx] = 0;
    }
    // third vertex, unless already in the bond (its two ends included)
    int nt = nthird[idx];
    bool seen = r.c == v || r.c == r.hi;
    for (int k = 0; k < nt && !seen; k++) seen = third[kMaxThird * idx + k] == r.c;
    if (!seen) {
      if (nt < kMaxThird) {
        third[kMaxThird * idx + nt] = r.c;
        nthird[idx] = nt + 1;
      } else {
        atomicOr(flags, F_EDGE);
      }
    }
    const int nb = nbtri[idx];
    if (nb == 0 || btri[kMaxTriPerEdge * idx + nb - 1] != r.t) {
      if (nb < kMaxTriPerEdge) {
        btri[kMaxTriPerEdge * idx + nb] = r.t;
        nbtri[idx] = nb + 1;
      } else {
        atomicOr(flags, F_EDGE);
      }
    }
  }
}

// ---- hinges --------------------------------------------------------------------
__global__ void k_pair_count(const int* __restrict__ nbtri, int nbond, int* __restrict__ pc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nbond) return;
  const int m = nbtri[i];
  pc[i] = m * (m - 1) / 2;
}

__global__ void k_pair_emit(const int* __restrict__ btri, const int* __restrict__ nbtri, const int* __restrict__ poff,
                            int nbond, int2* __restrict__ pairs, int* __restrict__ cnt1) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nbond) return;
  const int m = nbtri[i];
  int k = poff[i];
  for (int a = 0; a < m; a++)
    for (int b = a + 1; b < m; b++) {
      const int t1 = btri[kMaxTriPerEdge * i + a], t2 = btri[kMaxTriPerEdge * i + b];
      pairs[k++] = make_int2(t1, t2);  // t1 < t2: a bond's triangles are in order
      atomicAdd(&cnt1[t1], 1);
    }
}

__global__ void k_pair_scatter(const int2* __restrict__ pairs, int np, const int* __restrict__ toff,
                               int* __restrict__ cur, int* __restrict__ pb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const int2 p = pairs[i];
  pb[toff[p.x] + atomicAdd(&cur[p.x], 1)] = p.y;
}

// the hinge of triangles A, B when they share exactly two vertices: A's
// unshared vertex and the two after it in A's order, then B's unshared one
__device__ __forceinline__ bool hinge_nodes(const int* A, const int* B, int4& h) {
  bool sa[3] = {false, false, false}, sb[3] = {false, false, false};
  int ns = 0;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      if (A[i] == B[j]) {
        ns++;
        sa[i] = true;
        sb[j] = true;
      }
  if (ns != 2) return false;
  for (int i = 0; i < 3; i++)
    if (!sa[i]) {
      h.x = A[i];
      h.y = A[(i + 1) % 3];
      h.z = A[(i + 2) % 3];
    }
  for (int j = 0; j < 3; j++)
    if (!sb[j]) h.w = B[j];
  return true;
}

// sorts triangle t1's partners, drops repeats and pairs that are no hinge
__global__ void k_pair_sort(int* __restrict__ pb, const int* __restrict__ toff, int ntri, const int* __restrict__ tris,
                            int* __restrict__ hc, int* __restrict__ pn) {
  const int t1 = blockIdx.x * blockDim.x + threadIdx.x;
  if (t1 >= ntri) return;
  const int b = toff[t1], e = toff[t1 + 1];
  for (int i = b + 1; i < e; i++) {
    const int x = pb[i];
    int j = i - 1;
    while (j >= b && x < pb[j]) {
      pb[j + 1] = pb[j];
      j--;
    }
    pb[j + 1] = x;
  }
  int n = 0, h = 0;  // distinct partners (kept in front), hinges among them
  for (int i = b; i < e; i++) {
    if (i > b && pb[i] == pb[i - 1]) continue;
    const int t2 = pb[i];
    pb[b + n++] = t2;
    int4 hn;
    if (hinge_nodes(tris + 3 * t1, tris + 3 * t2, hn)) h++;
  }
  pn[t1] = n;
  hc[t1] = h;
}

__device__ __forceinline__ int find_bond(const int2* __restrict__ bab, const int* __restrict__ boff, int a, int b) {
  const int lo = min(a, b), hi = max(a, b);
  int l = boff[lo], r = boff[lo + 1] - 1;
  while (l <= r) {
    const int mid = (l + r) >> 1;
    const int y = bab[mid].y;
    if (y == hi) return mid;
    if (y < hi) l = mid + 1;
    else r = mid - 1;
  }
  return -1;
}

__global__ void k_hinges(const int* __restrict__ pb, const int* __restrict__ toff, const int* __restrict__ pn,
                         const int* __restrict__ hoff, int ntri, const int* __restrict__ tris,
                         const int2* __restrict__ bab, const int* __restrict__ boff, int4* __restrict__ hinges,
                         int* __restrict__ hbond) {
  const int t1 = blockIdx.x * blockDim.x + threadIdx.x;
  if (t1 >= ntri) return;
  const int b = toff[t1];
  int k = hoff[t1];
  for (int i = 0; i < pn[t1]; i++) {
    int4 hn;
    if (!hinge_nodes(tris + 3 * t1, tris + 3 * pb[b + i], hn)) continue;
    hinges[k] = hn;
    hbond[k] = find_bond(bab, boff, hn.y, hn.z);
    k++;
  }
}

// ---- element parameters (FP64, the reference's formulas) -----------------------
struct ParamIn {
  const double* x;  // coordinates, 3 per vertex
  double modulus, poisson;
  int n_th;
  const double* th;
  int n_kb;
  const double* kb;
  int n_kh;
  const double* kh;
  int n_l0;
  const double* l0;
  int n_t0;
  const double* t0;
};

__device__ __forceinline__ double thick(const ParamIn& P, int v) { return P.n_th == 1 ? P.th[0] : P.th[v]; }

// |b - a|^2 and the summed areas of the bond's adjacent triangles
__global__ void k_bond_geom(ParamIn P, const int2* __restrict__ bab, const int* __restrict__ third,
                            const int* __restrict__ nthird, int nbond, double* __restrict__ lsq,
                            double* __restrict__ asum) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nbond) return;
  const double* x1 = P.x + 3 * bab[i].x;
  const double* x2 = P.x + 3 * bab[i].y;
  const double d21[3] = {x2[0] - x1[0], x2[1] - x1[1], x2[2] - x1[2]};
  lsq[i] = d21[0] * d21[0] + d21[1] * d21[1] + d21[2] * d21[2];
  double a = 0.0;
  for (int k = 0; k < nthird[i]; k++) {
    const double* x3 = P.x + 3 * third[kMaxThird * i + k];
    const double d31[3] = {x3[0] - x1[0], x3[1] - x1[1], x3[2] - x1[2]};
    const double c[3] = {d21[1] * d31[2] - d21[2] * d31[1], d21[2] * d31[0] - d21[0] * d31[2],
                         d21[0] * d31[1] - d21[1] * d31[0]};
    a += fabs(sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2])) / 2;
  }
  asum[i] = a;
}

__global__ void k_bond_params(ParamIn P, const int2* __restrict__ bab, const double* __restrict__ lsq,
                              const double* __restrict__ asum, int nbond, double2* __restrict__ bpar) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nbond) return;
  const int a = bab[i].x, b = bab[i].y;
  double k;
  if (P.n_kb == 1) k = P.kb[0];
  else if (P.n_kb > 1) k = P.kb[i];
  else k = P.modulus * ((thick(P, a) + thick(P, b)) / 2) * (asum[i] / lsq[i]);
  double l0;
  if (P.n_l0 == 1) l0 = P.l0[0];
  else if (P.n_l0 > 1) l0 = P.l0[i];
  else {
    const double d[3] = {P.x[3 * a] - P.x[3 * b], P.x[3 * a + 1] - P.x[3 * b + 1], P.x[3 * a + 2] - P.x[3 * b + 2]};
    l0 = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  }
  bpar[i] = make_double2(k, l0);
}

__global__ void k_hinge_params(ParamIn P, const int4* __restrict__ hinges, const int* __restrict__ hbond,
                               const double* __restrict__ lsq, const double* __restrict__ asum, int nhinge,
                               double2* __restrict__ hpar, int* flags) {
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= nhinge) return;
  const int4 n = hinges[h];
  double k;
  if (P.n_kh == 1) k = P.kh[0];
  else if (P.n_kh > 1) k = P.kh[h];
  else {
    const int bi = hbond[h];
    if (bi < 0) {
      atomicOr(flags, F_NOBOND);
      k = 0.0;
    } else {
      const double t = (thick(P, n.x) + thick(P, n.y) + thick(P, n.z) + thick(P, n.w)) / 4;
      const double rig = P.modulus * (t * t * t) / (12 * (1 - P.poisson * P.poisson));
      k = rig * (lsq[bi] / asum[bi]);
    }
  }
  double t0;
  if (P.n_t0 == 1) t0 = P.t0[0];
  else if (P.n_t0 > 1) t0 = P.t0[h];
  else {
    const double *x1 = P.x + 3 * n.x, *x2 = P.x + 3 * n.y, *x3 = P.x + 3 * n.z, *x4 = P.x + 3 * n.w;
    double a[3], b[3], c[3];
    for (int d = 0; d < 3; d++) {
      a[d] = x2[d] - x1[d];
      b[d] = x3[d] - x2[d];
      c[d] = x4[d] - x3[d];
    }
    const double n1[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
    const double n2[3] = {b[1] * c[2] - b[2] * c[1], b[2] * c[0] - b[0] * c[2], b[0] * c[1] - b[1] * c[0]};
    const double cs = (n1[0] * n2[0] + n1[1] * n2[1] + n1[2] * n2[2]) /
                      (sqrt(n1[0] * n1[0] + n1[1] * n1[1] + n1[2] * n1[2]) *
                       sqrt(n2[0] * n2[0] + n2[1] * n2[1] + n2[2] * n2[2]));
    const double n1b3 = n1[0] * c[0] + n1[1] * c[1] + n1[2] * c[2];
    const double pi = 3.14159265358979323846;
    t0 = n1b3 >= 0 ? acos(cs) : 2 * pi - acos(cs);
  }
  hpar[h] = make_double2(k, t0);
}

// ---- fixed-DOF filter, colouring, colour order ---------------------------------
template <int PER>
__device__ __forceinline__ void nodes_of(const void* el, int e, int (&v)[PER]) {
  if constexpr (PER == 2) {
    const int2 b = static_cast<const int2*>(el)[e];
    v[0] = b.x;
    v[1] = b.y;
  } else {
    const int4 h = static_cast<const int4*>(el)[e];
    v[0] = h.x;
    v[1] = h.y;
    v[2] = h.z;
    v[3] = h.w;
  }
}

// keep[e] = 1 unless every coordinate of every vertex of e is fixed
template <int PER>
__global__ void k_keep(const void* __restrict__ el, int ne, const unsigned char* __restrict__ fixed,
                       int* __restrict__ keep) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  int v[PER];
  nodes_of<PER>(el, e, v);
  bool all = fixed != nullptr;
  for (int k = 0; k < PER && all; k++)
    for (int d = 0; d < 3; d++) all = all && fixed[3 * v[k] + d];
  keep[e] = all ? 0 : 1;
}

// kept element e goes to position kpos[e] of the compact list
template <int PER>
__global__ void k_compact(const void* __restrict__ el, const double2* __restrict__ par, int ne,
                          const int* __restrict__ keep, const int* __restrict__ kpos, void* __restrict__ el_out,
                          double2* __restrict__ par_out) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne || !keep[e]) return;
  if constexpr (PER == 2) static_cast<int2*>(el_out)[kpos[e]] = static_cast<const int2*>(el)[e];
  else static_cast<int4*>(el_out)[kpos[e]] = static_cast<const int4*>(el)[e];
  par_out[kpos[e]] = par[e];
}

// colour order: per block of 1024 elements, counts per colour
__global__ void __launch_bounds__(1024) k_colour_hist(const int* __restrict__ col, int ne, int* __restrict__ bc) {
  __shared__ int h[64];
  if (threadIdx.x < 64) h[threadIdx.x] = 0;
  __syncthreads();
  const int e = blockIdx.x * 1024 + threadIdx.x;
  if (e < ne) atomicAdd(&h[col[e]], 1);
  __syncthreads();
  if (threadIdx.x < 64) bc[blockIdx.x * 64 + threadIdx.x] = h[threadIdx.x];
}

// start of every (block, colour) run: colour-major over blocks in order
__global__ void k_colour_base(int* __restrict__ bc, int nb, int ncol, int* __restrict__ coff) {
  __shared__ int tot[64];
  const int c = threadIdx.x;
  int run = 0;
  if (c < 64)
    for (int b = 0; b < nb; b++) {
      const int x = bc[b * 64 + c];
      bc[b * 64 + c] = run;
      run += x;
    }
  if (c < 64) tot[c] = run;
  __syncthreads();
  if (c == 0) {
    int s = 0;
    for (int k = 0; k < ncol; k++) {
      coff[k] = s;
      s += tot[k];
    }
    coff[ncol] = s;
    for (int k = ncol; k < 64; k++) tot[k] = s;
  }
  __syncthreads();
  if (c < 64) {
    const int base = c < ncol ? coff[c] : coff[ncol];
    for (int b = 0; b < nb; b++) bc[b * 64 + c] += base;
  }
}

// position of element e: its colour's run in its block plus the elements of
// the same colour before it in the block
__global__ void __launch_bounds__(1024) k_colour_rank(const int* __restrict__ col, int ne, const int* __restrict__ bc,
                                                      int* __restrict__ perm) {
  __shared__ int wc[32][64];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < 32 * 64; i += 1024) (&wc[0][0])[i] = 0;
  __syncthreads();
  const int e = blockIdx.x * 1024 + threadIdx.x;
  const int c = e < ne ? col[e] : 64;
  const unsigned same = __match_any_sync(0xffffffffu, c);
  const int rank = __popc(same & ((1u << lane) - 1u));
  if (c < 64 && rank == 0) wc[w][c] = __popc(same);
  __syncthreads();
  if (threadIdx.x < 64) {
    int s = 0;
    for (int k = 0; k < 32; k++) {
      const int x = wc[k][threadIdx.x];
      wc[k][threadIdx.x] = s;
      s += x;
    }
  }
  __syncthreads();
  if (c < 64) perm[bc[blockIdx.x * 64 + c] + wc[w][c] + rank] = e;
}

template <int PER>
__global__ void k_gather(const void* __restrict__ el, const double2* __restrict__ par, const int* __restrict__ perm,
                         int ne, void* __restrict__ el_out, double2* __restrict__ par_out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= ne) return;
  const int e = perm[p];
  if constexpr (PER == 2) static_cast<int2*>(el_out)[p] = static_cast<const int2*>(el)[e];
  else static_cast<int4*>(el_out)[p] = static_cast<const int4*>(el)[e];
  par_out[p] = par[e];
}

__global__ void k_node_el(const unsigned char* __restrict__ fixed, int nvert, unsigned char* __restrict__ out) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nvert) return;
  out[v] = fixed ? (unsigned char)!(fixed[3 * v] && fixed[3 * v + 1] && fixed[3 * v + 2]) : (unsigned char)1;
}

// ---- host helpers ------------------------------------------------------------------
struct Scratch {
  cudaStream_t s;
  std::vector<void*> ptrs;
  cudaError_t err = cudaSuccess;
  template <typename T>
  T* alloc(size_t n) {
    void* p = nullptr;
    if (err == cudaSuccess) err = cudaMallocAsync(&p, (n ? n : 1) * sizeof(T), s);
    if (p) ptrs.push_back(p);
    return static_cast<T*>(p);
  }
  template <typename T>
  T* zeros(size_t n) {
    T* p = alloc<T>(n);
    if (err == cudaSuccess) err = cudaMemsetAsync(p, 0, (n ? n : 1) * sizeof(T), s);
    return p;
  }
  template <typename T>
  T* upload(const T* h, size_t n) {
    T* p = alloc<T>(n);
    if (err == cudaSuccess && n) err = cudaMemcpyAsync(p, h, n * sizeof(T), cudaMemcpyHostToDevice, s);
    return p;
  }
  int read(const int* d) {
    int v = 0;
    if (err == cudaSuccess) err = cudaMemcpyAsync(&v, d, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    return v;
  }
  void scan(const int* in, int* out, int n) {
    if (err == cudaSuccess) {
      k_scan<<<1, 1024, 0, s>>>(in, out, n);
      err = cudaGetLastError();
    }
  }
  // take p out of the scratch list (the caller owns it)
  void keep(void* p) {
    for (auto& q : ptrs)
      if (q == p) q = nullptr;
  }
  ~Scratch() {
    for (void* p : ptrs)
      if (p) cudaFreeAsync(p, s);
  }
};

// MINIM_GPU_BAH_SETUP_TIMING: host wall time of the set-up's phases (each
// phase ends at a synchronising read) printed to stderr
struct PhaseClock {
  bool on = std::getenv("MINIM_GPU_BAH_SETUP_TIMING") != nullptr;
  std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
  void mark(const char* what) {
    if (!on) return;
    const auto now = std::chrono::steady_clock::now();
    std::fprintf(stderr, "bah set-up %-22s %8.3f ms\n", what,
                 std::chrono::duration<double, std::milli>(now - t).count());
    t = now;
  }
};

void set_err(char* err, int len, const char* msg) {
  if (err && len > 0) std::snprintf(err, (size_t)len, "%s", msg);
}

template <int PER>
int colour_elements(Scratch& S, const void* el, const double2* par, int ne, int nvert,
                    const unsigned char* d_fixed, void** el_out, double2** par_out, int** off_out, int* ncol_out,
                    int* ne_out, int* flags) {
  const size_t esz = PER == 2 ? sizeof(int2) : sizeof(int4);
  // drop elements with every coordinate fixed
  int* keep = S.alloc<int>(ne);
  int* kpos = S.alloc<int>((size_t)ne + 1);
  if (S.err == cudaSuccess && ne) k_keep<PER><<<nblk(ne), kT, 0, S.s>>>(el, ne, d_fixed, keep);
  S.scan(keep, kpos, ne);
  PhaseClock clk;
  const int nk = S.read(kpos + ne);
  clk.mark(PER == 2 ? "bars kept" : "hinges kept");
  void* ek = S.alloc<char>((size_t)nk * esz);
  double2* pk = S.alloc<double2>(nk);
  if (S.err == cudaSuccess && ne) k_compact<PER><<<nblk(ne), kT, 0, S.s>>>(el, par, ne, keep, kpos, ek, pk);
  // greedy colouring in element order on the host (one 64-bit mask of used
  // colours per vertex): a sequential pass whose colour count the parallel
  // schemes tried here did not reach on meshes (a 100k-vertex sheet: 8 bar
  // and 19 hinge colours against 6 and 13), and every colour costs the
  // gradient scatter one barrier
  std::vector<char> he((size_t)nk * esz);
  if (S.err == cudaSuccess && nk) S.err = cudaMemcpyAsync(he.data(), ek, he.size(), cudaMemcpyDeviceToHost, S.s);
  if (S.err == cudaSuccess) S.err = cudaStreamSynchronize(S.s);
  std::vector<int> hc(nk);
  std::vector<unsigned long long> used(nvert, 0ull);
  int ncol = 0;
  for (int e = 0; e < nk && S.err == cudaSuccess; e++) {
    const int* v = reinterpret_cast<const int*>(he.data() + (size_t)e * esz);
    unsigned long long forb = 0;
    for (int k = 0; k < PER; k++) forb |= used[v[k]];
    if (forb == ~0ull) return 1;  // more than 64 colours: the host builder's multi-word greedy
    int c = 0;
    while (forb & (1ull << c)) c++;
    hc[e] = c;
    ncol = c + 1 > ncol ? c + 1 : ncol;
    for (int k = 0; k < PER; k++) used[v[k]] |= 1ull << c;
  }
  clk.mark(PER == 2 ? "bars coloured" : "hinges coloured");
  int* col = S.upload(hc.data(), (size_t)nk);
  // order by colour (element order within a colour)
  const int nbk = nblk(nk, 1024);
  int* bc = S.alloc<int>((size_t)(nbk ? nbk : 1) * 64);
  int* off = S.alloc<int>(65);
  int* perm = S.alloc<int>(nk);
  void* eo = S.alloc<char>((size_t)nk * esz);
  double2* po = S.alloc<double2>(nk);
  if (S.err == cudaSuccess && nk) {
    k_colour_hist<<<nbk, 1024, 0, S.s>>>(col, nk, bc);
    k_colour_base<<<1, 64, 0, S.s>>>(bc, nbk, ncol, off);
    k_colour_rank<<<nbk, 1024, 0, S.s>>>(col, nk, bc, perm);
    k_gather<PER><<<nblk(nk), kT, 0, S.s>>>(ek, pk, perm, nk, eo, po);
    S.err = cudaGetLastError();
  } else if (S.err == cudaSuccess) {
    S.err = cudaMemsetAsync(off, 0, sizeof(int), S.s);
  }
  if (clk.on && S.err == cudaSuccess) S.err = cudaStreamSynchronize(S.s);
  clk.mark(PER == 2 ? "bars ordered" : "hinges ordered");
  if (clk.on) std::fprintf(stderr, "bah set-up %s: %d colours\n", PER == 2 ? "bars" : "hinges", ncol);
  S.keep(eo);
  S.keep(po);
  S.keep(off);
  *el_out = eo;
  *par_out = po;
  *off_out = off;
  *ncol_out = ncol;
  *ne_out = nk;
  return 0;
}

}  // namespace
}  // namespace mg

using namespace mg;

extern "C" int mg_bah_topology_device(const minim_gpu_bah_params* q, const double* x0, int nvert, BahTopoDev* out,
                                      void* stream, char* err, int errlen) {
  if (q->ntri <= 0 || q->nbond > 0 || q->nhinge > 0) return MG_TOPO_HOST;
  const bool have_kb = q->n_kbond > 0, have_kh = q->n_khinge > 0;
  if ((!have_kb || !have_kh) && q->n_thickness <= 0) {
    set_err(err, errlen, "BarAndHinge requires either the rigidities or the thickness to be set");
    return MG_TOPO_INVALID;
  }
  if (q->n_thickness > 1 && q->n_thickness < nvert) {
    set_err(err, errlen, "BarAndHinge: thickness must have 1 or nvert entries");
    return MG_TOPO_INVALID;
  }
  Scratch S;
  S.s = static_cast<cudaStream_t>(stream);
  const int ntri = q->ntri, nrec = 3 * ntri;
  int* flags = S.zeros<int>(1);
  const int* tris = S.upload(q->tris, (size_t)3 * ntri);
  // bonds
  EdgeRec* rec = S.alloc<EdgeRec>(nrec);
  EdgeRec* bucket = S.alloc<EdgeRec>(nrec);
  int* cnt = S.zeros<int>(nvert);
  int* cur = S.zeros<int>(nvert);
  int* off = S.alloc<int>((size_t)nvert + 1);
  int* nbv = S.alloc<int>(nvert);
  int* boff = S.alloc<int>((size_t)nvert + 1);
  if (S.err == cudaSuccess) {
    k_edges<<<nblk(ntri), kT, 0, S.s>>>(tris, ntri, nvert, rec, cnt, flags);
    S.err = cudaGetLastError();
  }
  S.scan(cnt, off, nvert);
  if (S.err == cudaSuccess) {
    k_scatter_edges<<<nblk(nrec), kT, 0, S.s>>>(rec, nrec, off, cur, bucket);
    k_sort_edges<<<nblk(nvert), kT, 0, S.s>>>(bucket, off, nvert, nbv, flags);
    S.err = cudaGetLastError();
  }
  S.scan(nbv, boff, nvert);
  PhaseClock clk;
  const int nb = S.read(boff + nvert);
  clk.mark("bonds counted");
  if (S.err != cudaSuccess) return MG_TOPO_CUDA;
  if (S.read(flags)) return MG_TOPO_HOST;
  int2* bab = S.alloc<int2>(nb);
  int* third = S.alloc<int>((size_t)nb * kMaxThird);
  int* nthird = S.alloc<int>(nb);
  int* btri = S.alloc<int>((size_t)nb * kMaxTriPerEdge);
  int* nbtri = S.alloc<int>(nb);
  if (S.err == cudaSuccess && nvert) {
    k_bonds<<<nblk(nvert), kT, 0, S.s>>>(bucket, off, boff, nvert, bab, third, nthird, btri, nbtri, flags);
    S.err = cudaGetLastError();
  }
  // hinges
  int* pc = S.alloc<int>(nb);
  int* poff = S.alloc<int>((size_t)nb + 1);
  if (S.err == cudaSuccess && nb) {
    k_pair_count<<<nblk(nb), kT, 0, S.s>>>(nbtri, nb, pc);
    S.err = cudaGetLastError();
  }
  S.scan(pc, poff, nb);
  const int np = S.read(poff + nb);
  clk.mark("bonds written");
  if (S.err != cudaSuccess) return MG_TOPO_CUDA;
  if (S.read(flags)) return MG_TOPO_HOST;
  int2* pairs = S.alloc<int2>(np);
  int* cnt1 = S.zeros<int>(ntri);
  int* cur1 = S.zeros<int>(ntri);
  int* toff = S.alloc<int>((size_t)ntri + 1);
  int* pb = S.alloc<int>(np);
  int* hc = S.alloc<int>(ntri);
  int* pn = S.alloc<int>(ntri);
  int* hoff = S.alloc<int>((size_t)ntri + 1);
  if (S.err == cudaSuccess && nb) {
    k_pair_emit<<<nblk(nb), kT, 0, S.s>>>(btri, nbtri, poff, nb, pairs, cnt1);
    S.err = cudaGetLastError();
  }
  S.scan(cnt1, toff, ntri);
  if (S.err == cudaSuccess) {
    if (np) k_pair_scatter<<<nblk(np), kT, 0, S.s>>>(pairs, np, toff, cur1, pb);
    k_pair_sort<<<nblk(ntri), kT, 0, S.s>>>(pb, toff, ntri, tris, hc, pn);
    S.err = cudaGetLastError();
  }
  S.scan(hc, hoff, ntri);
  const int nh = S.read(hoff + ntri);
  clk.mark("hinges counted");
  if (S.err != cudaSuccess) return MG_TOPO_CUDA;
  // per-element arrays of the wrong length are the caller's error
  auto wrong = [&](int n, int want, const char* what) {
    if (n > 1 && n != want) {
      char m[96];
      std::snprintf(m, sizeof m, "BarAndHinge: %s has the wrong size", what);
      set_err(err, errlen, m);
      return true;
    }
    return false;
  };
  if (wrong(q->n_kbond, nb, "kBond") || wrong(q->n_khinge, nh, "kHinge") || wrong(q->n_length0, nb, "length0") ||
      wrong(q->n_theta0, nh, "theta0"))
    return MG_TOPO_INVALID;
  int4* hinges = S.alloc<int4>(nh);
  int* hbond = S.alloc<int>(nh);
  if (S.err == cudaSuccess && ntri) {
    k_hinges<<<nblk(ntri), kT, 0, S.s>>>(pb, toff, pn, hoff, ntri, tris, bab, boff, hinges, hbond);
    S.err = cudaGetLastError();
  }
  // parameters
  ParamIn P{};
  P.x = S.upload(x0, (size_t)3 * nvert);
  P.modulus = q->modulus;
  P.poisson = q->poisson_ratio;
  P.n_th = q->n_thickness;
  P.th = q->n_thickness > 0 ? S.upload(q->thickness, (size_t)(q->n_thickness == 1 ? 1 : nvert)) : nullptr;
  P.n_kb = q->n_kbond;
  P.kb = q->n_kbond > 0 ? S.upload(q->kbond, (size_t)q->n_kbond) : nullptr;
  P.n_kh = q->n_khinge;
  P.kh = q->n_khinge > 0 ? S.upload(q->khinge, (size_t)q->n_khinge) : nullptr;
  P.n_l0 = q->n_length0;
  P.l0 = q->n_length0 > 0 ? S.upload(q->length0, (size_t)q->n_length0) : nullptr;
  P.n_t0 = q->n_theta0;
  P.t0 = q->n_theta0 > 0 ? S.upload(q->theta0, (size_t)q->n_theta0) : nullptr;
  double* lsq = S.alloc<double>(nb);
  double* asum = S.alloc<double>(nb);
  double2* bpar = S.alloc<double2>(nb);
  double2* hpar = S.alloc<double2>(nh);
  if (S.err == cudaSuccess) {
    if (nb) k_bond_geom<<<nblk(nb), kT, 0, S.s>>>(P, bab, third, nthird, nb, lsq, asum);
    if (nb) k_bond_params<<<nblk(nb), kT, 0, S.s>>>(P, bab, lsq, asum, nb, bpar);
    if (nh) k_hinge_params<<<nblk(nh), kT, 0, S.s>>>(P, hinges, hbond, lsq, asum, nh, hpar, flags);
    S.err = cudaGetLastError();
  }
  const int fl = S.read(flags);
  clk.mark("hinges and parameters");
  if (S.err != cudaSuccess) return MG_TOPO_CUDA;
  if (fl & F_NOBOND) {
    set_err(err, errlen, "The hingeList should contain the index of the bond.");
    return MG_TOPO_INVALID;
  }
  if (fl) return MG_TOPO_HOST;
  S.keep(bab);
  S.keep(bpar);
  S.keep(hinges);
  S.keep(hpar);
  out->nvert = nvert;
  out->nbar = nb;
  out->nhinge = nh;
  out->bars = bab;
  out->bpar = bpar;
  out->hinges = hinges;
  out->hpar = hpar;
  return MG_TOPO_OK;
}

extern "C" int mg_bah_colour_device(const BahTopoDev* t, const unsigned char* fixed, BahColouredDev* out,
                                    void* stream) {
  Scratch S;
  S.s = static_cast<cudaStream_t>(stream);
  *out = BahColouredDev{};
  // on failure the outputs made so far are freed
  auto fail = [&](int code) {
    void* ps[7] = {out->bars, out->bpar, out->bar_off, out->hinges, out->hpar, out->hinge_off, out->node_el};
    for (void* p : ps)
      if (p) cudaFreeAsync(p, S.s);
    *out = BahColouredDev{};
    return code;
  };
  int* flags = S.zeros<int>(1);
  const unsigned char* d_fixed = fixed ? S.upload(fixed, (size_t)3 * t->nvert) : nullptr;
  void* el = nullptr;
  int rc = colour_elements<2>(S, t->bars, t->bpar, t->nbar, t->nvert, d_fixed, &el, &out->bpar, &out->bar_off,
                              &out->nbar_colors, &out->nbar, flags);
  out->bars = static_cast<int2*>(el);
  if (rc) return fail(MG_TOPO_HOST);
  if (S.err != cudaSuccess) return fail(MG_TOPO_CUDA);
  el = nullptr;
  rc = colour_elements<4>(S, t->hinges, t->hpar, t->nhinge, t->nvert, d_fixed, &el, &out->hpar, &out->hinge_off,
                          &out->nhinge_colors, &out->nhinge, flags);
  out->hinges = static_cast<int4*>(el);
  if (rc) return fail(MG_TOPO_HOST);
  out->node_el = S.alloc<unsigned char>(t->nvert);
  if (S.err == cudaSuccess) {
    k_node_el<<<nblk(t->nvert), kT, 0, S.s>>>(d_fixed, t->nvert, out->node_el);
    S.err = cudaGetLastError();
  }
  S.keep(out->node_el);
  const int fl = S.read(flags);
  if (S.err != cudaSuccess) return fail(MG_TOPO_CUDA);
  return fl ? fail(MG_TOPO_HOST) : MG_TOPO_OK;
}

extern "C" void mg_bah_free_device(void* p, void* stream) {
  if (p) cudaFreeAsync(p, static_cast<cudaStream_t>(stream));
}
