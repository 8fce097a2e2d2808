// stepped.cu -- the FP32 stage of an L-BFGS minimisation of one large binary
// PhaseField as a CUDA graph of phase kernels.
//
// The persistent grid kernel holds every phase of the minimiser in one
// function, so its register budget (128 per thread, 16 warps per SM) is set
// by the heaviest phase and its sweeps are latency-bound.  Here each phase
// is its own kernel with its own register allocation and occupancy, and the
// control flow stays on the device: one graph launch runs up to `slice`
// iterations as
//
//   begin -> WHILE(outer) { dirA -> dirB -> WHILE(line search) { trial } ->
//                           IF(no trial accepted) { grad } }
//
// A trial evaluates the energy and, in the same pass, the gradient at its
// point; when the trial is accepted that gradient is the accepted point's
// (the same values the reference's separate gradient call computes), so the
// gradient kernel runs only after a line search that accepted no trial.
//
// Each phase kernel writes one row of partial sums per block; the block that
// finishes last runs the phase's controller: it sums the rows in a fixed
// order, runs the scalar parts
// of Lbfgs::iteration / getDirection / backtrackingLinesearch
// (src/minimisers/Lbfgs.cpp:41-133, src/minimisers/linesearch.cpp:8-30) on
// the instance's state record, and set the loops' conditions.  Both loops
// are bounded: the line search by its 10 trials, the outer loop by `slice`
// iterations per launch.
//
// The first iteration and everything outside the FP32 stage (the switch to
// FP64 coordinates, convergence and NaN handling) stay with the persistent
// kernel: at the end of each iteration the controller decides on copies of
// the policy counters whether the minimisation simply continues; if not, it
// leaves the end-of-iteration bookkeeping to the persistent kernel (state
// `resume`), which redoes it from the same state.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <vector>

#include "kernels.cuh"

namespace mg {
namespace {

struct FlatTeam {
  __device__ __forceinline__ int tid() const { return blockIdx.x * blockDim.x + threadIdx.x; }
  __device__ __forceinline__ int nthr() const { return gridDim.x * blockDim.x; }
};

constexpr int kGroup = 16;       // blocks per group of the grouped row sums
constexpr int kMaxGroups = 128;  // groups per launch (2048 blocks)

// Device control block of the stepped path (one per instance).
struct StepCtl {
  double t, thr, e0;         // line search: multiplier, Armijo threshold, energy at x
  double kernels;            // kernel executions (launch count)
  unsigned long long tmark;  // %globaltimer at the end of the last controller
  int k, exhausted;          // trials so far; the policy's "line search exhausted"
  int iters, slice;          // iterations in this launch, at most `slice`
  int mt;                    // pairs used by this iteration's direction
  int gmode;                 // two-trial graph: the next trial pass is the gradient at t only
  int retry;                 // two-trial graph: the next outer pass only continues the line search
  int fresh;                 // two-trial graph: the next trial pass is the first of a new direction
  float fg;                  // -gamma
  float coefS[MINIM_MAXM], coefY[MINIM_MAXM];
  int so[MINIM_MAXM], yo[MINIM_MAXM];  // slot buffers: float4 offsets from the ring bases
  // stencil kernels' span (first block's start, last block's end), split
  // into the gap before, the kernel and the controller work after;
  // [0] trials, [1] gradient, [2] direction pass A, [3] direction pass B
  unsigned long long ks, ke;
  unsigned kdone;
  unsigned gdone[kMaxGroups];  // grouped row sums: blocks of each group done
  double gap_pre[4], kdur[4], gap_post[4];
  double work[4];         // the controllers' scalar work (span_end to phase_mark)
  int timing;             // record the spans above (MINIM_GPU_STEPPED_TIMING)
  unsigned long long tw;  // start of the current controller's scalar work
  int cur;                // its span slot
  unsigned acc_hist[11];  // iterations by the trial accepted (10: none)
  int tma_err;            // TMA trial pass: a copy wait gave up (1) or no tensor map fits a buffer (2)
};

// adds the last phase kernel's span to slot j of the span records
__device__ __forceinline__ void span_end(StepCtl* ctl, int j) {
  if (!ctl->timing) return;
  const unsigned long long now = globaltimer_ns();
  ctl->gap_pre[j] += (double)(ctl->ks - ctl->tmark);
  ctl->kdur[j] += (double)(ctl->ke - ctl->ks);
  ctl->gap_post[j] += (double)(now - ctl->ke);
  ctl->tw = now;
  ctl->cur = j;
}

// span bookkeeping of a stencil kernel (first block in, last block out)
__device__ __forceinline__ void span_begin(StepCtl* ctl) {
  if (blockIdx.x == 0 && threadIdx.x == 0 && threadIdx.y == 0) ctl->ks = globaltimer_ns();
}
// True, in every thread, in the block that finishes last: the blocks count
// themselves out after writing their partial rows; the last one also marks
// the kernel's end and sees every other block's row.
__device__ __forceinline__ bool last_block(StepCtl* ctl) {
  __shared__ int is_last;
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    __threadfence();
    is_last = atomicAdd(&ctl->kdone, 1u) == gridDim.x - 1;
    if (is_last) {
      ctl->ke = globaltimer_ns();
      ctl->kdone = 0;
      __threadfence();
    }
  }
  __syncthreads();
  return is_last != 0;
}

// Two-level form of last_block for wide rows: the last block of each group
// of kGroup blocks sums the group's rows in order into row `group` of part2;
// the block that completes the last group returns true, with the totals to
// be summed from the ngroups rows of part2 (the final sum reads ngroups rows
// instead of one per block, which is what makes a single block's sum of
// many wide rows slow).
__device__ inline bool last_block_grouped(StepCtl* ctl, const double* part, double* part2, int K,
                                          double* wide, double* rowbuf) {
  __shared__ int flag;
  const int nb = gridDim.x, g = blockIdx.x / kGroup, g0 = g * kGroup;
  const int members = min(kGroup, nb - g0), ngroups = (nb + kGroup - 1) / kGroup;
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    __threadfence();
    flag = atomicAdd(&ctl->gdone[g], 1u) == (unsigned)(members - 1);
    if (flag) ctl->gdone[g] = 0;
  }
  __syncthreads();
  if (!flag) return false;
  sum_rows_fixed(part + (size_t)g0 * MINIM_WIDE, members, K, rowbuf, wide);
  __syncthreads();
  const int tl = threadIdx.y * blockDim.x + threadIdx.x;
  for (int k = tl; k < K; k += blockDim.x * blockDim.y) part2[(size_t)g * MINIM_WIDE + k] = rowbuf[k];
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    __threadfence();
    flag = atomicAdd(&ctl->kdone, 1u) == (unsigned)(ngroups - 1);
    if (flag) {
      ctl->ke = globaltimer_ns();
      ctl->kdone = 0;
      __threadfence();
    }
  }
  __syncthreads();
  return flag != 0;
}

constexpr int kThreads = 256;

// One row of K <= 4 block sums (deterministic: warp butterflies, then warps
// in order).
template <int K>
__device__ void block_row(double (&v)[K], double* row) {
  __shared__ double red[kThreads / 32][K < 4 ? 4 : K];
  // linear thread index (blocks may be 2-D); the block has whole warps
  const int tl = threadIdx.y * blockDim.x + threadIdx.x;
  const int lane = tl & 31, w = tl >> 5, nw = (blockDim.x * blockDim.y) >> 5;
#pragma unroll
  for (int k = 0; k < K; k++) v[k] = warp_sum(v[k]);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < K; k++) red[w][k] = v[k];
  __syncthreads();
  if (tl < K) {
    double s = 0.0;
    for (int i = 0; i < nw; i++) s += red[i][tl];
    row[tl] = s;
  }
}

// The controllers mirror the state record and the control block in shared
// memory: every thread of the block loads a few words (issued before the
// partial rows are summed, so both wait on one memory round trip), thread 0
// (warp 0 for pass A) runs the scalar logic on the copies, and every thread
// writes them back.  Thread 0 working on global memory directly made one L2
// round trip per dependent access (its own stores evict the lines it reads).
struct Mirror {
  MinScalars st;
  StepCtl ctl;
};
constexpr int kMirrorWords = (int)(sizeof(Mirror) / 8);
static_assert(sizeof(MinScalars) % 8 == 0 && sizeof(StepCtl) % 8 == 0, "mirror copies 8-byte words");
constexpr int kMirrorRegs = 6;  // words per thread held in registers (blocks of >= 128 threads)
struct MirrorRegs {
  unsigned long long w[kMirrorRegs];
};
__device__ __forceinline__ const unsigned long long* mirror_src(const MinScalars* st, const StepCtl* ctl, int i) {
  constexpr int ns = (int)(sizeof(MinScalars) / 8);
  return i < ns ? reinterpret_cast<const unsigned long long*>(st) + i
                : reinterpret_cast<const unsigned long long*>(ctl) + (i - ns);
}
__device__ __forceinline__ MirrorRegs mirror_load(const MinScalars* st, const StepCtl* ctl) {
  const int tl = threadIdx.y * blockDim.x + threadIdx.x, nt = blockDim.x * blockDim.y;
  MirrorRegs r;
#pragma unroll
  for (int k = 0; k < kMirrorRegs; k++) {
    const int i = tl + k * nt;
    r.w[k] = i < kMirrorWords ? __ldcg(mirror_src(st, ctl, i)) : 0ull;
  }
  return r;
}
__device__ __forceinline__ void mirror_store(Mirror* m, const MirrorRegs& r, const MinScalars* st,
                                             const StepCtl* ctl) {
  const int tl = threadIdx.y * blockDim.x + threadIdx.x, nt = blockDim.x * blockDim.y;
#pragma unroll
  for (int k = 0; k < kMirrorRegs; k++) {
    const int i = tl + k * nt;
    if (i < kMirrorWords) reinterpret_cast<unsigned long long*>(m)[i] = r.w[k];
  }
  // words past the register batch (small blocks only)
  for (int i = tl + kMirrorRegs * nt; i < kMirrorWords; i += nt)
    reinterpret_cast<unsigned long long*>(m)[i] = __ldcg(mirror_src(st, ctl, i));
}
__device__ __forceinline__ void mirror_out(const Mirror* m, MinScalars* st, StepCtl* ctl) {
  const int tl = threadIdx.y * blockDim.x + threadIdx.x, nt = blockDim.x * blockDim.y;
  for (int i = tl; i < kMirrorWords; i += nt)
    *const_cast<unsigned long long*>(mirror_src(st, ctl, i)) = reinterpret_cast<const unsigned long long*>(m)[i];
}

// controllers, run by the last block of each phase kernel (defined below)
__device__ void ctl_a(const InstDesc* __restrict__ d, MinScalars* st, StepCtl* ctl, const double* part, int nb);
__device__ void ctl_b(const InstDesc* __restrict__ d, MinScalars* st, StepCtl* ctl, const double* part, int nb,
                      cudaGraphConditionalHandle ls, cudaGraphConditionalHandle grad, int spec);
__device__ void ctl_ls(const InstDesc* __restrict__ d, MinScalars* st, StepCtl* ctl, const double* part, int nb,
                       cudaGraphConditionalHandle ls);
__device__ void ctl_g(const InstDesc* __restrict__ d, MinScalars* st, StepCtl* ctl, const double* part, int nb,
                      cudaGraphConditionalHandle outer);
__device__ void ctl_lsg(const InstDesc* __restrict__ d, MinScalars* st, StepCtl* ctl, const double* part,
                        int nb, cudaGraphConditionalHandle ls, cudaGraphConditionalHandle grad,
                        cudaGraphConditionalHandle outer);
__device__ void ctl_lsg2(const InstDesc* __restrict__ d, MinScalars* st, StepCtl* ctl, const double* part,
                         int nb, cudaGraphConditionalHandle outer);

// ---- vector and stencil kernels -------------------------------------------------

// S_k.g, Y_k.g, S_k.y_new, Y_k.y_new for the pairs of this iteration (row
// layout: dot * 16 + pair in age order).  M (= Lbfgs m) is a compile-time
// constant so that every load of a sweep step is unconditional and can be
// issued before any is used: pairs not yet stored (the first m - 1
// iterations) read g instead, and their sums are ignored.  The block's
// threads split into NG parts of at most 8 pairs each (balanced sizes).
// Offsets are signed: g lies below the ring buffers in the workspace.
template <int M>
__global__ void __launch_bounds__(kThreads, 4)
k_dir_a(const InstDesc* __restrict__ d, MinScalars* st, StepCtl* ctl, double* part) {
  if (ctl->retry) return;  // this pass of the loop only continues a line search
  span_begin(ctl);
  constexpr int NG = (M + 7) / 8;
  constexpr int GS = (M + NG - 1) / NG;  // pairs per part
  __shared__ double wide[8 * MINIM_WIDE];
  __shared__ int so[16], yo[16];
  const int n = d->ndof;
  const long long hs = d->hstride;
  const int ii = st->ii + 1, mt = ii < M ? ii : M, c = ii % M;
  const int pend = st->pend;
  const bool np = pend >= 0;
  const float* G = d->G[st->gi];
  const float* Yn = np ? d->Yb + (long long)st->yidx[pend] * hs : G;
  const float4* Sb4 = reinterpret_cast<const float4*>(d->Sb);
  const float4* Yb4 = reinterpret_cast<const float4*>(d->Yb);
  const int gS = (int)(reinterpret_cast<const float4*>(G) - Sb4);
  const int gY = (int)(reinterpret_cast<const float4*>(G) - Yb4);
  if (threadIdx.x < 16) {
    const int k = threadIdx.x;
    if (k < mt) {
      const int s = (c - mt + k + 2 * M) % M;
      so[k] = (int)(((long long)st->sidx[s] * hs) >> 2);
      yo[k] = (int)(((long long)st->yidx[s] * hs) >> 2);
    } else {
      so[k] = gS;
      yo[k] = gY;
    }
  }
  __syncthreads();
  const int psz = (blockDim.x / NG) & ~31;
  const int part_ = min((int)threadIdx.x / psz, NG - 1);
  const int k0 = GS * part_;
  const int pt = threadIdx.x - part_ * psz;
  float acc[4 * GS];
#pragma unroll
  for (int k = 0; k < 4 * GS; k++) acc[k] = 0.f;
  int o_s[GS], o_y[GS];
#pragma unroll
  for (int j = 0; j < GS; j++) {
    o_s[j] = so[min(k0 + j, 15)];
    o_y[j] = yo[min(k0 + j, 15)];
  }
  const int nq4 = n >> 2;
  const bool active = (int)threadIdx.x < NG * psz;
  if (active) {
    for (int i = blockIdx.x * psz + pt; i < nq4; i += gridDim.x * psz) {
      const float4 g = ld4(G, i);
      const float4 yn = ld4(Yn, i);
      float4 sv[GS], yv[GS];
#pragma unroll
      for (int j = 0; j < GS; j++) {
        sv[j] = Sb4[o_s[j] + i];
        yv[j] = Yb4[o_y[j] + i];
      }
#pragma unroll
      for (int j = 0; j < GS; j++) {
        acc[j] += dot4(sv[j], g);
        acc[GS + j] += dot4(yv[j], g);
        acc[2 * GS + j] += dot4(sv[j], yn);
        acc[3 * GS + j] += dot4(yv[j], yn);
      }
    }
    if (blockIdx.x == 0)
      for (int i = 4 * nq4 + pt; i < n; i += psz) {
        const float g = G[i], yn = Yn[i];
#pragma unroll
        for (int j = 0; j < GS; j++) {
          const float sv = d->Sb[4ll * o_s[j] + i], yv = d->Yb[4ll * o_y[j] + i];
          acc[j] += sv * g;
          acc[GS + j] += yv * g;
          acc[2 * GS + j] += sv * yn;
          acc[3 * GS + j] += yv * yn;
        }
      }
  }
  // pairs k0 .. k0 + GS - 1 of this part into the row (dot * 16 + pair)
  float v[32];
#pragma unroll
  for (int j = 0; j < 8; j++) {
#pragma unroll
    for (int dd = 0; dd < 4; dd++) v[8 * dd + j] = (j < GS && active) ? acc[dd * GS + min(j, GS - 1)] : 0.f;
  }
  wide_clear_row(wide);
  wide_store_row(v, k0, wide);
  __syncthreads();
  for (int k = threadIdx.x; k < MINIM_WIDE; k += blockDim.x) {
    double sum = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) sum += wide[w * MINIM_WIDE + k];
    part[(size_t)blockIdx.x * MINIM_WIDE + k] = sum;
  }
  {
    __shared__ double rowbuf[MINIM_WIDE];
    double* part2 = part + (size_t)gridDim.x * MINIM_WIDE;
    if (last_block_grouped(ctl, part, part2, MINIM_WIDE, wide, rowbuf))
      ctl_a(d, st, ctl, part2, (gridDim.x + kGroup - 1) / kGroup);
  }
}

// P = -gamma g - S w + gamma Y u with g.P and P.P (M compile-time, unused
// pairs read g with weight 0)
template <int M>
__global__ void __launch_bounds__(kThreads, 4)
k_dir_b(const InstDesc* __restrict__ d, MinScalars* st, StepCtl* ctl, double* part, cudaGraphConditionalHandle ls,
        cudaGraphConditionalHandle grad, int spec) {
  if (ctl->retry) return;  // this pass of the loop only continues a line search
  span_begin(ctl);
  const int n = d->ndof, nq4 = n >> 2, mt = ctl->mt;
  const float* G = d->G[st->gi];
  float* P = d->Sb + (long long)st->pbuf * d->hstride;
  const float4* Sb4 = reinterpret_cast<const float4*>(d->Sb);
  const float4* Yb4 = reinterpret_cast<const float4*>(d->Yb);
  const int gS = (int)(reinterpret_cast<const float4*>(G) - Sb4);
  const int gY = (int)(reinterpret_cast<const float4*>(G) - Yb4);
  const float fg = ctl->fg;
  int so[M], yo[M];
  float cS[M], cY[M];
#pragma unroll
  for (int k = 0; k < M; k++) {
    const bool used = k < mt;
    so[k] = used ? ctl->so[k] : gS;
    yo[k] = used ? ctl->yo[k] : gY;
    cS[k] = used ? ctl->coefS[k] : 0.f;
    cY[k] = used ? ctl->coefY[k] : 0.f;
  }
  Acc d1, d2;
  const int t0 = blockIdx.x * blockDim.x + threadIdx.x, nt = gridDim.x * blockDim.x;
  // the sweep runs from the end of the vectors down: pass A swept upwards,
  // so the vectors' last ~100 MB it read are still in L2
  for (int r = t0; r < nq4; r += nt) {
    const int i = nq4 - 1 - r;
    const float4 g = ld4(G, i);
    float4 sv[M], yv[M];
#pragma unroll
    for (int k = 0; k < M; k++) {
      sv[k] = Sb4[so[k] + i];
      yv[k] = Yb4[yo[k] + i];
    }
    float4 q = make_float4(fg * g.x, fg * g.y, fg * g.z, fg * g.w);
#pragma unroll
    for (int k = 0; k < M; k++) {
      q = axpy4(cS[k], sv[k], q);
      q = axpy4(cY[k], yv[k], q);
    }
    st4(P, i, q);
    if (spec != 2) {
      d1.add(dot4(q, g));
      d2.add(dot4(q, q));
    }
  }
  for (int i = 4 * nq4 + t0; i < n; i += nt) {
    const float g = G[i];
    float q = fg * g;
#pragma unroll
    for (int k = 0; k < M; k++) {
      q = fmaf(cS[k], d->Sb[4ll * so[k] + i], q);
      q = fmaf(cY[k], d->Yb[4ll * yo[k] + i], q);
    }
    P[i] = q;
    d1.add(q * g);
    d2.add(q * q);
  }
  // two-trial graph: g.P is summed by the first trial pass, whose
  // controller does the set-up below, so this kernel ends here
  if (spec == 2) return;
  double v[2] = {d1.total(), d2.total()};
  block_row<2>(v, part + (size_t)blockIdx.x * MINIM_WIDE);
  if (last_block(ctl)) ctl_b(d, st, ctl, part, gridDim.x, ls, grad, spec);
}

// Energy at x + t P (line-search trial)
__global__ void __launch_bounds__(kThreads, 3)
k_eonly(const InstDesc* __restrict__ d, MinScalars* st, StepCtl* ctl, double* part, cudaGraphConditionalHandle ls,
        cudaGraphConditionalHandle grad, cudaGraphConditionalHandle outer) {
  span_begin(ctl);
  FlatTeam tm;
  const float* P = d->Sb + (long long)st->pbuf * d->hstride;
  CView<float> cv{d->X32[st->xi], P, (float)ctl->t};
  FusedEmit ne{nullptr, nullptr, nullptr, nullptr, nullptr};
  double e;
  if ((d->pf.n[2] & 3) == 0) e = pf1_eval_quad<float>(tm, d->pf, cv, (float*)nullptr, &ne, true, false);
  else e = pf1_eval<float>(tm, d->pf, cv, (float*)nullptr, &ne, true, false);
  double v[1] = {e};
  block_row<1>(v, part + (size_t)blockIdx.x * MINIM_WIDE);
  if (last_block(ctl)) ctl_ls(d, st, ctl, part, gridDim.x, ls);
}

// Gradient at the accepted point x + t P: writes the point, the gradient and
// y = g_new - g_old; E, g.g, P.y, y.y
template <bool SPEC>
__global__ void __launch_bounds__(kThreads, 3)
k_grad(const InstDesc* __restrict__ d, MinScalars* st, StepCtl* ctl, double* part, cudaGraphConditionalHandle ls,
       cudaGraphConditionalHandle grad, cudaGraphConditionalHandle outer) {
  span_begin(ctl);
  FlatTeam tm;
  const int xi = st->xi, gi = st->gi;
  const float* P = d->Sb + (long long)st->pbuf * d->hstride;
  CView<float> cv{d->X32[xi], P, (float)ctl->t};
  FusedEmit em{d->G[1 - gi], d->G[gi], P, d->Yb + (long long)st->ybuf * d->hstride, nullptr};
  double e;
  if ((d->pf.n[2] & 3) == 0) e = pf1_eval_quad<float>(tm, d->pf, cv, d->X32[1 - xi], &em, true, true);
  else e = pf1_eval<float>(tm, d->pf, cv, d->X32[1 - xi], &em, true, true);
  double v[4] = {e, em.gg.total(), em.py.total(), em.yy.total()};
  block_row<4>(v, part + (size_t)blockIdx.x * MINIM_WIDE);
  if (last_block(ctl)) {
    if (SPEC) ctl_lsg(d, st, ctl, part, gridDim.x, ls, grad, outer);
    else ctl_g(d, st, ctl, part, gridDim.x, outer);
  }
}

// ---- line-shaped stencil (binary PhaseField, nz % 4 == 0) ------------------------
// Threads are laid out as (nz/4 quads along z) x (lines per block), so a
// thread's quad index needs no division and each line's x, y come from one
// division; a quad's four cells are evaluated from 16-byte loads of the quad
// and of its four neighbour lines plus two scalars at the z ends.  The trial
// energy is summed per quad in FP32 and per thread with compensation; the
// gradient variants also write the point, g and y = g - g_old.
// MODE 0: trial energy; 1: gradient at the accepted point; 2: trial energy
// with the gradient at the trial point (kept when the trial is accepted);
// 3: as 2 for two trials in one pass, at t and at t/2 (the next trial of the
// backtracking sequence), the second written to the spare buffers.

// x, P of a quad, its two z-end cells and its four neighbour lines
struct QuadLoads {
  float4 xc, pc, xym, pym, xyp, pyp, xxm, pxm, xxp, pxp;
  float xzm, pzm, xzp, pzp;
};
struct LineCoef {
  float fb, Fi, pr, V;
  bool dx_on, dy_on;
};

// energy of the quad at x + t P (returned) and, with want_g, its gradient;
// c4 receives the quad's point
__device__ __forceinline__ float quad_eval(const QuadLoads& L, float t, const LineCoef& K, bool want_g, float4& c4,
                                           float4& g4) {
  // trial point x + t P with one rounding (fused multiply-add)
  auto tr = [t](float4 a, float4 b) {
    return make_float4(fmaf(t, b.x, a.x), fmaf(t, b.y, a.y), fmaf(t, b.z, a.z), fmaf(t, b.w, a.w));
  };
  c4 = tr(L.xc, L.pc);
  const float cc[4] = {c4.x, c4.y, c4.z, c4.w};
  const float zm = fmaf(t, L.pzm, L.xzm), zp = fmaf(t, L.pzp, L.xzp);
  const float4 ym = tr(L.xym, L.pym), yp = tr(L.xyp, L.pyp), xm = tr(L.xxm, L.pxm), xp = tr(L.xxp, L.pxp);
  const float ymv[4] = {ym.x, ym.y, ym.z, ym.w}, ypv[4] = {yp.x, yp.y, yp.z, yp.w};
  const float xmv[4] = {xm.x, xm.y, xm.z, xm.w}, xpv[4] = {xp.x, xp.y, xp.z, xp.w};
  const float fih = 0.5f * K.Fi, fi2 = 2.f * K.Fi, fb4 = 4.f * K.fb;
  float es = 0.f, g[4];
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const float c = cc[j];
    const float cm = j == 0 ? zm : cc[j - 1], cp = j == 3 ? zp : cc[j + 1];
    // differences to the neighbours: their sum (the Laplacian) and their
    // squares (the gradient energy), per direction
    float gm = c - cm, gp = c - cp;
    float lap = gm + gp, s2 = fmaf(gm, gm, gp * gp);
    if (K.dy_on) {
      gm = c - ymv[j];
      gp = c - ypv[j];
      lap += gm + gp;
      s2 = fmaf(gm, gm, fmaf(gp, gp, s2));
    }
    if (K.dx_on) {
      gm = c - xmv[j];
      gp = c - xpv[j];
      lap += gm + gp;
      s2 = fmaf(gm, gm, fmaf(gp, gp, s2));
    }
    const float a = fmaf(c, c, -1.f);  // (c + 1)(c - 1)
    es = fmaf(K.fb * a, a, fmaf(fih, s2, es));
    if (K.pr != 0.f) es -= K.pr * (0.5f * (c + 1) * K.V);
    g[j] = 0.f;
    if (want_g) {
      g[j] = fmaf(fb4 * c, a, fi2 * lap);
      if (K.pr != 0.f) g[j] -= 0.5f * K.pr * K.V;
    }
  }
  g4 = make_float4(g[0], g[1], g[2], g[3]);
  return es;
}

// Pointers and trial multiplier of one line-stencil pass.  The first trial
// (at t) writes its point, gradient and y = g - g_old to Xa, Ga, Ya; with
// `two` the second (at t/2) writes to Xb, Gb, Yb.
struct LinesIO {
  const float* X;
  const float* P;
  const float* Go;
  float* Xa;
  float* Ga;
  float* Ya;
  float* Xb;
  float* Gb;
  float* Yb;
  float t;
  bool two;
};
// per-thread compensated sums of one pass: energy, g.g, P.y, y.y of each
// trial and g_old.P
struct LinesAcc {
  Acc e, gg, py, yy, e2, gg2, py2, yy2, gpa;
};

constexpr int lines_min_blocks(int mode) { return mode == 3 ? 2 : (mode ? 3 : 4); }

// One quad of a line-stencil pass from its loads: the trial point(s), energy
// and gradient, the writes of the point, g and y, and the pass's sums.
template <int MODE>
__device__ __forceinline__ void lines_quad(const LinesIO& io, const LineCoef& K, const QuadLoads& L, int q, float t,
                                           bool two, LinesAcc& a) {
  constexpr bool WANT_G = MODE != 0;
  constexpr bool DUAL = MODE == 3;
  float4 go = make_float4(0.f, 0.f, 0.f, 0.f);
  if (WANT_G) go = ld4(io.Go, q);
  float4 c4, gv;
  if (DUAL) a.gpa.add(dot4(go, L.pc));  // g.P for the first pass of a direction
  a.e.add(quad_eval(L, t, K, WANT_G, c4, gv));
  if (WANT_G) {
    st4(io.Xa, q, c4);
    st4(io.Ga, q, gv);
    a.gg.add(dot4(gv, gv));
    const float4 yv = make_float4(gv.x - go.x, gv.y - go.y, gv.z - go.z, gv.w - go.w);
    st4(io.Ya, q, yv);
    a.py.add(dot4(L.pc, yv));
    a.yy.add(dot4(yv, yv));
  }
  if (DUAL && two) {
    a.e2.add(quad_eval(L, 0.5f * t, K, true, c4, gv));
    st4(io.Xb, q, c4);
    st4(io.Gb, q, gv);
    a.gg2.add(dot4(gv, gv));
    const float4 yv = make_float4(gv.x - go.x, gv.y - go.y, gv.z - go.z, gv.w - go.w);
    st4(io.Yb, q, yv);
    a.py2.add(dot4(L.pc, yv));
    a.yy2.add(dot4(yv, yv));
  }
}

// The stencil's constants of a binary PhaseField
__device__ __forceinline__ LineCoef line_coef(const PotPF& Pf) {
  LineCoef K;
  K.V = (float)Pf.vol_of_type[1];
  K.fb = (float)Pf.kappa[0] / 16 * K.V;
  K.Fi = 0.25f / (float)Pf.res2 * (float)Pf.kappaP[0] * K.V;
  K.pr = (Pf.flags & PF_PRESSURE) ? (float)Pf.pressure[0] : 0.f;
  K.dx_on = Pf.n[0] > 1;
  K.dy_on = Pf.n[1] > 1;
  return K;
}

// The sweep of a line-stencil pass over every line of the grid (blocks of
// (nz/4) x lines threads, lines dealt round-robin to the blocks).
template <int MODE>
__device__ __forceinline__ void lines_sweep(const PotPF& Pf, const LinesIO& io, LinesAcc& a) {
  constexpr bool DUAL = MODE == 3;
  const int nx = Pf.n[0], ny = Pf.n[1], nz = Pf.n[2], nz4 = nz >> 2;
  const float* X = io.X;
  const float* Pd = io.P;
  const float t = io.t;
  const LineCoef K = line_coef(Pf);
  const int zq = threadIdx.x, nl = nx * ny;
  const int z0 = 4 * zq;
  const int izm = z0 == 0 ? nz - 1 : z0 - 1, izp = z0 + 4 == nz ? 0 : z0 + 4;
  const bool two = DUAL && io.two;
  if (zq < nz4) {
    for (int l = blockIdx.x * blockDim.y + threadIdx.y; l < nl; l += gridDim.x * blockDim.y) {

      const int x = l / ny, y = l - x * ny;
      const int lym = x * ny + (y == 0 ? ny - 1 : y - 1), lyp = x * ny + (y == ny - 1 ? 0 : y + 1);
      const int lxm = (x == 0 ? nx - 1 : x - 1) * ny + y, lxp = (x == nx - 1 ? 0 : x + 1) * ny + y;
      const int q = l * nz4 + zq;
      // every load of the quad first
      QuadLoads L;
      L.xc = ld4(X, q);
      L.pc = ld4(Pd, q);
      L.xzm = X[l * nz + izm];
      L.pzm = Pd[l * nz + izm];
      L.xzp = X[l * nz + izp];
      L.pzp = Pd[l * nz + izp];
      L.xym = ld4(X, lym * nz4 + zq);
      L.pym = ld4(Pd, lym * nz4 + zq);
      L.xyp = ld4(X, lyp * nz4 + zq);
      L.pyp = ld4(Pd, lyp * nz4 + zq);
      L.xxm = ld4(X, lxm * nz4 + zq);
      L.pxm = ld4(Pd, lxm * nz4 + zq);
      L.xxp = ld4(X, lxp * nz4 + zq);
      L.pxp = ld4(Pd, lxp * nz4 + zq);
      lines_quad<MODE>(io, K, L, q, t, two, a);
    }
  }
}

// ---- line stencil through TMA plane tiles (two trials per pass) -----------------
// The same pass as lines_sweep<3>, with the field and the direction brought
// into shared memory by the tensor memory accelerator.  A block owns a strip
// of kTmaY lines (y0 .. y0 + kTmaY - 1) over a run of planes x = xa .. xb - 1
// and walks it along x.  One plane tile is, per array (x and P), the strip's
// lines with their y neighbours -- one 3-D box of {nz, kTmaY + 2, 1} --
// and a ring of NS tiles (kTmaStages = 4 by default; 6 or 8 through
// MINIM_GPU_LINES_TMA) holds planes x - 1, x and x + 1 while the next
// planes land: every value is brought on chip once per block, the x
// neighbours come from the ring and the y neighbours from the tile.
//
// A tile holds kTmaY + 2 lines per array: line y0 - 1 + j in slot j.
// Inside the grid one box brings all of them; a strip at the periodic
// boundary in y (y0 = 0 or y0 + kTmaY = ny) brings them as kTmaY + 2
// one-line boxes with the line index wrapped.  Plane wrap in x is the box's
// own coordinate.  Every box starts at z = 0.
//
// Thread 0 issues the copies; each tile has an mbarrier that completes when
// its bytes have landed.  Waits are bounded: a wait that gives up sets *err
// (the pass's results are then unusable), the block issues no further copy,
// and before it exits it waits (bounded again) for every copy it issued.
constexpr int kTmaY = 4;
constexpr int kTmaSlots = kTmaY + 2;
constexpr int kTmaStages = 4;
// whether the stepped graph's trial pass uses the tiles unless
// MINIM_GPU_LINES_TMA says otherwise
constexpr int kTmaLinesDefault = 0;
// tensor maps of one instance's buffers: for each of the three coordinate
// buffers and the MINIM_MAXM + 1 direction slots, the strip box and the
// one-line box
constexpr int kTmaBufs = 3 + MINIM_MAXM + 1;
struct alignas(128) TmaMaps {
  CUtensorMap box[kTmaBufs];
  CUtensorMap line[kTmaBufs];
  const float* xbase[3];
};

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int c0, int c1, int c2,
                                            unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
          "r"(smem_u32(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_map_acquire(const CUtensorMap* map) {
  asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(map) : "memory");
}

// bytes of dynamic shared memory of the TMA line stencil with ns stages for
// lines of nz (the stages plus room to align the first to 128 bytes)
__host__ __device__ constexpr size_t tma_lines_smem(int nz, int ns = kTmaStages) {
  return (size_t)ns * 2 * kTmaSlots * nz * sizeof(float) + 128;
}
// whether a grid takes the TMA line stencil: whole warps of quads, tile
// slots on 128-byte boundaries, at least two strips
__host__ __device__ constexpr bool tma_lines_fits(int nx, int ny, int nz) {
  return nz % 32 == 0 && nz <= 256 && ny % kTmaY == 0 && ny >= 2 * kTmaY && nx >= 3;
}
// the strip and plane run of block b of a grid of (ny / kTmaY) * nch blocks
struct TmaRun {
  int y0, xa, xb;
};
__host__ __device__ inline TmaRun tma_run(int b, int nch, int nx) {
  const int strip = b / nch, c = b - strip * nch;
  return {strip * kTmaY, (int)((long long)c * nx / nch), (int)((long long)(c + 1) * nx / nch)};
}

// Launch shape of the TMA line stencil: blocks of (nz / 4) x kTmaY threads,
// (ny / kTmaY) strips times nch plane runs, about `target` blocks.
inline int tma_shape(const int* grid, int target, int* nch) {
  const int nstrip = grid[1] / kTmaY;
  *nch = std::max(1, std::min(grid[0], target / nstrip));
  return nstrip * *nch;
}

template <int NS>
__device__ __forceinline__ void lines_sweep_tma(const PotPF& Pf, const LinesIO& io, LinesAcc& a,
                                                const CUtensorMap* mbx, const CUtensorMap* mlx,
                                                const CUtensorMap* mbp, const CUtensorMap* mlp, int nch, int* err) {
  extern __shared__ unsigned char tma_raw[];
  __shared__ __align__(8) unsigned long long full[NS];
  float* sm = reinterpret_cast<float*>(tma_raw + ((128u - (smem_u32(tma_raw) & 127u)) & 127u));
  const int nx = Pf.n[0], ny = Pf.n[1], nz = Pf.n[2], nz4 = nz >> 2;
  const TmaRun run = tma_run(blockIdx.x, nch, nx);
  const int y0 = run.y0;
  const bool wrap = y0 == 0 || y0 + kTmaY == ny;
  const int sfl = kTmaSlots * nz;  // floats of one array's tile
  const unsigned bytes = 2u * (unsigned)sfl * (unsigned)sizeof(float);
  const int nplanes = run.xb - run.xa + 2;  // planes xa - 1 .. xb
  const bool lead = threadIdx.x == 0 && threadIdx.y == 0;
  auto issue = [&](int k) {
    const int s = k % NS;
    int px = run.xa - 1 + k;
    px = px < 0 ? px + nx : (px >= nx ? px - nx : px);
    float* dx = sm + (size_t)s * 2 * sfl;
    float* dp = dx + sfl;
    mbar_expect_tx(&full[s], bytes);
    if (!wrap) {
      tma_load_3d(dx, mbx, 0, y0 - 1, px, &full[s]);
      tma_load_3d(dp, mbp, 0, y0 - 1, px, &full[s]);
    } else {
      for (int j = 0; j < kTmaSlots; j++) {
        int yl = y0 - 1 + j;
        yl = yl < 0 ? yl + ny : (yl >= ny ? yl - ny : yl);
        tma_load_3d(dx + j * nz, mlx, 0, yl, px, &full[s]);
        tma_load_3d(dp + j * nz, mlp, 0, yl, px, &full[s]);
      }
    }
  };
  if (lead) {
    for (int s = 0; s < NS; s++) mbar_init(&full[s], 1);
    mbar_init_fence();
    tma_map_acquire(wrap ? mlx : mbx);
    tma_map_acquire(wrap ? mlp : mbp);
  }
  __syncthreads();
  // issued / waited: planes issued and planes whose wait has run (the same
  // in every thread)
  int issued = nplanes < NS ? nplanes : NS, waited = 0;
  if (lead)
    for (int k = 0; k < issued; k++) issue(k);
  const LineCoef K = line_coef(Pf);
  const float t = io.t;
  const int zq = threadIdx.x, ly = threadIdx.y;
  const int z0 = 4 * zq;
  const int izm = z0 == 0 ? nz - 1 : z0 - 1, izp = z0 + 4 == nz ? 0 : z0 + 4;
  const int y = y0 + ly;
  bool failed = false;
  unsigned long long limit = 1000000000ull;
  for (int x = run.xa; x < run.xb; x++) {
    // planes x - 1, x, x + 1 are planes i, i + 1, i + 2 of the run
    const int i = x - run.xa;
    bool bad = false;
    while (waited <= i + 2) {
      const int s = waited % NS;
      if (!failed && !mbar_wait(&full[s], (unsigned)(waited / NS) & 1u, limit)) bad = true;
      waited++;
    }
    if (__syncthreads_or(bad)) {
      if (!failed && lead) atomicExch(err, 1);
      failed = true;
      limit = 1000000ull;
    }
    if (failed) break;
    if (zq < nz4) {
      const float* bm = sm + (size_t)(i % NS) * 2 * sfl;
      const float* bc = sm + (size_t)((i + 1) % NS) * 2 * sfl;
      const float* bq = sm + (size_t)((i + 2) % NS) * 2 * sfl;
      auto q4 = [&](const float* b, int slot) { return reinterpret_cast<const float4*>(b + slot * nz)[zq]; };
      const int sc = ly + 1;
      const float* xc = bc + sc * nz;
      const float* pc = bc + sfl + sc * nz;
      QuadLoads L;
      L.xc = q4(bc, sc);
      L.pc = q4(bc + sfl, sc);
      L.xzm = xc[izm];
      L.pzm = pc[izm];
      L.xzp = xc[izp];
      L.pzp = pc[izp];
      L.xym = q4(bc, sc - 1);
      L.pym = q4(bc + sfl, sc - 1);
      L.xyp = q4(bc, sc + 1);
      L.pyp = q4(bc + sfl, sc + 1);
      L.xxm = q4(bm, sc);
      L.pxm = q4(bm + sfl, sc);
      L.xxp = q4(bq, sc);
      L.pxp = q4(bq + sfl, sc);
      lines_quad<3>(io, K, L, (x * ny + y) * nz4 + zq, t, io.two, a);
    }
    // plane i is done in every thread: its stage takes plane i + NS
    __syncthreads();
    if (issued < nplanes && issued == i + NS) {
      if (lead) issue(issued);
      issued++;
    }
  }
  // After a failed wait, copies issued earlier may still be in flight.  A
  // stage has at most one fill outstanding, so they are among the last
  // NS planes issued: wait for each (bounded) before leaving.
  if (failed) {
    for (int k = issued > NS ? issued - NS : 0; k < issued; k++)
      mbar_wait(&full[k % NS], (unsigned)(k / NS) & 1u, 1000000ull);
    __syncthreads();
  }
}

// the block's row of partial sums of a line-stencil pass
template <int MODE>
__device__ __forceinline__ void lines_row(const LinesAcc& a, double* row) {
  if (MODE == 3) {
    double v[9] = {a.e.total(),   a.gg.total(),  a.py.total(),  a.yy.total(), a.e2.total(),
                   a.gg2.total(), a.py2.total(), a.yy2.total(), a.gpa.total()};
    block_row<9>(v, row);
  } else if (MODE != 0) {
    double v[4] = {a.e.total(), a.gg.total(), a.py.total(), a.yy.total()};
    block_row<4>(v, row);
  } else {
    double v[1] = {a.e.total()};
    block_row<1>(v, row);
  }
}

template <int MODE, int MINB = lines_min_blocks(MODE), int MAXT = kThreads>
__global__ void __launch_bounds__(MAXT, MINB)
k_lines(const InstDesc* __restrict__ d, MinScalars* st, StepCtl* ctl, double* part, cudaGraphConditionalHandle ls,
        cudaGraphConditionalHandle grad, cudaGraphConditionalHandle outer) {
  constexpr bool DUAL = MODE == 3;
  span_begin(ctl);
  const int xi = st->xi, gi = st->gi;
  LinesIO io;
  io.X = d->X32[xi];
  io.P = d->Sb + (long long)st->pbuf * d->hstride;
  io.Go = d->G[gi];
  io.t = (float)ctl->t;
  io.Xa = d->X32[1 - xi];
  io.Ga = d->G[1 - gi];
  io.Ya = d->Yb + (long long)st->ybuf * d->hstride;
  // two-trial pass, or (gmode) the gradient at t alone
  io.two = DUAL && ctl->gmode == 0;
  io.Xb = DUAL ? d->X32s : nullptr;
  io.Gb = DUAL ? d->Gs : nullptr;
  io.Yb = DUAL ? d->Yb + (long long)st->ybuf2 * d->hstride : nullptr;
  LinesAcc a;
  lines_sweep<MODE>(d->pf, io, a);
  lines_row<MODE>(a, part + (size_t)blockIdx.x * MINIM_WIDE);
  if (last_block(ctl)) {
    if (MODE == 0) ctl_ls(d, st, ctl, part, gridDim.x, ls);
    else if (MODE == 1) ctl_g(d, st, ctl, part, gridDim.x, outer);
    else if (MODE == 2) ctl_lsg(d, st, ctl, part, gridDim.x, ls, grad, outer);
    else ctl_lsg2(d, st, ctl, part, gridDim.x, outer);
  }
}

// One line-stencil pass outside the graph, with no controller: the same
// sweep as k_lines<MODE> on the given buffers, each block's partial row to
// part.  For checking the stencil against an FP64 evaluation.
template <int MODE>
__global__ void __launch_bounds__(kThreads, lines_min_blocks(MODE))
k_lines_probe(const InstDesc* __restrict__ d, LinesIO io, double* part) {
  LinesAcc a;
  lines_sweep<MODE>(d->pf, io, a);
  lines_row<MODE>(a, part + (size_t)blockIdx.x * MINIM_WIDE);
}

// The graph's two-trial pass with its lines staged through tensor-map tiles
// (k_lines<3> with lines_sweep_tma).  maps holds the tensor maps of the
// instance's buffers: the point's map is found by the buffer's address (the
// controllers exchange the three coordinate buffers), the direction's by
// its ring slot.  A copy wait that gave up, or a buffer with no map, sets
// ctl->tma_err; later passes of the launch then skip their sweeps and the
// controller ends the graph's loop instead of taking a step.
template <int MAXT, int MINB, int NS>
__global__ void __launch_bounds__(MAXT, MINB)
k_lines_tma(const InstDesc* __restrict__ d, MinScalars* st, StepCtl* ctl, double* part,
            cudaGraphConditionalHandle ls, cudaGraphConditionalHandle grad, cudaGraphConditionalHandle outer,
            const TmaMaps* __restrict__ maps, int nch) {
  span_begin(ctl);
  const int xi = st->xi, gi = st->gi;
  LinesIO io;
  io.X = d->X32[xi];
  io.P = d->Sb + (long long)st->pbuf * d->hstride;
  io.Go = d->G[gi];
  io.t = (float)ctl->t;
  io.Xa = d->X32[1 - xi];
  io.Ga = d->G[1 - gi];
  io.Ya = d->Yb + (long long)st->ybuf * d->hstride;
  io.two = ctl->gmode == 0;
  io.Xb = d->X32s;
  io.Gb = d->Gs;
  io.Yb = d->Yb + (long long)st->ybuf2 * d->hstride;
  int ix = -1;
  for (int i = 0; i < 3; i++)
    if (maps->xbase[i] == io.X) ix = i;
  const int ip = 3 + st->pbuf;
  const bool lead = threadIdx.x == 0 && threadIdx.y == 0;
  const bool nomap = ix < 0 || ip >= kTmaBufs;
  if (nomap && lead) atomicExch(&ctl->tma_err, 2);
  const bool skip = __syncthreads_or(nomap || (lead && *(volatile int*)&ctl->tma_err != 0));
  LinesAcc a;
  if (!skip)
    lines_sweep_tma<NS>(d->pf, io, a, &maps->box[ix], &maps->line[ix], &maps->box[ip], &maps->line[ip], nch,
                        &ctl->tma_err);
  lines_row<3>(a, part + (size_t)blockIdx.x * MINIM_WIDE);
  if (last_block(ctl)) {
    if (*(volatile int*)&ctl->tma_err) {
      if (lead) cudaGraphSetConditional(outer, 0u);
    } else {
      ctl_lsg2(d, st, ctl, part, gridDim.x, outer);
    }
  }
}

// One TMA line-stencil pass outside the graph (two trials, no controller):
// the sweep of lines_sweep_tma on the buffers of io, whose tensor maps are
// maps->box[0] / line[0] (x) and box[1] / line[1] (P).
__global__ void __launch_bounds__(kThreads, 3)
k_lines_tma_probe(const InstDesc* __restrict__ d, LinesIO io, const TmaMaps* __restrict__ maps, int nch,
                  double* part, int* err) {
  LinesAcc a;
  lines_sweep_tma<kTmaStages>(d->pf, io, a, &maps->box[0], &maps->line[0], &maps->box[1], &maps->line[1], nch, err);
  lines_row<3>(a, part + (size_t)blockIdx.x * MINIM_WIDE);
}

// ---- controllers (one block) ----------------------------------------------------

__global__ void k_begin(const InstDesc* __restrict__ d, const MinScalars* __restrict__ st, StepCtl* ctl,
                        int slice, int timing, cudaGraphConditionalHandle outer) {
  if (threadIdx.x == 0) {
    ctl->timing = timing;
    ctl->retry = 0;
    ctl->tma_err = 0;
    ctl->iters = 0;
    ctl->slice = slice;
    ctl->kernels = 1;
    ctl->tmark = globaltimer_ns();
    const bool go = st->status == ST_RUNNING && st->initialised && st->stage == 0 && st->resume == 0 &&
                    st->iter > 0 && st->iter <= d->mp.max_iter;
    cudaGraphSetConditional(outer, go ? 1u : 0u);
  }
}

// Device time since the previous controller finished (the phase kernel just
// run, with its launch) goes to phase ph of the state's phase timers
// (0 gradient, 1 line-search trials, 2 direction); phase_mark ends it.
__device__ __forceinline__ void phase_time(MinScalars* st, StepCtl* ctl, int ph) {
  st->tphase[ph] += (double)(globaltimer_ns() - ctl->tmark);
}
__device__ __forceinline__ void phase_mark(StepCtl* ctl) {
  const unsigned long long now = globaltimer_ns();
  if (ctl->timing) ctl->work[ctl->cur] += (double)(now - ctl->tw);
  ctl->tmark = now;
}

// dirA sums, the compact-form algebra of getDirection, pass-B coefficients
__device__ void ctl_a(const InstDesc* __restrict__ d, MinScalars* st_g, StepCtl* ctl_g, const double* part, int nb) {
  __shared__ double wide[8 * MINIM_WIDE];
  __shared__ double wout[MINIM_WIDE];
  __shared__ Mirror mir;
  const MirrorRegs mr = mirror_load(st_g, ctl_g);
  sum_rows_fixed(part, nb, MINIM_WIDE, wout, wide);
  mirror_store(&mir, mr, st_g, ctl_g);
  __syncthreads();
  MinScalars* st = &mir.st;
  StepCtl* ctl = &mir.ctl;
  // warp 0: the algebra (lbfgs_compact_warp), lane k on pair k
  const int lane = threadIdx.y * blockDim.x + threadIdx.x;
  if (lane < 32) [&] {
  if (lane == 0) {
    phase_time(st, ctl, 2);
    span_end(ctl, 2);
  }
  const int m = d->mp.m, n = d->ndof;
  const long long hs = d->hstride;
  const int ii = st->ii + 1, mt = ii < m ? ii : m, c = ii % m;
  const int pend = st->pend;
  double(*SY)[MINIM_MAXM] = st->SY;
  double(*YY)[MINIM_MAXM] = st->YY;
  const bool on = lane < mt;
  const int slk = on ? ring_slot(c, mt, lane, m) : 0;
  // the mt x mt blocks of S^T Y and Y^T Y in age order, staged in shared
  // memory from the state record; the newest pair's column (pend, the last
  // in age order) is then set from this pass's sums and written back, so
  // nothing is read back from global memory after being written.  Every
  // lane issues all its loads (up to 8 entries of each, its pair's scalars)
  // before using any: one memory round trip instead of one per entry.
  double* Rs = wide;
  double* Ys = wide + MINIM_MAXM * MINIM_MAXM;
  double rv[8], yv[8];
  const int ne = mt * mt;
#pragma unroll
  for (int j = 0; j < 8; j++) {
    const int e = lane + 32 * j;
    rv[j] = 0.0;
    yv[j] = 0.0;
    if (e < ne) {
      const int a = e / mt, b = e - a * mt;
      const int sa = ring_slot(c, mt, a, m), sb = ring_slot(c, mt, b, m);
      rv[j] = SY[sa][sb];
      yv[j] = YY[sa][sb];
    }
  }
  const double sig = on ? st->sigma[slk] : 0.0;
  const int sid = on ? st->sidx[slk] : 0, yid = on ? st->yidx[slk] : 0;
#pragma unroll
  for (int j = 0; j < 8; j++) {
    const int e = lane + 32 * j;
    if (e < ne) {
      const int a = e / mt, b = e - a * mt;
      Rs[a * MINIM_MAXM + b] = rv[j];
      Ys[a * MINIM_MAXM + b] = yv[j];
    }
  }
  __syncwarp();
  double sg = 0.0, yg = 0.0;
  if (on) {
    sg = sig * wout[lane];
    yg = wout[MINIM_MAXM + lane];
    if (pend >= 0) {  // pend == kn: age index mt - 1
      const double syn = sig * wout[2 * MINIM_MAXM + lane], yyn = wout[3 * MINIM_MAXM + lane];
      Rs[lane * MINIM_MAXM + mt - 1] = syn;
      Ys[lane * MINIM_MAXM + mt - 1] = yyn;
      Ys[(mt - 1) * MINIM_MAXM + lane] = yyn;
      SY[slk][pend] = syn;
      YY[slk][pend] = yyn;
      YY[pend][slk] = yyn;
    }
  }
  __syncwarp();
  const double gamma = Rs[(mt - 1) * (MINIM_MAXM + 1)] / Ys[(mt - 1) * (MINIM_MAXM + 1)];
  double u, w;
  lbfgs_compact_warp(
      mt, gamma, sg, yg, [=](int a, int b) { return Rs[a * MINIM_MAXM + b]; },
      [=](int a, int b) { return Ys[a * MINIM_MAXM + b]; }, u, w);
  if (lane < MINIM_MAXM) {
    ctl->coefS[lane] = on ? (float)(-w * sig) : 0.f;
    ctl->coefY[lane] = on ? (float)(gamma * u) : 0.f;
    ctl->so[lane] = on ? (int)(((long long)sid * hs) >> 2) : 0;
    ctl->yo[lane] = on ? (int)(((long long)yid * hs) >> 2) : 0;
  }
  __syncwarp();
  if (lane == 0) {
    // the two-trial graph's first pass tries the unit step along P at once
    // and checks that P is a descent direction afterwards (fresh); the other
    // graph's pass-B controller overwrites these
    ctl->t = 1.0;
    ctl->gmode = d->mp.linesearch == 0 ? 0 : 1;
    ctl->fresh = 1;
    ctl->fg = (float)(-gamma);
    ctl->mt = mt;
    st->ii = ii;
    st->pend = -1;
    st->abytes += (4.0 * mt + 2.0) * 4.0 * n;
    phase_mark(ctl);
  }
  }();
  __syncthreads();
  mirror_out(&mir, st_g, ctl_g);
}

// dirB sums: step cap, descent check, line-search set-up
__device__ void ctl_b(const InstDesc* __restrict__ d, MinScalars* st_g, StepCtl* ctl_g, const double* part, int nb,
                      cudaGraphConditionalHandle ls, cudaGraphConditionalHandle grad, int spec) {
  __shared__ double wide[8 * MINIM_WIDE];
  __shared__ double v[2];
  __shared__ Mirror mir;
  const MirrorRegs mr = mirror_load(st_g, ctl_g);
  sum_rows_fixed(part, nb, 2, v, wide);
  mirror_store(&mir, mr, st_g, ctl_g);
  __syncthreads();
  MinScalars* st = &mir.st;
  StepCtl* ctl = &mir.ctl;
  if (threadIdx.x == 0 && threadIdx.y == 0) [&] {
  phase_time(st, ctl, 2);
  span_end(ctl, 3);
  double gp = v[0], scale = 1.0;
  if (d->mp.max_step != 0) {
    const double ss = sqrt(v[1]);
    if (ss > d->mp.max_step) scale = d->mp.max_step / ss;
  }
  gp *= scale;
  double gs = gp;
  if (gs > 0) {
    gs = -gs;
    scale = -scale;
  }
  ctl->t = scale;
  if (spec == 2) {
    // two-trial graph: the first trial pass follows unconditionally; without
    // a line search it is the gradient at the full step
    ctl->gmode = d->mp.linesearch == 0 ? 0 : 1;
    if (d->mp.linesearch == 0) {
      ctl->thr = -0.5 * gs;
      ctl->e0 = st->E;
      ctl->k = 0;
      ctl->exhausted = 1;
    } else {
      ctl->exhausted = 0;
    }
  } else if (d->mp.linesearch == 0) {
    ctl->thr = -0.5 * gs;
    ctl->e0 = st->E;
    ctl->k = 0;
    ctl->exhausted = 1;
    cudaGraphSetConditional(ls, 1u);
    if (spec) cudaGraphSetConditional(grad, 0u);
  } else {
    ctl->exhausted = 0;
    cudaGraphSetConditional(ls, 0u);
    if (spec) cudaGraphSetConditional(grad, 1u);
  }
  phase_mark(ctl);
  }();
  __syncthreads();
  mirror_out(&mir, st_g, ctl_g);
}

// one line-search trial: Armijo test, or halve the step (10 trials at most;
// after the last failure the halved step is taken unevaluated)
__device__ void ctl_ls(const InstDesc* __restrict__ d, MinScalars* st_g, StepCtl* ctl_g, const double* part, int nb,
         cudaGraphConditionalHandle ls) {
  __shared__ double wide[8 * MINIM_WIDE];
  __shared__ double v[1];
  __shared__ Mirror mir;
  const MirrorRegs mr = mirror_load(st_g, ctl_g);
  sum_rows_fixed(part, nb, 1, v, wide);
  mirror_store(&mir, mr, st_g, ctl_g);
  __syncthreads();
  MinScalars* st = &mir.st;
  StepCtl* ctl = &mir.ctl;
  if (threadIdx.x == 0 && threadIdx.y == 0) [&] {
  phase_time(st, ctl, 1);
  span_end(ctl, 0);
  st->evals++;
  st->abytes += 8.0 * d->ndof;
  ctl->kernels += 1;
  bool more = false;
  if (ctl->e0 - v[0] >= ctl->thr) {
    ctl->exhausted = ctl->k >= 8;
  } else {
    ctl->t *= 0.5;
    ctl->thr *= 0.5;
    ctl->k++;
    more = ctl->k < 10;
  }
  cudaGraphSetConditional(ls, more ? 1u : 0u);
  phase_mark(ctl);
  }();
  __syncthreads();
  mirror_out(&mir, st_g, ctl_g);
}

// The pair update of Lbfgs::iteration with the sums {E, g.g, P.y, y.y} of
// the gradient at the accepted point, then the end-of-iteration decision
// (continue here, or hand over to the persistent kernel).  Thread 0.
__device__ void commit_grad(const InstDesc* __restrict__ d, MinScalars* st, StepCtl* ctl, const double* v,
                            cudaGraphConditionalHandle outer) {
  const MinParams& mp = d->mp;
  const int n = d->ndof;
  st->E = v[0];
  st->gg = v[1];
  st->gi ^= 1;
  st->xi ^= 1;
  const double t = ctl->t, py = v[2], yyv = v[3];
  const double sy = t * py;
  if (sy != 0 && isfinite(sy)) {
    const int m = mp.m, c = st->ii % m;
    const int os = st->sidx[c], oy = st->yidx[c];
    st->sidx[c] = st->pbuf;
    st->yidx[c] = st->ybuf;
    st->rho[c] = 1.0 / sy;
    st->sigma[c] = t;
    st->yy[c] = yyv;
    st->pbuf = os;
    st->ybuf = oy;
    st->pend = c;
  } else {
    st->ii--;
  }
  // the persistent kernel's end-of-iteration rules, on copies
  const bool exh = ctl->exhausted != 0;
  const bool finite = isfinite(st->E) && isfinite(st->gg);
  const double r = sqrt(st->gg / n);
  const bool conv = r < mp.tol;
  const bool mixed = mp.precision == 0;
  int cool = st->cool, stall = st->stall, exr = st->exhausted_run, why = 0;
  double best = st->best_rms;
  if (mixed) {
    if (cool > 0) cool--;
    if (r < 0.999 * best) {
      best = r;
      stall = 0;
    } else {
      stall++;
    }
    exr = exr * 7 / 8 + (exh ? 8 : 0);
    why = conv ? 1
               : ((exr >= 20 || (exh && r < 1000.0 * mp.tol))
                      ? 2
                      : ((stall >= 100 && r < 100.0 * mp.tol && cool == 0) ? 3 : 0));
  }
  bool stop;
  if (finite && !conv && why == 0) {
    if (mixed) {
      st->cool = cool;
      st->stall = stall;
      st->exhausted_run = exr;
      st->best_rms = best;
    }
    st->iter++;
    ctl->iters++;
    stop = st->iter > mp.max_iter || ctl->iters >= ctl->slice;
  } else {
    st->resume = 1;
    st->resume_exhausted = exh ? 1 : 0;
    stop = true;
  }
  cudaGraphSetConditional(outer, stop ? 0u : 1u);
  phase_mark(ctl);
}


// gradient sums: the pair update of Lbfgs::iteration, then the end-of-
// iteration decision (continue here, or hand over to the persistent kernel)
__device__ void ctl_g(const InstDesc* __restrict__ d, MinScalars* st_g, StepCtl* ctl_g, const double* part, int nb,
        cudaGraphConditionalHandle outer) {
  __shared__ double wide[8 * MINIM_WIDE];
  __shared__ double v[4];
  __shared__ Mirror mir;
  const MirrorRegs mr = mirror_load(st_g, ctl_g);
  sum_rows_fixed(part, nb, 4, v, wide);
  mirror_store(&mir, mr, st_g, ctl_g);
  __syncthreads();
  MinScalars* st = &mir.st;
  StepCtl* ctl = &mir.ctl;
  if (threadIdx.x == 0 && threadIdx.y == 0) [&] {
  phase_time(st, ctl, 0);
  span_end(ctl, 1);
  st->evals++;
  st->abytes += 24.0 * d->ndof;
  ctl->kernels += 3;
  commit_grad(d, st, ctl, v, outer);
  }();
  __syncthreads();
  mirror_out(&mir, st_g, ctl_g);
}

// A line-search trial that also evaluated the gradient at its point (x, g
// and y written to the next buffers): Armijo test; when it passes, that
// gradient is the accepted point's and the iteration completes here; when
// it fails the step is halved (10 trials at most, after which the halved
// step is taken unevaluated and the gradient kernel runs).
__device__ void ctl_lsg(const InstDesc* __restrict__ d, MinScalars* st_g, StepCtl* ctl_g, const double* part,
                        int nb, cudaGraphConditionalHandle ls, cudaGraphConditionalHandle grad,
                        cudaGraphConditionalHandle outer) {
  __shared__ double wide[8 * MINIM_WIDE];
  __shared__ double v[4];
  __shared__ Mirror mir;
  const MirrorRegs mr = mirror_load(st_g, ctl_g);
  sum_rows_fixed(part, nb, 4, v, wide);
  mirror_store(&mir, mr, st_g, ctl_g);
  __syncthreads();
  MinScalars* st = &mir.st;
  StepCtl* ctl = &mir.ctl;
  if (threadIdx.x == 0 && threadIdx.y == 0) [&] {
  phase_time(st, ctl, 1);
  span_end(ctl, 0);
  st->evals++;
  ctl->kernels += 1;
  if (ctl->e0 - v[0] >= ctl->thr) {
    ctl->exhausted = ctl->k >= 8;
    ctl->acc_hist[ctl->k]++;
    cudaGraphSetConditional(ls, 0u);
    cudaGraphSetConditional(grad, 0u);
    st->evals++;
    st->abytes += 24.0 * d->ndof;
    ctl->kernels += 2;
    commit_grad(d, st, ctl, v, outer);
  } else {
    st->abytes += 8.0 * d->ndof;
    ctl->t *= 0.5;
    ctl->thr *= 0.5;
    ctl->k++;
    const bool more = ctl->k < 10;
    if (!more) ctl->acc_hist[10]++;
    cudaGraphSetConditional(ls, more ? 1u : 0u);
    cudaGraphSetConditional(grad, more ? 0u : 1u);
    phase_mark(ctl);
  }
  }();
  __syncthreads();
  mirror_out(&mir, st_g, ctl_g);
}

// Two consecutive trials of the backtracking sequence from one pass (t and
// t / 2, each with its gradient): the Armijo test of the first, then, if it
// failed, of the second, as the sequential line search takes them.  When the
// second is accepted its point, gradient and y (written to the spare
// buffers) become the next ones by exchanging buffer pointers and slots.
// After the tenth failed trial (or without a line search) the next pass is
// the gradient at the step alone (gmode), which completes the iteration.
// A pass that completes no iteration sets `retry`: the outer loop runs once
// more with the direction kernels returning at once, so the common pass
// (one of the two trials accepted) costs one conditional node, not two.
__device__ void ctl_lsg2(const InstDesc* __restrict__ d, MinScalars* st_g, StepCtl* ctl_g, const double* part,
                         int nb, cudaGraphConditionalHandle outer) {
  __shared__ double wide[8 * MINIM_WIDE];
  __shared__ double v[9];
  __shared__ Mirror mir;
  const MirrorRegs mr = mirror_load(st_g, ctl_g);
  sum_rows_fixed(part, nb, 9, v, wide);
  mirror_store(&mir, mr, st_g, ctl_g);
  __syncthreads();
  MinScalars* st = &mir.st;
  StepCtl* ctl = &mir.ctl;
  if (threadIdx.x == 0 && threadIdx.y == 0) [&] {
  phase_time(st, ctl, 1);
  span_end(ctl, 0);
  ctl->kernels += 1;
  const double n = (double)d->ndof;
  if (ctl->fresh) {
    // the set-up of the line search (the other graph's ctl_b, without a step
    // cap): when g.P > 0 the direction is reversed, and this pass, made at
    // +P, is discarded and made again at -P
    ctl->fresh = 0;
    const double gp = v[8];
    ctl->e0 = st->E;
    ctl->k = 0;
    ctl->exhausted = ctl->gmode ? 0 : 1;
    ctl->thr = -0.5 * (gp > 0 ? -gp : gp);
    if (gp > 0) {
      ctl->t = -1.0;
      ctl->retry = 1;
      cudaGraphSetConditional(outer, 1u);
      phase_mark(ctl);
      return;
    }
  }
  if (ctl->gmode) {
    ctl->gmode = 0;
    ctl->retry = 0;
    st->evals++;
    st->abytes += 24.0 * n;
    commit_grad(d, st, ctl, v, outer);
    return;
  }
  for (int j = 0; j < 2; j++) {
    st->evals++;
    if (ctl->e0 - v[4 * j] >= ctl->thr) {
      ctl->exhausted = ctl->k >= 8;
      ctl->acc_hist[ctl->k]++;
      if (j == 1) {
        InstDesc* dw = const_cast<InstDesc*>(d);
        float* tx = dw->X32[1 - st->xi];
        dw->X32[1 - st->xi] = dw->X32s;
        dw->X32s = tx;
        float* tg = dw->G[1 - st->gi];
        dw->G[1 - st->gi] = dw->Gs;
        dw->Gs = tg;
        const int ty = st->ybuf;
        st->ybuf = st->ybuf2;
        st->ybuf2 = ty;
      }
      ctl->retry = 0;
      st->evals++;
      st->abytes += 24.0 * n;
      commit_grad(d, st, ctl, v + 4 * j, outer);
      return;
    }
    st->abytes += 8.0 * n;
    ctl->t *= 0.5;
    ctl->thr *= 0.5;
    ctl->k++;
    if (ctl->k >= 10) break;
  }
  if (ctl->k >= 10) {
    ctl->acc_hist[10]++;
    ctl->gmode = 1;
  }
  ctl->retry = 1;
  cudaGraphSetConditional(outer, 1u);
  phase_mark(ctl);
  }();
  __syncthreads();
  mirror_out(&mir, st_g, ctl_g);
}

int occupancy(const void* f, int threads) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, threads, 0) != cudaSuccess) return 0;
  return per_sm;
}

}  // namespace

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
// the driver's tensor-map encoder, looked up through the runtime (the
// library does not link the driver library itself)
EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return (EncodeTiledFn) nullptr;
    return (EncodeTiledFn)f;
  }();
  return fn;
}
// A tensor map of an FP32 field of grid n at base (dimensions z, y, x
// innermost first) whose box is `lines` lines of one plane.
int encode_lines_map(CUtensorMap* m, const float* base, const int* n, int lines) {
  const EncodeTiledFn f = encode_tiled();
  if (!f) return (int)cudaErrorNotSupported;
  const cuuint64_t dim[3] = {(cuuint64_t)n[2], (cuuint64_t)n[1], (cuuint64_t)n[0]};
  const cuuint64_t stride[2] = {(cuuint64_t)n[2] * sizeof(float), (cuuint64_t)n[2] * n[1] * sizeof(float)};
  const cuuint32_t box[3] = {(cuuint32_t)n[2], (cuuint32_t)lines, 1u};
  const cuuint32_t es[3] = {1u, 1u, 1u};
  const CUresult r = f(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dim, stride, box, es,
                       CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                       CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : (int)cudaErrorInvalidValue;
}

// A stepped graph and the records its kernels run on.  Graphs are kept per
// process, one per shape (grid, history length, SM count, iterations per
// launch, trials per pass): a launch copies the instance's descriptor and
// state record into the graph's own copies and back afterwards, so a new
// instance of a shape seen before reuses the graph built for it
// (instantiating a graph with conditional nodes costs far more than the two
// small copies).
struct SteppedGraph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  StepCtl* ctl = nullptr;
  double* part = nullptr;
  InstDesc* d = nullptr;     // the graph's copy of the descriptor
  MinScalars* st = nullptr;  // the graph's copy of the state record
  int n[3] = {0, 0, 0};
  int m = 0, nsm = 0, slice = 0, dual = 0, spec = 0, tma = 0;
  // TMA trial pass: the tensor maps of the instance's buffers, and the
  // buffer addresses they were encoded for
  TmaMaps* maps = nullptr;
  const void* enc[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  int enc_hstride = 0;
};

}  // namespace mg

using namespace mg;

#define SCK(call)               \
  do {                          \
    const int e_ = (int)(call); \
    if (e_ != 0) return e_;     \
  } while (0)

namespace {

int add_kernel(cudaGraphNode_t* node, cudaGraph_t g, const cudaGraphNode_t* deps, int ndeps, const void* f,
               int blocks, dim3 threads, void** args, unsigned smem = 0) {
  cudaKernelNodeParams p{};
  p.func = const_cast<void*>(f);
  p.gridDim = dim3(blocks);
  p.blockDim = threads;
  p.sharedMemBytes = smem;
  p.kernelParams = args;
  return (int)cudaGraphAddKernelNode(node, g, deps, ndeps, &p);
}

int add_cond(cudaGraphNode_t* node, cudaGraph_t g, const cudaGraphNode_t* deps, int ndeps,
             cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type, cudaGraph_t* body) {
  cudaGraphNodeParams p{};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = h;
  p.conditional.type = type;
  p.conditional.size = 1;
  SCK(cudaGraphAddNode(node, g, deps, nullptr, (size_t)ndeps, &p));
  *body = p.conditional.phGraph_out[0];
  return 0;
}
int add_while(cudaGraphNode_t* node, cudaGraph_t g, const cudaGraphNode_t* deps, int ndeps,
              cudaGraphConditionalHandle h, cudaGraph_t* body) {
  return add_cond(node, g, deps, ndeps, h, cudaGraphCondTypeWhile, body);
}

template <int M>
void dir_kernels_m(const void** a, const void** b) {
  *a = (const void*)k_dir_a<M>;
  *b = (const void*)k_dir_b<M>;
}
// the direction kernels for history length m (1 .. MINIM_MAXM)
bool dir_kernels(int m, const void** a, const void** b) {
  switch (m) {
#define MG_DIR_CASE(M)      \
  case M:                   \
    dir_kernels_m<M>(a, b); \
    return true;
    MG_DIR_CASE(1) MG_DIR_CASE(2) MG_DIR_CASE(3) MG_DIR_CASE(4) MG_DIR_CASE(5) MG_DIR_CASE(6)
    MG_DIR_CASE(7) MG_DIR_CASE(8) MG_DIR_CASE(9) MG_DIR_CASE(10) MG_DIR_CASE(11) MG_DIR_CASE(12)
    MG_DIR_CASE(13) MG_DIR_CASE(14) MG_DIR_CASE(15) MG_DIR_CASE(16)
#undef MG_DIR_CASE
    default:
      return false;
  }
}

int build(SteppedGraph* sg, int m, const int* grid, int nsm, int slice, int dual, int spec, int tma,
          cudaStream_t s) {
  const void* fa = nullptr;
  const void* fb = nullptr;
  if (!dir_kernels(m, &fa, &fb)) return (int)cudaErrorInvalidValue;
  // the line-shaped stencil when z splits into quads and a block holds whole
  // warps of lines (nz / 4 quads x lines per block <= 256 threads)
  const int nz4 = grid[2] / 4;
  const bool lines = grid[2] % 4 == 0 && nz4 <= 256;
  int by = lines ? kThreads / nz4 : 1;
  while (lines && by > 1 && (nz4 * by) % 32) by--;
  const bool use_lines = lines && (nz4 * by) % 32 == 0;
  const dim3 sblock = use_lines ? dim3(nz4, by) : dim3(kThreads);
  // trials that also evaluate the gradient at their point (kept when the
  // trial is accepted) unless MINIM_GPU_SPECULATIVE=0; two trials per pass
  // (with the gradient-only pass folded into the same kernel) when the
  // workspace has the spare buffers
  const bool two = spec && use_lines && dual;
  const int bmode = two ? 2 : spec;  // direction pass B's set-up of the trials
  // blocks of at most 192 threads take the two-trial pass compiled for
  // three blocks per SM (96 registers) unless MINIM_GPU_LINES_B3=0
  const char* b3env = std::getenv("MINIM_GPU_LINES_B3");
  const bool b3 = sblock.x * sblock.y <= 192 && !(b3env && b3env[0] == '0');
  const void* f3 = b3 ? (const void*)k_lines<3, 3, 192> : (const void*)k_lines<3>;
  const void* fe = spec ? (use_lines ? (dual ? f3 : (const void*)k_lines<2>) : (const void*)k_grad<true>)
                        : (use_lines ? (const void*)k_lines<0> : (const void*)k_eonly);
  const void* fg = use_lines ? (const void*)k_lines<1> : (const void*)k_grad<false>;
  const int occ_a = occupancy(fa, kThreads), occ_b = occupancy(fb, kThreads);
  const int occ_e = occupancy(fe, (int)(sblock.x * sblock.y)), occ_g = occupancy(fg, (int)(sblock.x * sblock.y));
  if (!occ_a || !occ_b || !occ_e || !occ_g) return (int)cudaErrorInvalidConfiguration;
  const int nb_a = nsm * occ_a, nb_b = nsm * occ_b, nb_g = nsm * occ_g;
  int nb_e = nsm * occ_e;
  // the two-trial pass through tensor-map tiles (on request, where the grid
  // takes it): blocks of (nz / 4) x kTmaY threads over strips x plane runs
  const bool use_tma = tma && two && tma_lines_fits(grid[0], grid[1], grid[2]);
  // tma: 1, 2, 3: rings of 4, 6, 8 plane stages
  dim3 eblock = sblock;
  unsigned esmem = 0;
  int nch = 1;
  if (use_tma) {
    const int ns = tma == 3 ? 8 : (tma == 2 ? 6 : 4);
    fe = ns == 8 ? (const void*)k_lines_tma<kThreads, 2, 8>
                 : (ns == 6 ? (const void*)k_lines_tma<kThreads, 2, 6> : (const void*)k_lines_tma<kThreads, 3, 4>);
    eblock = dim3(nz4, kTmaY);
    esmem = (unsigned)tma_lines_smem(grid[2], ns);
    SCK(cudaFuncSetAttribute(fe, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)esmem));
    int occ = 0;
    SCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fe, (int)(eblock.x * eblock.y), (int)esmem));
    if (!occ) return (int)cudaErrorInvalidConfiguration;
    nb_e = tma_shape(grid, nsm * occ, &nch);
    SCK(cudaMallocAsync((void**)&sg->maps, sizeof(TmaMaps), s));
  }
  const int nb_max = std::max(std::max(nb_a, nb_b), std::max(nb_e, nb_g));
  SCK(cudaMallocAsync((void**)&sg->d, sizeof(InstDesc), s));
  SCK(cudaMallocAsync((void**)&sg->st, sizeof(MinScalars), s));
  SCK(cudaMallocAsync((void**)&sg->ctl, sizeof(StepCtl), s));
  if ((nb_a + kGroup - 1) / kGroup > kMaxGroups) return (int)cudaErrorInvalidConfiguration;
  // rows of every block, then the group rows of the direction pass A
  SCK(cudaMallocAsync((void**)&sg->part, ((size_t)nb_max + kMaxGroups) * MINIM_WIDE * sizeof(double), s));
  SCK(cudaMemsetAsync(sg->ctl, 0, sizeof(StepCtl), s));
  for (int k = 0; k < 3; k++) sg->n[k] = grid[k];
  sg->m = m;
  sg->nsm = nsm;
  sg->slice = slice;
  sg->dual = dual;
  sg->spec = spec;
  sg->tma = tma;
  const InstDesc* d = sg->d;
  MinScalars* st = sg->st;
  int timing = std::getenv("MINIM_GPU_STEPPED_TIMING") != nullptr;
  cudaGraph_t g = nullptr;
  SCK(cudaGraphCreate(&g, 0));
  sg->graph = g;
  cudaGraphConditionalHandle h_outer, h_ls = 0;
  SCK(cudaGraphConditionalHandleCreate(&h_outer, g, 1, cudaGraphCondAssignDefault));
  StepCtl* ctl = sg->ctl;
  double* part = sg->part;
  cudaGraphNode_t n_begin, n_outer;
  {
    void* args[] = {(void*)&d, (void*)&st, (void*)&ctl, (void*)&sg->slice, (void*)&timing, (void*)&h_outer};
    SCK(add_kernel(&n_begin, g, nullptr, 0, (const void*)k_begin, 1, 32, args));
  }
  cudaGraph_t body;
  SCK(add_while(&n_outer, g, &n_begin, 1, h_outer, &body));
  if (!two) SCK(cudaGraphConditionalHandleCreate(&h_ls, body, 0, 0));
  cudaGraphConditionalHandle h_grad = 0;
  if (spec && !two) SCK(cudaGraphConditionalHandleCreate(&h_grad, body, 0, 0));
  cudaGraphNode_t na, nb, nls, ngr;
  {
    void* args[] = {(void*)&d, (void*)&st, (void*)&ctl, (void*)&part};
    SCK(add_kernel(&na, body, nullptr, 0, fa, nb_a, kThreads, args));
  }
  {
    void* args[] = {(void*)&d, (void*)&st, (void*)&ctl, (void*)&part, (void*)&h_ls, (void*)&h_grad, (void*)&bmode};
    SCK(add_kernel(&nb, body, &na, 1, fb, nb_b, kThreads, args));
  }
  void* args_s[] = {(void*)&d, (void*)&st, (void*)&ctl, (void*)&part, (void*)&h_ls, (void*)&h_grad, (void*)&h_outer};
  cudaGraph_t ls_body;
  if (two) {
    // dirA -> dirB -> trial pass: a pass that accepts a trial (or is the
    // gradient-only pass) ends the iteration; one that does not sets
    // `retry`, and the next pass of the outer loop skips the direction
    cudaGraphNode_t nt;
    if (use_tma) {
      TmaMaps* maps = sg->maps;
      void* args_t[] = {(void*)&d,     (void*)&st,      (void*)&ctl,  (void*)&part, (void*)&h_ls,
                        (void*)&h_grad, (void*)&h_outer, (void*)&maps, (void*)&nch};
      SCK(add_kernel(&nt, body, &nb, 1, fe, nb_e, eblock, args_t, esmem));
    } else {
      SCK(add_kernel(&nt, body, &nb, 1, fe, nb_e, sblock, args_s));
    }
    SCK(cudaGraphInstantiate(&sg->exec, g, 0));
    return 0;
  }
  SCK(add_while(&nls, body, &nb, 1, h_ls, &ls_body));
  {
    cudaGraphNode_t ne;
    SCK(add_kernel(&ne, ls_body, nullptr, 0, fe, nb_e, sblock, args_s));
  }
  if (spec) {
    // the gradient kernel runs only when no trial was accepted
    cudaGraph_t g_body;
    SCK(add_cond(&ngr, body, &nls, 1, h_grad, cudaGraphCondTypeIf, &g_body));
    cudaGraphNode_t ng;
    SCK(add_kernel(&ng, g_body, nullptr, 0, fg, nb_g, sblock, args_s));
  } else {
    SCK(add_kernel(&ngr, body, &nls, 1, fg, nb_g, sblock, args_s));
  }
  SCK(cudaGraphInstantiate(&sg->exec, g, 0));
  return 0;
}

}  // namespace

namespace {
std::mutex g_graphs_mu;
std::vector<SteppedGraph*> g_graphs;  // most recently used last
constexpr size_t kMaxGraphs = 8;

void free_graph(SteppedGraph* sg) {
  if (sg->exec) cudaGraphExecDestroy(sg->exec);
  if (sg->graph) cudaGraphDestroy(sg->graph);
  if (sg->ctl) cudaFree(sg->ctl);
  if (sg->part) cudaFree(sg->part);
  if (sg->d) cudaFree(sg->d);
  if (sg->st) cudaFree(sg->st);
  if (sg->maps) cudaFree(sg->maps);
  delete sg;
}
}  // namespace

// Runs up to `slice` FP32 L-BFGS iterations (history m) of the binary
// PhaseField instance (device descriptor d, host copy hd, state st) as one
// graph launch on stream s, with the graph of this shape (built on first
// use).  The trial pass stages its lines through tensor-map tiles when
// MINIM_GPU_LINES_TMA=1 (default kTmaLinesDefault) and the grid takes them.
// Adds the kernels executed to *kernels.  Returns a cudaError_t
// (cudaErrorLaunchTimeout when a tile's copy wait gave up).
extern "C" int mg_stepped_pf1_run(InstDesc* d, const InstDesc* hd, MinScalars* st, int m, const int* grid,
                                  int nsm, int slice, int dual, void* stream, double* kernels) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const char* env = std::getenv("MINIM_GPU_SPECULATIVE");
  const int spec = !(env && env[0] == '0');
  const char* tenv = std::getenv("MINIM_GPU_LINES_TMA");
  const int tma = tenv ? std::atoi(tenv) : kTmaLinesDefault;
  std::lock_guard<std::mutex> lk(g_graphs_mu);
  SteppedGraph* sg = nullptr;
  for (size_t i = 0; i < g_graphs.size(); i++) {
    SteppedGraph* c = g_graphs[i];
    if (c->n[0] == grid[0] && c->n[1] == grid[1] && c->n[2] == grid[2] && c->m == m && c->nsm == nsm &&
        c->slice == slice && c->dual == dual && c->spec == spec && c->tma == tma) {
      sg = c;
      g_graphs.erase(g_graphs.begin() + (long)i);
      g_graphs.push_back(sg);
      break;
    }
  }
  if (!sg) {
    if (g_graphs.size() >= kMaxGraphs) {
      SCK(cudaDeviceSynchronize());
      free_graph(g_graphs.front());
      g_graphs.erase(g_graphs.begin());
    }
    sg = new SteppedGraph;
    const int rc = build(sg, m, grid, nsm, slice, dual, spec, tma, s);
    if (rc) {
      cudaStreamSynchronize(s);
      free_graph(sg);
      return rc;
    }
    g_graphs.push_back(sg);
  }
  const bool timing = std::getenv("MINIM_GPU_STEPPED_TIMING") != nullptr;
  if (timing) {  // span records of this launch only
    const size_t o = offsetof(StepCtl, gap_pre);
    SCK(cudaMemsetAsync(reinterpret_cast<char*>(sg->ctl) + o, 0, sizeof(StepCtl) - o, s));
  }
  if (sg->maps) {
    // tensor maps of this instance's three coordinate buffers (the set is
    // the same whichever the controllers have exchanged) and m + 1
    // direction slots, encoded again when the buffers differ from the last
    const void* enc[5] = {hd->X32[0], hd->X32[1], hd->X32s, hd->Sb, nullptr};
    bool same = hd->hstride == sg->enc_hstride;
    for (int k = 0; k < 4; k++) same = same && enc[k] == sg->enc[k];
    if (!same) {
      if (!hd->X32s || m + 1 > MINIM_MAXM + 1) return (int)cudaErrorInvalidValue;
      TmaMaps hm{};
      const float* xb[3] = {hd->X32[0], hd->X32[1], hd->X32s};
      for (int k = 0; k < kTmaBufs; k++) {
        const float* base = k < 3 ? xb[k] : (k - 3 <= m ? hd->Sb + (long long)(k - 3) * hd->hstride : nullptr);
        if (!base) continue;
        SCK(encode_lines_map(&hm.box[k], base, grid, kTmaSlots));
        SCK(encode_lines_map(&hm.line[k], base, grid, 1));
      }
      for (int k = 0; k < 3; k++) hm.xbase[k] = xb[k];
      SCK(cudaMemcpyAsync(sg->maps, &hm, sizeof hm, cudaMemcpyHostToDevice, s));
      SCK(cudaStreamSynchronize(s));
      for (int k = 0; k < 4; k++) sg->enc[k] = enc[k];
      sg->enc_hstride = hd->hstride;
    }
  }
  SCK(cudaMemcpyAsync(sg->d, d, sizeof(InstDesc), cudaMemcpyDeviceToDevice, s));
  SCK(cudaMemcpyAsync(sg->st, st, sizeof(MinScalars), cudaMemcpyDeviceToDevice, s));
  SCK(cudaGraphLaunch(sg->exec, s));
  // the accepted trial's buffers may have been exchanged in the copy
  SCK(cudaMemcpyAsync(d, sg->d, sizeof(InstDesc), cudaMemcpyDeviceToDevice, s));
  SCK(cudaMemcpyAsync(st, sg->st, sizeof(MinScalars), cudaMemcpyDeviceToDevice, s));
  StepCtl c;
  SCK(cudaMemcpyAsync(&c, sg->ctl, sizeof c, cudaMemcpyDeviceToHost, s));
  SCK(cudaStreamSynchronize(s));
  if (kernels) *kernels += c.kernels;
  if (c.tma_err) return (int)cudaErrorLaunchTimeout;
  if (timing) {
    static const char* name[4] = {"trials", "gradient", "dirA", "dirB"};
    for (int j = 0; j < 4; j++)
      std::fprintf(stderr, "stepped spans (ms): %-8s gap %.3f kernel %.3f row sums %.3f scalar work %.3f\n",
                   name[j], c.gap_pre[j] * 1e-6, c.kdur[j] * 1e-6, c.gap_post[j] * 1e-6, c.work[j] * 1e-6);
    std::fprintf(stderr, "stepped accepted trial:");
    for (int k = 0; k < 11; k++) std::fprintf(stderr, " %u", c.acc_hist[k]);
    std::fprintf(stderr, "\n");
  }
  return 0;
}

// Frees every cached stepped graph (the device must be idle).
extern "C" void mg_stepped_free_all() {
  std::lock_guard<std::mutex> lk(g_graphs_mu);
  for (SteppedGraph* sg : g_graphs) free_graph(sg);
  g_graphs.clear();
}

// One line-stencil pass outside the graph (no controller), for checking the
// stencil against an FP64 evaluation: mode 0 the trial energy at X + t P;
// mode 3 the points, gradients and y = g - Go at t (Xa, Ga, Ya) and at t/2
// (Xb, Gb, Yb).  Each block's partial row goes to part (at most max_rows
// rows of MINIM_WIDE doubles); *rows receives the block count.  The grid
// must take the line stencil (nz % 4 == 0, nz / 4 <= 256).  Returns a
// cudaError_t.
extern "C" int mg_stepped_lines_probe(const InstDesc* d, const int* grid, int mode, const float* X,
                                      const float* P, const float* Go, float t, float* Xa, float* Ga, float* Ya,
                                      float* Xb, float* Gb, float* Yb, double* part, int max_rows, int nsm,
                                      int* rows, void* stream) {
  const int nz4 = grid[2] / 4;
  if (grid[2] % 4 != 0 || nz4 > 256 || nz4 < 1) return (int)cudaErrorInvalidValue;
  int by = kThreads / nz4;
  while (by > 1 && (nz4 * by) % 32) by--;
  if ((nz4 * by) % 32) return (int)cudaErrorInvalidValue;
  const dim3 blk(nz4, by);
  const void* f = mode == 3 ? (const void*)k_lines_probe<3> : (const void*)k_lines_probe<0>;
  if (mode != 0 && mode != 3) return (int)cudaErrorInvalidValue;
  const int occ = occupancy(f, (int)(blk.x * blk.y));
  if (occ < 1) return (int)cudaErrorInvalidConfiguration;
  const int nb = std::min(nsm * occ, max_rows);
  LinesIO io{X, P, Go, Xa, Ga, Ya, Xb, Gb, Yb, t, mode == 3};
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (mode == 3) k_lines_probe<3><<<nb, blk, 0, s>>>(d, io, part);
  else k_lines_probe<0><<<nb, blk, 0, s>>>(d, io, part);
  *rows = nb;
  return (int)cudaGetLastError();
}


// The TMA line stencil's two-trial pass outside the graph: the points,
// gradients and y = g - Go at t (Xa, Ga, Ya) and t/2 (Xb, Gb, Yb) of
// lines_sweep_tma, for checking it against the direct line stencil and an
// FP64 evaluation.  Arguments as mg_stepped_lines_probe's; the grid must
// satisfy tma_lines_fits.  Synchronises the stream; a copy wait that gave up
// returns cudaErrorLaunchTimeout.
extern "C" int mg_stepped_lines_tma_probe(const InstDesc* d, const int* grid, const float* X, const float* P,
                                          const float* Go, float t, float* Xa, float* Ga, float* Ya, float* Xb,
                                          float* Gb, float* Yb, double* part, int max_rows, int nsm, int* rows,
                                          void* stream) {
  if (!tma_lines_fits(grid[0], grid[1], grid[2])) return (int)cudaErrorInvalidValue;
  const dim3 blk(grid[2] / 4, kTmaY);
  const void* f = (const void*)k_lines_tma_probe;
  const int smem = (int)tma_lines_smem(grid[2]);
  SCK(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  int occ = 0;
  SCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, f, (int)(blk.x * blk.y), smem));
  if (occ < 1) return (int)cudaErrorInvalidConfiguration;
  int nch = 1;
  const int nb = tma_shape(grid, nsm * occ, &nch);
  if (nb > max_rows) return (int)cudaErrorInvalidConfiguration;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  TmaMaps hm{};
  SCK(encode_lines_map(&hm.box[0], X, grid, kTmaSlots));
  SCK(encode_lines_map(&hm.line[0], X, grid, 1));
  SCK(encode_lines_map(&hm.box[1], P, grid, kTmaSlots));
  SCK(encode_lines_map(&hm.line[1], P, grid, 1));
  char* dm = nullptr;
  SCK(cudaMallocAsync((void**)&dm, sizeof(TmaMaps) + 128, s));
  TmaMaps* maps = reinterpret_cast<TmaMaps*>(dm);
  int* err = reinterpret_cast<int*>(dm + sizeof(TmaMaps));
  int herr = 0;
  int rc = (int)cudaMemcpyAsync(maps, &hm, sizeof hm, cudaMemcpyHostToDevice, s);
  if (!rc) rc = (int)cudaMemsetAsync(err, 0, sizeof(int), s);
  if (!rc) {
    LinesIO io{X, P, Go, Xa, Ga, Ya, Xb, Gb, Yb, t, true};
    k_lines_tma_probe<<<nb, blk, smem, s>>>(d, io, maps, nch, part, err);
    rc = (int)cudaGetLastError();
  }
  if (!rc) rc = (int)cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(dm, s);
  if (!rc) rc = (int)cudaStreamSynchronize(s);
  if (!rc && herr) rc = (int)cudaErrorLaunchTimeout;
  *rows = nb;
  return rc;
}
