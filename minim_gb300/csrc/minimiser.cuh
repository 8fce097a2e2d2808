// minimiser.cuh -- device-resident Lbfgs / Fire / GradDescent iterations.
//
// One implementation serves both teams (one CTA per instance in a batch, or
// the whole grid for a single instance).  It follows the reference's
// iteration semantics step by step:
//   Minimiser::minimise           src/Minimiser.cpp:27-38
//   Lbfgs::iteration/getDirection src/minimisers/Lbfgs.cpp:41-133
//   Fire::init/iteration          src/minimisers/Fire.cpp:27-90
//   GradDescent::iteration        src/minimisers/GradDescent.cpp:27-46
//   backtrackingLinesearch        src/minimisers/linesearch.cpp:8-30
// Differences of representation, not of algorithm:
//   * vectors are FP32, every dot product and energy is reduced in FP64;
//   * a step is kept as (scalar t, direction P): trial points x + t*P are
//     evaluated on the fly, the accepted point is written by the gradient
//     evaluation that follows, and s = t*P is stored as (t, P) -- the
//     reference scales the step by tau = 0.5, which is exact in binary;
//   * the energy at the current point is carried from the last evaluation
//     instead of being recomputed at the start of each line search;
//   * the L-BFGS direction uses the compact representation (same direction);
//   * precision MIXED runs FP32 coordinates while FP32 can make progress,
//     FP64 coordinates near convergence; the final convergence test is on
//     FP64 coordinates (the gradient from the FP64 stage's arithmetic:
//     double-float for Lennard-Jones pairs, general PhaseField and
//     BarAndHinge; each component stored in FP32).
// Vector passes move 4 floats per access (float4): every FP32 vector starts
// on a 16-byte boundary (history buffers are strided by a multiple of 64).
#pragma once
#include "potentials.cuh"

namespace mg {

// Writes the gradient (FP32), applies fixed-dof constraints and accumulates
// g.g and, for L-BFGS, y = g_new - g_old with P.y and y.y.
struct FusedEmit {
  float* G;
  const float* Gold;
  const float* P;
  float* Y;
  const unsigned char* fixed;
  Acc gg, py, yy;
  template <typename T>
  __device__ __forceinline__ void operator()(int i, T v) {
    float g = (fixed && fixed[i]) ? 0.f : (float)v;
    G[i] = g;
    gg.add(g * g);
    if (Y) {
      const float y = g - Gold[i];
      Y[i] = y;
      py.add(P[i] * y);
      yy.add(y * y);
    }
  }
  // four consecutive DOFs 4*i4 .. 4*i4+3 (16-byte aligned); pre4 loads
  // the old gradient and the direction ahead of the stencil's arithmetic
  struct Pre4 {
    float4 go, p;
  };
  __device__ __forceinline__ void prefetch4(int i4) const {
    if (Y) prefetch_line(Gold, i4);
  }
  __device__ __forceinline__ Pre4 pre4(int i4) const {
    Pre4 r{};
    if (Y) {
      r.go = ld4(Gold, i4);
      r.p = ld4(P, i4);
    }
    return r;
  }
  __device__ __forceinline__ void emit4(int i4, float4 g, const Pre4& pre) {
    if (fixed) {
      const int i = 4 * i4;
      if (fixed[i]) g.x = 0.f;
      if (fixed[i + 1]) g.y = 0.f;
      if (fixed[i + 2]) g.z = 0.f;
      if (fixed[i + 3]) g.w = 0.f;
    }
    st4(G, i4, g);
    gg.add(dot4(g, g));
    if (Y) {
      const float4 go = pre.go;
      const float4 y = make_float4(g.x - go.x, g.y - go.y, g.z - go.z, g.w - go.w);
      st4(Y, i4, y);
      py.add(dot4(pre.p, y));
      yy.add(dot4(y, y));
    }
  }
};

// FP64 output (API evaluation)
struct StoreEmit64 {
  double* G;
  const unsigned char* fixed;
  template <typename T>
  __device__ __forceinline__ void operator()(int i, T v) {
    G[i] = (fixed && fixed[i]) ? 0.0 : (double)v;
  }
};

// Work counters and phase timers are only read from thread 0 (which stores
// the state): only thread 0 updates them, so the other threads issue no FP64
// instruction for them (FP64 runs at 1/64 of the FP32 rate on GB300).
#define MG_ACCT(ctr, expr)            \
  do {                                \
    if (threadIdx.x == 0) (ctr) += (expr); \
  } while (0)

template <class Team, int KIND>
struct Runner {
  Team& tm;
  const InstDesc& in;
  void* smem_pot;     // potential scratch (LJ tiles)
  int lj_tile;
  // uniform scalars (every thread holds identical copies)
  int n, status, initd, iter, ii, stage, xi, gi, evals, fp64_iters, stall, nsteps, pbuf, ybuf;
  int exhausted_run, switch_reason, pend, cool, fp64_fails, resume, resume_exhausted;
  double E, gg, best_rms, dt, a, dtmax, gnorm;
  double rms_v, gnorm_v;  // sqrt(gg / n) and sqrt(gg) of the current gradient
  double abytes, pairs32, pairs64;
  double tph[3];
  // shared arrays (one copy per block; written by thread 0 between barriers)
  double *rho, *sig, *yy, *alpha;
  int *sidx, *yidx;
  double *SY, *YY, *wout;  // m x m matrices, reduction out
  float *coefS, *coefY;     // pass-B coefficients (FP32: no conversion per element)
  long long* boff;                         // history buffer offsets of the slots in order
  unsigned long long* mbar;                // stage "full" barriers (grid team, shared)
  unsigned long long* mbar_empty;          // stage "empty" barriers
  int* stage_err;                          // shared: a stage wait gave up
  unsigned sq;                             // stage uses so far in this launch (uniform)

  __device__ float* Sbuf(int b) const { return in.Sb + (size_t)b * in.hstride; }
  __device__ float* Ybuf(int b) const { return in.Yb + (size_t)b * in.hstride; }
  __device__ int n4() const { return n >> 2; }
  __device__ bool has_constraints() const {
    if constexpr (KIND == K_PF)
      return in.fixed != nullptr || (in.pf.flags & (PF_FIXFLUID | PF_HARD | PF_VOLUME));
    return in.fixed != nullptr;
  }
  __device__ bool global_projection() const {
    return KIND == K_PF && (in.pf.flags & PF_VOLUME);
  }

  // ---- work accounting -------------------------------------------------------------
  __device__ double xbytes() const { return stage ? 8.0 : 4.0; }
  // one potential evaluation: coordinates read (plus the direction for a
  // trial point), gradient written; pair count for Lennard-Jones
  __device__ void count_eval(bool trial, bool want_g) {
    if (threadIdx.x != 0) return;
    double b = xbytes() + (trial ? 4.0 : 0.0) + (want_g ? 4.0 : 0.0);
    if constexpr (KIND == K_LJ) {
      const double np = in.lj.np;
      // N (N - 1) / 2 pairs per evaluation (with a cutoff the pairs evaluated
      // are not counted)
      const double pairs = in.lj.rc2 > 0 ? 0.0 : 0.5 * np * (np - 1);
      if (stage) MG_ACCT(pairs64, pairs);
      else MG_ACCT(pairs32, pairs);
    }
    MG_ACCT(abytes, b * n);
  }

  // ---- potential dispatch -------------------------------------------------------
  // kFast: the FP64-coordinate evaluations of a MIXED-precision minimiser
  // use double-float arithmetic (general PhaseField, BarAndHinge; about 47
  // bits); the API evaluation, FP64-precision minimisations, Anneal's
  // Metropolis energies and a start already near convergence (switch
  // reason 5) use FP64 throughout.  At such a start the gradient may be
  // exactly zero in FP64 but not in double-float, and the first L-BFGS step
  // is a unit step along -g/|g| whenever |g| > 0 (src/minimisers/
  // Lbfgs.cpp:93-97): double-float rounding noise would set its direction.
  __device__ bool df_stage() const { return in.mp.method != 3 && in.mp.precision == 0 && switch_reason != 5; }
  template <typename T, bool kFast = true, class Emit>
  __device__ double pot_eval(CView<T> cv, T* xw, Emit& em, bool want_e, bool want_g) {
    if constexpr (KIND == K_LJ) {
      if (in.lj.rc2 > 0)
        return lj_cells_eval<T>(tm, in.lj, cv, xw, &em, want_e, want_g, (int2*)nullptr, (int*)nullptr, 0);
      if constexpr (!Team::kGrid) {
        // batched path: each pair once, when positions and forces of all
        // particles fit the tile buffer
        const int ntp = ((in.lj.np + 31) >> 5) + (((in.lj.np + 31) >> 5) & 1);
        const bool fits = (size_t)32 * ntp * 7 * sizeof(T) <= kLjSmemBudget && (blockDim.x & 31) == 0;
        if constexpr (std::is_same_v<T, float>) {
          // FP32: tile pairs dealt to the warps, per-warp force accumulators
          if (want_g && (blockDim.x & 31) == 0 &&
              lj_dealt_bytes(in.lj.np, blockDim.x >> 5) <= kLjSmemBudget)
            return lj_eval_dealt(tm, in.lj, cv, xw, &em, want_e, smem_pot);
        }
        if (fits && want_g) return lj_eval_sym<T>(tm, in.lj, cv, xw, &em, want_e, smem_pot);
        if (fits && want_e && !xw) return lj_energy_sym<T>(tm, in.lj, cv, smem_pot);
      }
      return lj_eval<T>(tm, in.lj, cv, xw, &em, want_e, want_g, smem_pot, lj_tile);
    } else if constexpr (KIND == K_PF) {
      if constexpr (kFast && std::is_same_v<T, double>) {
        // the FP32 coordinate buffers are free while the coordinates are FP64
        if (df_stage()) return pf_eval_df(tm, in.pf, cv, xw, &em, want_e, want_g, in.X32[0], in.X32[1]);
      }
      return pf_eval<T>(tm, in.pf, cv, xw, &em, want_e, want_g);
    } else if constexpr (KIND == K_PF1) {
      if ((in.pf.n[2] & 3) == 0) return pf1_eval_quad<T>(tm, in.pf, cv, xw, &em, want_e, want_g);
      return pf1_eval<T>(tm, in.pf, cv, xw, &em, want_e, want_g);
    } else {
      if constexpr (kFast && std::is_same_v<T, double>) {
        if (df_stage())
          return bah_eval_df(tm, in.bah, cv, xw, in.GA, &em, want_e, want_g, in.X32[0], in.X32[1]);
      }
      return bah_eval<T>(tm, in.bah, cv, xw, in.GA, &em, want_e, want_g);
    }
  }

  // Energy (energy-only semantics) and constrained gradient at X[xi] + t*P.
  // write_x: the point is also written to X[1-xi] and becomes current.
  // With want_y the difference to the current gradient goes to Ybuf(ybuf)
  // and py = P.y, yyv = y.y are returned.  The new gradient becomes current.
  __device__ void grad_eval(double t, const float* P, bool write_x, bool want_y, double& py,
                            double& yyv) {
    const unsigned long long t_start = globaltimer_ns();
    float* Gn = in.G[1 - gi];
    const bool proj = global_projection();
    // with a global projection the gradient is finished in a second pass
    FusedEmit em{Gn, in.G[gi], P, (want_y && !proj) ? Ybuf(ybuf) : nullptr, in.fixed};
    double ep;
    if (stage == 0) {
      CView<float> cv{in.X32[xi], P, (float)t};
      ep = pot_eval<float>(cv, write_x ? in.X32[1 - xi] : nullptr, em, true, true);
    } else {
      CView<double> cv{in.X64[xi], P, t};
      ep = pot_eval<double>(cv, write_x ? in.X64[1 - xi] : nullptr, em, true, true);
    }
    if (proj) {
      em.gg = Acc();
      tm.sync();
      if constexpr (KIND == K_PF) pf_volume_project<float>(tm, in.pf, Gn);
      const float* Go = in.G[gi];
      float* Y = want_y ? Ybuf(ybuf) : nullptr;
      for (int i = tm.tid(); i < n; i += tm.nthr()) {
        const float g = Gn[i];
        em.gg.add(g * g);
        if (Y) {
          const float y = g - Go[i];
          Y[i] = y;
          em.py.add(P[i] * y);
          em.yy.add(y * y);
        }
      }
    }
    if (stage == 0) {
      // FP32 partials summed as FP32 pairs; the square roots of the gradient
      // norm once per team (warp 0), not in every thread
      float ps[4], pc[4];
      to_pair(ep, ps[0], pc[0]);
      ps[1] = em.gg.s; pc[1] = em.gg.c;
      ps[2] = em.py.s; pc[2] = em.py.c;
      ps[3] = em.yy.s; pc[3] = em.yy.c;
      const double nd = (double)n;
      double v[6];
      tm.template reduce_pairs<4, 2>(ps, pc, v, [nd](double* o) {
        o[4] = sqrt(o[1] / nd);
        o[5] = sqrt(o[1]);
      });
      E = v[0];
      gg = v[1];
      py = v[2];
      yyv = v[3];
      rms_v = v[4];
      gnorm_v = v[5];
    } else {
      double v[4] = {ep, em.gg.total(), em.py.total(), em.yy.total()};
      tm.reduce(v);
      E = v[0];
      gg = v[1];
      py = v[2];
      yyv = v[3];
      rms_v = sqrt(gg / n);
      gnorm_v = sqrt(gg);
    }
    evals++;
    count_eval(P != nullptr, true);
    if (write_x) MG_ACCT(abytes, xbytes() * n);
    if (want_y) MG_ACCT(abytes, 8.0 * n);
    gi = 1 - gi;
    if (write_x) xi = 1 - xi;
    MG_ACCT(tph[0], (double)(globaltimer_ns() - t_start));
  }

  __device__ double energy_at(double t, const float* P) {
    const unsigned long long t_start = globaltimer_ns();
    FusedEmit ne{nullptr, nullptr, nullptr, nullptr, nullptr};
    double ep;
    if (stage == 0) {
      CView<float> cv{in.X32[xi], P, (float)t};
      ep = pot_eval<float>(cv, nullptr, ne, true, false);
    } else {
      CView<double> cv{in.X64[xi], P, t};
      ep = pot_eval<double>(cv, nullptr, ne, true, false);
    }
    double v[1] = {ep};
    if (stage == 0) {
      float ps[1], pc[1];
      to_pair(ep, ps[0], pc[0]);
      tm.template reduce_pairs<1>(ps, pc, v);
    } else {
      tm.reduce(v);
    }
    evals++;
    count_eval(P != nullptr, false);
    MG_ACCT(tph[1], (double)(globaltimer_ns() - t_start));
    return v[0];
  }

  // g . P over the team
  __device__ double dot_gP(const float* P) {
    const float* G = in.G[gi];
    Acc d;
    for (int i = tm.tid(); i < n4(); i += tm.nthr()) d.add(dot4(ld4(G, i), ld4(P, i)));
    for (int i = 4 * n4() + tm.tid(); i < n; i += tm.nthr()) d.add(G[i] * P[i]);
    float ps[1] = {d.s}, pc[1] = {d.c};
    double v[1];
    tm.template reduce_pairs<1>(ps, pc, v);
    return v[0];
  }

  // State::applyConstraints on the direction P, then returns g.P
  __device__ double constrain_dir(float* P) {
    // the element form (PhaseFieldUnstructured) applies fixed degrees of
    // freedom after its own constraints
    bool fixed_last = false;
    if constexpr (KIND == K_PF) fixed_last = (in.pf.flags & PF_UNSTR) != 0;
    if (in.fixed && !fixed_last) {
      for (int i = tm.tid(); i < n; i += tm.nthr())
        if (in.fixed[i]) P[i] = 0.f;
    }
    if constexpr (KIND == K_PF) {
      if (in.pf.flags & (PF_FIXFLUID | PF_HARD)) {
        tm.sync();
        pf_local_constrain<float>(tm, in.pf, P);
      }
      if (global_projection()) {
        tm.sync();
        pf_volume_project<float>(tm, in.pf, P);
      }
    }
    if (in.fixed && fixed_last) {
      tm.sync();
      for (int i = tm.tid(); i < n; i += tm.nthr())
        if (in.fixed[i]) P[i] = 0.f;
    }
    tm.sync();
    return dot_gP(P);
  }

  // backtrackingLinesearch: the step is t0 * P with g.step = gs <= 0.
  // Returns the accepted multiplier (t0 * tau^k, or t0 * tau^10 when no
  // trial passed -- that last point is taken without being evaluated).
  // `exhausted` (for the precision policy only) reports that no trial
  // passed or that one passed only after 8 or more halvings: the energy no
  // longer resolves the decrease the gradient predicts.
  __device__ double linesearch(const float* P, double t0, double gs, bool& exhausted) {
    const double c = 0.5, tau = 0.5;
    double thr = -c * gs;
    const double e0 = E;
    double t = t0;
    exhausted = true;
    for (int k = 0; k < 10; k++) {
      const double e = energy_at(t, P);
      if (!tm.ok()) return t;
      if (e0 - e >= thr) { exhausted = k >= 8; break; }
      t = t * tau;
      thr = thr * tau;
    }
    return t;
  }

  // ---- L-BFGS ---------------------------------------------------------------------
  // Direction -H g of Lbfgs::getDirection in the compact representation of
  // Byrd, Nocedal & Schnabel (1994): with the stored pairs in order oldest ->
  // newest, R = upper triangle of S^T Y, D its diagonal and
  // gamma = s_n.y_n / y_n.y_n,
  //   H g = gamma g + S w - gamma Y u,   R u = S^T g,
  //   R^T w = (D + gamma Y^T Y) u - gamma Y^T g,
  // which equals the two-loop recursion's result for any pairs with s.y != 0
  // (including s.y < 0, which the reference keeps).  Two passes over the
  // history and two team reductions, instead of 2 min(m,i) + 1.  The new
  // pair's column of S^T Y and Y^T Y is computed in the first pass.
  // Writes P = Sbuf(pbuf); returns the scale folded into the step
  // (initStep/|g| on the first iteration, or the maxStep cap).
  __device__ double lbfgs_direction(double& gp) {
    float* P = Sbuf(pbuf);
    const float* G = in.G[gi];
    const int m = in.mp.m;
    if (ii == 0) {
      for (int i = tm.tid(); i < n4(); i += tm.nthr()) {
        const float4 g = ld4(G, i);
        st4(P, i, make_float4(-g.x, -g.y, -g.z, -g.w));
      }
      for (int i = 4 * n4() + tm.tid(); i < n; i += tm.nthr()) P[i] = -G[i];
      tm.sync();
      MG_ACCT(abytes, 8.0 * n);
      const double gn = gnorm_v;
      const double scale = gn > 0 ? in.mp.init_step / gn : 1.0;
      gp = -gg * scale;
      return scale;
    }
    const int mt = ii < m ? ii : m;
    const int c = ii % m;
    const int kn = (c - 1 + m) % m;  // newest slot
    MG_ACCT(abytes, (4.0 * mt + 2.0) * 4.0 * n);
    const bool np = pend >= 0;
    const bool staged = stage_chunk(2 + 2 * mt) > 0;
    if (staged) pass_a_staged(G, mt, c, np);
    else pass_a_plain(G, mt, c, np);
    if (!tm.ok()) return 1.0;
    direction_algebra(mt, c, kn, np);
    pend = -1;
    Acc pv[2];
    if (staged && stage_chunk(1 + 2 * mt) > 0) pass_b_staged(G, P, mt, pv);
    else pass_b_plain(G, P, mt, pv);
    double v[2];
    {
      float ps[2] = {pv[0].s, pv[1].s}, pc[2] = {pv[0].c, pv[1].c};
      tm.template reduce_pairs<2>(ps, pc, v);
    }
    gp = v[0];
    double scale = 1.0;
    if (in.mp.max_step != 0) {
      const double ss = sqrt(v[1]);
      if (ss > in.mp.max_step) scale = in.mp.max_step / ss;
    }
    gp *= scale;
    return scale;
  }

  // slot (in age order k = 0 .. mt-1, oldest first) of the history ring
  __device__ __forceinline__ int slot_of(int k, int mt, int c) const {
    const int m = in.mp.m;
    return (c - mt + k + 2 * m) % m;
  }

  // ---- staging of vector passes through shared memory (grid team) ------------------
  // Chunk length for nv vectors: the largest multiple of 64 floats whose nv
  // rows fit one stage (0 = the passes read global memory directly).
  __device__ int stage_chunk(int nv) const {
    if constexpr (!Team::kGrid || Team::kCluster) {
      return 0;
    } else {
      if (in.stage_bytes <= 0) return 0;
      const int ch = (in.stage_bytes / (4 * nv)) & ~63;
      return ch >= 64 ? ch : 0;
    }
  }
  __device__ StageRing make_ring(int nv) const {
    StageRing r;
    r.base = static_cast<char*>(smem_pot);
    r.full = mbar;
    r.empty = mbar_empty;
    r.err = stage_err;
    r.stage_bytes = in.stage_bytes;
    r.n = n;
    r.nv = nv;
    r.ch = stage_chunk(nv);
    r.sq = sq;
    r.mine = r.j = r.issued = 0;
    return r;
  }
  // after a staged sweep: keep the use count, stop the team on a failed wait
  __device__ void ring_done(StageRing& r) {
    const bool ok = r.end();
    sq = r.sq;
    if (!ok) {
      tm.fail();
      __syncthreads();
    }
  }

  // pass A: S_k.g, Y_k.g and, for a new pair, S_k.y_new, Y_k.y_new;
  // value index = dot * 16 + slot order (oldest first)
  __device__ __noinline__ void pass_a_plain(const float* G, int mt, int c, bool np) {
    // everything the loops use is held in registers (no member access
    // through memory inside them)
    const long long hs = in.hstride;
    const int nn = n, nq4 = n >> 2, t0 = tm.tid(), nt = tm.nthr(), pd = in.pf_dist * nt;
    const float* Yn = np ? Ybuf(yidx[pend]) : nullptr;
    const float* Sb = in.Sb;
    const float* Yb = in.Yb;
    tm.wide_clear();
    for (int k0 = 0; k0 < mt; k0 += 8) {
      const float* Sp[8];
      const float* Yp[8];
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const int k = k0 + j;
        const int s = slot_of(k, mt, c);
        Sp[j] = Sb + ((k < mt) ? sidx[s] : 0) * hs;
        Yp[j] = Yb + ((k < mt) ? yidx[s] : 0) * hs;
      }
      const int nk = min(8, mt - k0);
      float acc[32];
#pragma unroll
      for (int k = 0; k < 32; k++) acc[k] = 0.f;
      for (int i = t0; i < nq4; i += nt) {
        const int ip = i + pd;  // pf_dist sweep steps ahead: fetch into L2 now
        if (pd > 0 && ip < nq4) {
          prefetch_line(G, ip);
          if (np) prefetch_line(Yn, ip);
#pragma unroll
          for (int j = 0; j < 8; j++)
            if (j < nk) {
              prefetch_line(Sp[j], ip);
              prefetch_line(Yp[j], ip);
            }
        }
        const float4 g = ld4(G, i);
        const float4 yn = np ? ld4(Yn, i) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int j = 0; j < 8; j++) {
          if (j < nk) {
            const float4 s = ld4(Sp[j], i);
            const float4 y = ld4(Yp[j], i);
            acc[j] += dot4(s, g);
            acc[8 + j] += dot4(y, g);
            acc[16 + j] += dot4(s, yn);
            acc[24 + j] += dot4(y, yn);
          }
        }
      }
      for (int i = 4 * nq4 + t0; i < nn; i += nt) {
        const float g = G[i];
        const float yn = np ? Yn[i] : 0.f;
#pragma unroll
        for (int j = 0; j < 8; j++) {
          if (j < nk) {
            const float s = Sp[j][i], y = Yp[j][i];
            acc[j] += s * g;
            acc[8 + j] += y * g;
            acc[16 + j] += s * yn;
            acc[24 + j] += y * yn;
          }
        }
      }
      tm.wide_store32(acc, k0);
    }
    tm.wide_combine(4 * MINIM_MAXM, wout);
  }

  // pass A through shared memory: vectors g, y_new (when np), S_0..S_mt-1,
  // Y_0..Y_mt-1 arrive chunk by chunk; all 4 mt sums stay in registers
  __device__ __noinline__ void pass_a_staged(const float* G, int mt, int c, bool np) {
    if constexpr (Team::kGrid) {
      const long long hs = in.hstride;
      const float* Yn = np ? Ybuf(yidx[pend]) : G;
      const int nv = 2 + 2 * mt;
      auto vec = [&](int v) -> const float* {
        if (v == 0) return G;
        if (v == 1) return Yn;
        if (v < 2 + mt) return in.Sb + (long long)sidx[slot_of(v - 2, mt, c)] * hs;
        return in.Yb + (long long)yidx[slot_of(v - 2 - mt, mt, c)] * hs;
      };
      // the block's threads split into one part per group of 8 slots; a
      // part's threads hold that group's 32 sums (no more live registers
      // than one group needs)
      const int ng = (mt + 7) >> 3;
      const int part_size = blockDim.x / ng;
      const int part = min((int)threadIdx.x / part_size, ng - 1);
      const int k0 = 8 * part;
      const int pt = threadIdx.x - part * part_size;
      float a0[8], a1[8], a2[8], a3[8];
#pragma unroll
      for (int k = 0; k < 8; k++) a0[k] = a1[k] = a2[k] = a3[k] = 0.f;
      StageRing rg = make_ring(nv);
      rg.begin(tm.ok(), vec);
      const int ch = rg.ch;
      while (rg.j < rg.mine) {
        const float* sb = rg.acquire();
        if (!sb) break;
        if ((int)threadIdx.x < ng * part_size) {
          const int cnt = rg.count();
          for (int i = pt; i < cnt; i += part_size) {
            const float g = sb[i];
            const float yn = np ? sb[ch + i] : 0.f;
#pragma unroll
            for (int k = 0; k < 8; k++) {
              if (k0 + k < mt) {
                const float sv = sb[(2 + k0 + k) * ch + i];
                const float yv = sb[(2 + mt + k0 + k) * ch + i];
                a0[k] = fmaf(sv, g, a0[k]);
                a1[k] = fmaf(yv, g, a1[k]);
                a2[k] = fmaf(sv, yn, a2[k]);
                a3[k] = fmaf(yv, yn, a3[k]);
              }
            }
          }
        }
        rg.release(vec);
      }
      ring_done(rg);
      tm.wide_clear();
      {
        float v[32];
#pragma unroll
        for (int j = 0; j < 8; j++) {
          v[j] = a0[j];
          v[8 + j] = a1[j];
          v[16 + j] = a2[j];
          v[24 + j] = a3[j];
        }
        tm.wide_store32(v, k0);
      }
      tm.wide_combine(4 * MINIM_MAXM, wout);
    }
  }

  // small dense algebra on warp 0 of every block (bitwise the same in all):
  // R u = S^T g, R^T w = (D + gamma Y^T Y) u - gamma Y^T g, coefficients of
  // P = -(gamma g + S w - gamma Y u)
  __device__ __noinline__ void direction_algebra(int mt, int c, int kn, bool np) {
    const int m = in.mp.m;
    const long long hs = in.hstride;
    if (threadIdx.x < 32) {
      const int lane = threadIdx.x;
      const bool on = lane < mt;
      const int slk = on ? ring_slot(c, mt, lane, m) : 0;
      double sg = 0.0, yg = 0.0;
      if (on) {
        sg = sig[slk] * wout[lane];
        yg = wout[MINIM_MAXM + lane];
        if (np) {
          SY[slk * MINIM_MAXM + pend] = sig[slk] * wout[2 * MINIM_MAXM + lane];
          YY[slk * MINIM_MAXM + pend] = wout[3 * MINIM_MAXM + lane];
          YY[pend * MINIM_MAXM + slk] = wout[3 * MINIM_MAXM + lane];
        }
      }
      __syncwarp();
      const double gamma = SY[kn * MINIM_MAXM + kn] / YY[kn * MINIM_MAXM + kn];
      const double* sy_ = SY;
      const double* yy_ = YY;
      double u, w;
      lbfgs_compact_warp(
          mt, gamma, sg, yg,
          [=](int a, int b) { return sy_[ring_slot(c, mt, a, m) * MINIM_MAXM + ring_slot(c, mt, b, m)]; },
          [=](int a, int b) { return yy_[ring_slot(c, mt, a, m) * MINIM_MAXM + ring_slot(c, mt, b, m)]; }, u, w);
      if (lane < MINIM_MAXM) {
        coefS[lane] = on ? (float)(-w * sig[slk]) : 0.f;
        coefY[lane] = on ? (float)(gamma * u) : 0.f;
        boff[lane] = on ? (long long)sidx[slk] * hs : 0;
        boff[MINIM_MAXM + lane] = on ? (long long)yidx[slk] * hs : 0;
      }
      if (lane == 0) wout[MINIM_WIDE - 1] = gamma;
    }
    __syncthreads();
  }

  // pass B: P = -(gamma g + S w - gamma Y u), with g.P and P.P; the slot
  // buffers and coefficients are read from shared memory (broadcast)
  __device__ __noinline__ void pass_b_plain(const float* G, float* P, int mt, Acc (&v)[2]) {
    const int nn = n, nq4 = n >> 2, t0 = tm.tid(), nt = tm.nthr(), pd = in.pf_dist * nt;
    const float fg = (float)(-wout[MINIM_WIDE - 1]);
    // slot buffers as 32-bit float4 offsets from the ring bases (the host
    // keeps (m + 1) * hstride below 2^33 floats)
    const float4* Sb4 = reinterpret_cast<const float4*>(in.Sb);
    const float4* Yb4 = reinterpret_cast<const float4*>(in.Yb);
    unsigned so[MINIM_MAXM], yo[MINIM_MAXM];
    float cS[MINIM_MAXM], cY[MINIM_MAXM];
#pragma unroll
    for (int k = 0; k < MINIM_MAXM; k++) {
      so[k] = (unsigned)(boff[k] >> 2);
      yo[k] = (unsigned)(boff[MINIM_MAXM + k] >> 2);
      cS[k] = coefS[k];
      cY[k] = coefY[k];
    }
    Acc d1, d2;
    for (int i = t0; i < nq4; i += nt) {
      const int ip = i + pd;  // pf_dist sweep steps ahead: fetch into L2 now
      if (pd > 0 && ip < nq4) {
        prefetch_line(G, ip);
#pragma unroll
        for (int k = 0; k < MINIM_MAXM; k++)
          if (k < mt) {
            prefetch_line(reinterpret_cast<const float*>(Sb4 + so[k]), ip);
            prefetch_line(reinterpret_cast<const float*>(Yb4 + yo[k]), ip);
          }
      }
      const float4 g = ld4(G, i);
      float4 q = make_float4(fg * g.x, fg * g.y, fg * g.z, fg * g.w);
#pragma unroll
      for (int k = 0; k < MINIM_MAXM; k++) {
        if (k < mt) {
          q = axpy4(cS[k], Sb4[so[k] + i], q);
          q = axpy4(cY[k], Yb4[yo[k] + i], q);
        }
      }
      st4(P, i, q);
      d1.add(dot4(q, g));
      d2.add(dot4(q, q));
    }
    for (int i = 4 * nq4 + t0; i < nn; i += nt) {
      const float g = G[i];
      float q = fg * g;
      for (int k = 0; k < mt; k++) {
        q += cS[k] * in.Sb[boff[k] + i];
        q += cY[k] * in.Yb[boff[MINIM_MAXM + k] + i];
      }
      P[i] = q;
      d1.add(q * g);
      d2.add(q * q);
    }
    v[0] = d1;
    v[1] = d2;
  }

  // pass B through shared memory: g, S_0..S_mt-1, Y_0..Y_mt-1 arrive chunk by
  // chunk; P is written straight to global memory
  __device__ __noinline__ void pass_b_staged(const float* G, float* P, int mt, Acc (&v)[2]) {
    if constexpr (Team::kGrid) {
      const int nv = 1 + 2 * mt;
      auto vec = [&](int k) -> const float* {
        if (k == 0) return G;
        if (k < 1 + mt) return in.Sb + boff[k - 1];
        return in.Yb + boff[MINIM_MAXM + k - 1 - mt];
      };
      const float fg = (float)(-wout[MINIM_WIDE - 1]);
      float cS[MINIM_MAXM], cY[MINIM_MAXM];
#pragma unroll
      for (int k = 0; k < MINIM_MAXM; k++) {
        cS[k] = coefS[k];
        cY[k] = coefY[k];
      }
      Acc d1, d2;
      StageRing rg = make_ring(nv);
      rg.begin(tm.ok(), vec);
      const int ch = rg.ch;
      while (rg.j < rg.mine) {
        const float* sb = rg.acquire();
        if (!sb) break;
        const int i0 = rg.i0();
        const int cnt = rg.count();
        for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
          const float g = sb[i];
          float q = fg * g;
#pragma unroll
          for (int k = 0; k < MINIM_MAXM; k++) {
            if (k < mt) {
              q = fmaf(cS[k], sb[(1 + k) * ch + i], q);
              q = fmaf(cY[k], sb[(1 + mt + k) * ch + i], q);
            }
          }
          P[i0 + i] = q;
          d1.add(q * g);
          d2.add(q * q);
        }
        rg.release(vec);
      }
      ring_done(rg);
      v[0] = d1;
      v[1] = d2;
    }
  }

  __device__ void lbfgs_iteration(bool& exhausted) {
    double py, yyv;
    exhausted = false;
    if (iter == 0) {
      grad_eval(0.0, nullptr, false, false, py, yyv);
      ii = 0;
    } else {
      ii++;
    }
    double gp;
    const unsigned long long t_dir = globaltimer_ns();
    double scale = lbfgs_direction(gp);
    MG_ACCT(tph[2], (double)(globaltimer_ns() - t_dir));
    float* P = Sbuf(pbuf);
    if (has_constraints()) gp = scale * constrain_dir(P);
    double gs = gp;
    if (gs > 0) { gs = -gs; scale = -scale; }
    double t = scale;
    if (in.mp.linesearch == 0) t = linesearch(P, scale, gs, exhausted);
    if (!tm.ok()) return;
    grad_eval(t, P, true, true, py, yyv);
    const double sy = t * py;
    if (sy != 0 && isfinite(sy)) {
      const int m = in.mp.m;
      const int c = ii % m;
      const int os = sidx[c], oy = yidx[c];
      __syncthreads();
      if (threadIdx.x == 0) {
        sidx[c] = pbuf; yidx[c] = ybuf;
        rho[c] = 1.0 / sy; sig[c] = t; yy[c] = yyv;
      }
      pbuf = os; ybuf = oy;
      pend = c;
      __syncthreads();
    } else {
      ii--;
    }
  }

  // ---- FIRE -----------------------------------------------------------------------
  __device__ void fire_iteration(bool& exhausted) {
    const int nMin = 5;
    const double fInc = 1.1, fDec = 0.5, fA = 0.99, aStart = 0.1;
    double py, yyv;
    exhausted = false;
    if (iter == 0) {
      dt = dtmax;
      grad_eval(0.0, nullptr, false, false, py, yyv);
      gnorm = gnorm_v;
    }
    const float* G = in.G[gi];
    float* Vv = in.V;
    const int nn = n, nq4 = n >> 2, t0 = tm.tid(), nt = tm.nthr();
    Acc d1, d2;
    for (int i = t0; i < nq4; i += nt) {
      const float4 v = ld4(Vv, i);
      d1.add(dot4(v, ld4(G, i)));
      d2.add(dot4(v, v));
    }
    for (int i = 4 * nq4 + t0; i < nn; i += nt) {
      const float v = Vv[i];
      d1.add(v * G[i]);
      d2.add(v * v);
    }
    // v.g and v.v as FP32 pairs; |v| and the FIRE mixing factor a |v| / |g|
    // + dt once per team (thread 0 of warp 0)
    double r[4];
    {
      float ps[2] = {d1.s, d2.s}, pc[2] = {d1.c, d2.c};
      const double a_ = a, gn_ = gnorm, dt_ = dt;
      tm.template reduce_pairs<2, 2>(ps, pc, r, [a_, gn_, dt_](double* o) {
        o[2] = sqrt(o[1]);
        o[3] = a_ * o[2] / gn_ + dt_;
      });
    }
    MG_ACCT(abytes, 8.0 * n);
    const double p = -r[0];
    double c1, c2;
    if (p > 0) {
      c1 = 1 - a;
      c2 = r[3];
      nsteps++;
    } else {
      c1 = 0.0;
      c2 = dt;
      nsteps = 0;
    }
    if (p > 0 && nsteps > nMin) {
      a = a * fA;
      dt = dt * fInc;
      if (dt > dtmax) dt = dtmax;
    } else if (p <= 0) {
      a = aStart;
      dt = dt * fDec;
    }
    float* P = Sbuf(0);
    const float f1 = (float)c1, f2 = (float)c2, fdt = (float)dt;
    const bool mix = p > 0;
    Acc dg;
    for (int i = t0; i < nq4; i += nt) {
      const float4 g = ld4(G, i);
      const float4 vo = ld4(Vv, i);
      float4 v;
      v.x = mix ? f1 * vo.x - f2 * g.x : -f2 * g.x;
      v.y = mix ? f1 * vo.y - f2 * g.y : -f2 * g.y;
      v.z = mix ? f1 * vo.z - f2 * g.z : -f2 * g.z;
      v.w = mix ? f1 * vo.w - f2 * g.w : -f2 * g.w;
      st4(Vv, i, v);
      const float4 s = make_float4(fdt * v.x, fdt * v.y, fdt * v.z, fdt * v.w);
      st4(P, i, s);
      dg.add(dot4(g, s));
    }
    for (int i = 4 * nq4 + t0; i < nn; i += nt) {
      const float v = mix ? f1 * Vv[i] - f2 * G[i] : -f2 * G[i];
      Vv[i] = v;
      const float s = fdt * v;
      P[i] = s;
      dg.add(G[i] * s);
    }
    MG_ACCT(abytes, 16.0 * n);
    double gs = 0.0;
    if (has_constraints()) {
      gs = constrain_dir(P);
    } else if (in.mp.linesearch == 0) {  // g.P only for the line search
      float ps[1] = {dg.s}, pc[1] = {dg.c};
      double v[1];
      tm.template reduce_pairs<1>(ps, pc, v);
      gs = v[0];
    }
    double t = 1.0;
    if (in.mp.linesearch == 0) t = linesearch(P, 1.0, gs, exhausted);
    if (!tm.ok()) return;
    grad_eval(t, P, true, false, py, yyv);
    gnorm = gnorm_v;
  }

  // ---- gradient descent -------------------------------------------------------------
  __device__ void gd_iteration(bool& exhausted) {
    double py, yyv;
    exhausted = false;
    grad_eval(0.0, nullptr, false, false, py, yyv);
    const float* G = in.G[gi];
    const double gs = -in.mp.alpha * gg;
    double t = -in.mp.alpha;
    if (in.mp.linesearch == 0) t = linesearch(G, -in.mp.alpha, gs, exhausted);
    if (!tm.ok()) return;
    // x += t * g (materialise the accepted point)
    if (stage == 0) {
      CView<float> cv{in.X32[xi], G, (float)t};
      float* Xn = in.X32[1 - xi];
      for (int i = tm.tid(); i < n; i += tm.nthr()) Xn[i] = cv(i);
    } else {
      CView<double> cv{in.X64[xi], G, t};
      double* Xn = in.X64[1 - xi];
      for (int i = tm.tid(); i < n; i += tm.nthr()) Xn[i] = cv(i);
    }
    xi = 1 - xi;
    tm.sync();
    MG_ACCT(abytes, (2.0 * xbytes() + 4.0) * n);
  }

  // ---- simulated annealing -------------------------------------------------------------
  // Anneal::iteration / acceptMetropolis (src/minimisers/Anneal.cpp:53-88):
  // every coordinate moves by displacement * U(-1, 1) from the last accepted
  // state (X64[xi]) into X64[1 - xi], the energy there decides by the
  // Metropolis rule, and an accepted point becomes current by swapping the
  // two buffers.  FP64 coordinates throughout.
  __device__ void anneal_iteration() {
    const MinParams& mp = in.mp;
    const double T = mp.ntsched > 0 ? mp.tsched[iter < mp.ntsched ? iter : mp.ntsched - 1]
                                    : mp.temp_init / (1 + mp.cooling_rate * iter);
    const double* Xc = in.X64[xi];
    double* Xn = in.X64[1 - xi];
    for (int i = tm.tid(); i < n; i += tm.nthr()) {
      const double r = 2 * anneal_unit(mp.seed, iter, (unsigned)i) - 1;
      Xn[i] = __dadd_rn(Xc[i], __dmul_rn(r, mp.displacement));
    }
    tm.sync();
    const unsigned long long t_start = globaltimer_ns();
    FusedEmit ne{nullptr, nullptr, nullptr, nullptr, nullptr};
    CView<double> cv{Xn, nullptr, 0.0};
    double v[1] = {pot_eval<double, false>(cv, nullptr, ne, true, false)};
    tm.reduce(v);
    evals++;
    count_eval(false, false);
    MG_ACCT(tph[1], (double)(globaltimer_ns() - t_start));
    MG_ACCT(abytes, 16.0 * n);  // the displacement pass: read x, write x'
    const double En = v[0];
    const double u = anneal_unit(mp.seed, iter, (unsigned)n);
    if (En < E || u < exp((E - En) / T)) {
      xi = 1 - xi;
      E = En;
      nsteps = 0;
    } else {
      nsteps++;
    }
  }
  // Anneal::checkConvergence (lines 91-94), then the loop's iter++
  __device__ bool anneal_post() {
    fp64_iters++;
    if (in.mp.max_rej > 0 && nsteps >= in.mp.max_rej) { status = ST_CONVERGED; return true; }
    iter++;
    return false;
  }

  // ---- precision stages -------------------------------------------------------------
  __device__ void to_fp64() {
    const float* X = in.X32[xi];
    double* X64 = in.X64[xi];
    for (int i = tm.tid(); i < n; i += tm.nthr()) X64[i] = (double)X[i];
    tm.sync();
    MG_ACCT(abytes, 12.0 * n);
    stage = 1;
  }
  __device__ void to_fp32() {
    const double* X64 = in.X64[xi];
    float* X = in.X32[xi];
    for (int i = tm.tid(); i < n; i += tm.nthr()) X[i] = (float)X64[i];
    tm.sync();
    MG_ACCT(abytes, 12.0 * n);
    stage = 0;
  }
  // the current gradient (and energy) again at the current point, in the
  // current precision
  __device__ void reeval() {
    double py, yyv;
    grad_eval(0.0, nullptr, false, false, py, yyv);
    if (in.mp.method == 1) gnorm = gnorm_v;
  }

  __device__ double rms() const { return rms_v; }

  // ---- driver -------------------------------------------------------------------------
  __device__ void load(const MinScalars& s) {
    status = s.status; initd = s.initialised; iter = s.iter; ii = s.ii; stage = s.stage;
    xi = s.xi; gi = s.gi; evals = s.evals; fp64_iters = s.fp64_iters; stall = s.stall;
    nsteps = s.nsteps; pbuf = s.pbuf; ybuf = s.ybuf; E = s.E; gg = s.gg; best_rms = s.best_rms;
    exhausted_run = s.exhausted_run; switch_reason = s.switch_reason; pend = s.pend; cool = s.cool;
    fp64_fails = s.fp64_fails;
    resume = s.resume; resume_exhausted = s.resume_exhausted;
    dt = s.dt; a = s.a; dtmax = s.dtmax; gnorm = s.gnorm;
    rms_v = sqrt(gg / n);
    gnorm_v = sqrt(gg);
    abytes = s.abytes; pairs32 = s.pairs32; pairs64 = s.pairs64;
    tph[0] = s.tphase[0]; tph[1] = s.tphase[1]; tph[2] = s.tphase[2];
    for (int k = threadIdx.x; k < MINIM_MAXM * MINIM_MAXM; k += blockDim.x) {
      SY[k] = (&s.SY[0][0])[k];
      YY[k] = (&s.YY[0][0])[k];
    }
    for (int k = threadIdx.x; k < MINIM_MAXM; k += blockDim.x) {
      rho[k] = s.rho[k]; sig[k] = s.sigma[k]; yy[k] = s.yy[k];
      sidx[k] = s.sidx[k]; yidx[k] = s.yidx[k]; alpha[k] = 0.0;
    }
    __syncthreads();
  }

  __device__ void store(MinScalars& s) {
    __syncthreads();
    if (tm.block0() && threadIdx.x == 0) {
      s.status = status; s.iter = iter; s.ii = ii; s.stage = stage; s.xi = xi; s.gi = gi;
      s.evals = evals; s.fp64_iters = fp64_iters; s.stall = stall; s.nsteps = nsteps;
      s.pbuf = pbuf; s.ybuf = ybuf; s.E = E; s.gg = gg; s.best_rms = best_rms;
      s.exhausted_run = exhausted_run; s.switch_reason = switch_reason; s.pend = pend; s.cool = cool;
      s.fp64_fails = fp64_fails;
      s.resume = resume; s.resume_exhausted = resume_exhausted;
      s.dt = dt; s.a = a; s.dtmax = dtmax; s.gnorm = gnorm; s.initialised = 1;
      s.abytes = abytes; s.pairs32 = pairs32; s.pairs64 = pairs64;
      s.tphase[0] = tph[0]; s.tphase[1] = tph[1]; s.tphase[2] = tph[2];
      for (int k = 0; k < MINIM_MAXM * MINIM_MAXM; k++) {
        (&s.SY[0][0])[k] = SY[k];
        (&s.YY[0][0])[k] = YY[k];
      }
      for (int k = 0; k < MINIM_MAXM; k++) {
        s.rho[k] = rho[k]; s.sigma[k] = sig[k]; s.yy[k] = yy[k];
        s.sidx[k] = sidx[k]; s.yidx[k] = yidx[k];
      }
    }
    __syncthreads();
  }

  // End of an iteration: precision policy, convergence, iteration count.
  // Returns true when the minimisation has stopped (status set).
  __device__ bool post_iteration(bool exhausted) {
    const MinParams& mp = in.mp;
    const bool mixed = (mp.precision == 0);
    if (stage == 1) fp64_iters++;
      if (!isfinite(E) || !isfinite(gg)) {
        // FP32 overflows where FP64 does not (e.g. Lennard-Jones pairs at
        // very short range): evaluate the same point in FP64 before giving up
        if (stage == 0 && mixed) {
          switch_reason = 4;
          to_fp64();
          reeval();
        }
        if (!isfinite(E) || !isfinite(gg)) { status = ST_NAN; return true; }
      }
      const double r = rms();
      bool conv = r < mp.tol;
      if (mixed) {
        if (cool > 0) cool--;
        if (stage == 0) {
          // Leave the FP32 stage when FP32 has done what it can: converged in
          // FP32; the line search keeps failing to find an Armijo point (the
          // FP32 energy no longer resolves the decrease: failures accumulate
          // in a decaying score, or one failure within 1000x of tol); or the
          // RMS gradient has not improved by 0.1% for 100 iterations within
          // 100x of the tolerance (the FP32 gradient floor).
          if (r < 0.999 * best_rms) { best_rms = r; stall = 0; }
          else stall++;
          exhausted_run = exhausted_run * 7 / 8 + (exhausted ? 8 : 0);
          const int why = conv ? 1
                        : ((exhausted_run >= 20 || (exhausted && r < 1000.0 * mp.tol)) ? 2
                        : ((stall >= 100 && r < 100.0 * mp.tol && cool == 0) ? 3 : 0));
          if (why) {
            switch_reason = why;
            to_fp64();
            if (mp.method != 2) {
              reeval();
              conv = rms() < mp.tol;
            } else {
              conv = false;  // the next iteration's FP64 gradient decides
            }
            best_rms = rms();
            stall = 0;
            exhausted_run = 0;
          }
        } else {
          // An FP64 run that has moved far from convergence (FIRE restarts,
          // a basin change), or that has not improved its RMS gradient by 1%
          // in 2000 iterations (an orbit that will not converge), continues
          // in FP32; a stalled run may re-enter FP64 on a stall only after
          // 5000 more iterations, twice as many after each FP64 stage that
          // ended on a stall (up to 80000): an orbit that FP64 does not
          // settle either (FIRE with a large time step) spends a shrinking
          // share of its iterations in the costlier FP64 arithmetic.
          if (r < 0.99 * best_rms) { best_rms = r; stall = 0; }
          else stall++;
          const bool far = r > 1e4 * mp.tol && r > 100.0 * best_rms;
          if (far || stall >= 2000) {
            if (!far) {
              cool = 5000 << (fp64_fails < 4 ? fp64_fails : 4);
              fp64_fails++;
            }
            to_fp32();
            reeval();
            best_rms = rms();
            stall = 0;
            exhausted_run = 0;
            conv = false;
          }
        }
      }
    if (conv) { status = ST_CONVERGED; return true; }
    iter++;
    return false;
  }

  // Minimiser::minimise, resumable: runs at most `slice` iterations.
  __device__ void run(int slice) {
    const MinParams& mp = in.mp;
    if (status != ST_RUNNING) return;
    const bool mixed = (mp.precision == 0);
    if (!initd) {
      // Minimiser::init; the coordinates come from the resident FP64 copy
      initd = 1;
      {
        const double* xr = in.xres;
        float* X32 = in.X32[0];
        double* X64 = in.X64[0];
        for (int i = tm.tid(); i < n; i += tm.nthr()) {
          const double v = xr[i];
          X32[i] = (float)v;
          if (X64) X64[i] = v;
        }
        tm.sync();
        xi = 0;
        gi = 0;
      }
      if (mp.precision == 1) stage = 1;
      if (mixed && mp.method != 3) {
        // A start already near convergence stays in FP64: rounding it to
        // FP32 would only add noise that the FP64 stage must then relax
        // (a sheet started at its rest shape).  The FP64 gradient at the
        // exact start decides.
        stage = 1;
        switch_reason = 5;  // the decision's evaluation in FP64 arithmetic
        double py, yyv;
        grad_eval(0.0, nullptr, false, false, py, yyv);
        if (!(rms() < 100.0 * mp.tol)) {
          stage = 0;
          switch_reason = 0;
        }
      }
      if (mp.method == 0) {
        ii = 0;
        if (threadIdx.x == 0)
          for (int k = 0; k < MINIM_MAXM; k++) {
            rho[k] = 0; sig[k] = 0; yy[k] = 0; sidx[k] = k; yidx[k] = k;
          }
        pbuf = mp.m; ybuf = mp.m;
        pend = -1;
        __syncthreads();
      } else if (mp.method == 3) {
        // Anneal::init: the current state and its energy
        nsteps = 0;
        gg = 0.0;
        E = energy_at(0.0, nullptr);
      } else if (mp.method == 1) {
        for (int i = tm.tid(); i < n; i += tm.nthr()) in.V[i] = 0.f;
        tm.sync();
        a = 0.1; nsteps = 0;
        dtmax = mp.dt_max;
        if (dtmax == 0) {
          double py, yyv;
          grad_eval(0.0, nullptr, false, false, py, yyv);
          const double gn = gnorm_v;
          dtmax = (gn != 0) ? 0.1 / sqrt(gn) : 1.0;
        }
      }
      best_rms = 1e300;
      stall = 0;
      exhausted_run = 0;
      cool = 0;
      fp64_fails = 0;
    }
    // an iteration run outside this kernel (the stepped FP32 path) may hand
    // its end-of-iteration bookkeeping over to here
    bool done = false;
    if (resume) {
      resume = 0;
      done = post_iteration(resume_exhausted != 0);
    }
    for (int s = 0; s < slice && !done; s++) {
      if (iter > mp.max_iter) { status = ST_MAXITER; break; }
      bool exhausted = false;
      if (mp.method == 3) {
        anneal_iteration();
        if (!tm.ok()) { status = ST_TIMEOUT; break; }
        done = anneal_post();
        continue;
      }
      if (mp.method == 0) lbfgs_iteration(exhausted);
      else if (mp.method == 1) fire_iteration(exhausted);
      else gd_iteration(exhausted);
      if (!tm.ok()) { status = ST_TIMEOUT; break; }
      done = post_iteration(exhausted);
    }
    if (status != ST_RUNNING) {
      // hand the final coordinates back to the resident FP64 copy
      double* xr = in.xres;
      if (stage == 1) {
        const double* X = in.X64[xi];
        for (int i = tm.tid(); i < n; i += tm.nthr()) xr[i] = X[i];
      } else {
        const float* X = in.X32[xi];
        for (int i = tm.tid(); i < n; i += tm.nthr()) xr[i] = (double)X[i];
      }
      tm.sync();
    }
  }
};

}  // namespace mg
