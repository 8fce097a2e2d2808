// engine.h -- data layout shared by the host runtime and the device kernels.
//
// Everything an instance needs on the device lives in one InstDesc (plain
// data, device pointers): the potential's parameters, the minimiser's
// parameters, the vector buffers and a pointer to its MinScalars (the
// minimiser state that persists between launches, so a minimisation can be
// run in slices and resumed).
#pragma once
#include <stddef.h>
#include <stdint.h>
#include <vector_types.h>

#define MINIM_MAXM 16
#define MINIM_MAXF 4
#define MINIM_WIDE 64  // values reduced together in one wide reduction (row width of partial sums)

namespace mg {

// ---- potentials -------------------------------------------------------------
struct PotLJ {
  int ndim;        // 2 or 3
  int np;          // particles
  double s6;       // sigma^6
  double eps;      // epsilon
  // cutoff (no counterpart in the reference, which sums every pair): pairs
  // with r^2 >= rc2 are left out, found through a hashed cell list
  double rc2;      // 0: every pair
  double inv_cs;   // 1 / cell size (the cell size is rc * (1 + 1e-3))
  int hbits;       // log2 of the hash table's buckets
  int* cells;      // scratch: lj_cell_ints(np, hbits) ints
};
#ifdef __CUDACC__
#define MG_HD __host__ __device__
#else
#define MG_HD
#endif
// Lennard-Jones shared memory of the one-CTA paths (positions and eight
// warps' force accumulators of the dealt FP32 evaluation, the symmetric
// tiles of the double-float and FP32 evaluations)
MG_HD inline size_t lj_dealt_bytes(int np, int nwarps) {
  const size_t nt = (size_t)(np + 31) >> 5;
  return 32 * nt * (4 * sizeof(float)) + 32 * nt * (3 * sizeof(float)) * (size_t)nwarps;
}
// The one-CTA Lennard-Jones paths are chosen against this fixed shared-
// memory budget (not the memory a launch gives), so that an instance's path
// -- and its result -- does not depend on the other instances of its launch;
// each launch then gives the bytes its instances' paths use
// (lj_smem_bytes).
constexpr size_t kLjSmemBudget = 48 * 1024;
MG_HD inline size_t lj_sym_bytes(int np, size_t elem) {
  const size_t nt = (size_t)(np + 31) >> 5, ntp = nt + (nt & 1);
  return 32 * ntp * 7 * elem;
}
// shared memory of a one-CTA launch for a cluster of np particles with the
// given threads: the dealt FP32 gradient, the FP64-stage (double-float) and
// FP32 symmetric tiles when they fit the budget, and at least 128 tile
// entries for the generic pair loop (whose result does not depend on its
// tile length, a multiple of 4)
MG_HD inline size_t lj_smem_bytes(int np, int threads) {
  size_t need = 128 * 32;
  const size_t dealt = lj_dealt_bytes(np, threads >> 5);
  if (dealt <= kLjSmemBudget && need < dealt) need = dealt;
  const size_t sd = lj_sym_bytes(np, 8), sf = lj_sym_bytes(np, 4);
  if (sd <= kLjSmemBudget) {
    if (need < sd) need = sd;
  } else if (sf <= kLjSmemBudget && need < sf) {
    need = sf;
  }
  return (need + 127) & ~(size_t)127;
}

// ints of the cell-list scratch: bucket starts (H + 1), cursors (H), the
// particles in bucket order (N), each particle's bucket (N), one int of
// padding, and each particle's 64-bit cell key (2 N)
inline size_t lj_cell_ints(int np, int hbits) { return 2 * ((size_t)1 << hbits) + 4 * (size_t)np + 2; }

enum PfFlags : unsigned {
  PF_SOLID = 1u << 0,      // aux[] present: node types and solid-neighbour masks
  PF_CONTACT = 1u << 1,    // wet[] present (binary wetting term)
  PF_PRESSURE = 1u << 2,
  PF_SOFT = 1u << 3,       // soft density penalty
  PF_HARD = 1u << 4,       // hard density projection
  PF_VOLUME = 1u << 5,     // fixed-volume projection
  PF_FORCE = 1u << 6,
  PF_CONFINE = 1u << 7,
  PF_NODE_KAPPA = 1u << 8, // per-node kappa / kappaP arrays
  PF_FIXFLUID = 1u << 9,
  // PhaseFieldUnstructured (element form): pressure on fixed fluids too, the
  // soft density over the first three fluids, no node terms on solid nodes
  PF_UNSTR = 1u << 10,
  PF_UVOL = 1u << 11,      // fixed volume as an energy penalty (vol_target, vol_coef)
  PF_NALL = 1u << 12,      // DENSITY_FIXED: the last fluid is 1 minus the others
};

struct PotPF {
  int n[3];
  int nfluid;
  int ngrid;
  unsigned flags;
  // per node: bits 0-3 = node type + 1 (0 = solid, 1 = bulk, 2..8 = surface
  // types 1..7); bits 4-9 = solid flags of the face neighbours in the order
  // x-, x+, y-, y+, z-, z+.  NULL when there is no solid.
  const uint16_t* aux;
  double vol_of_type[9];    // nodeVol by (type + 1), includes res^3
  double res, res2;
  double kappa[MINIM_MAXF], kappaP[MINIM_MAXF];
  const double* kappa_node;   // ngrid*nfluid (PF_NODE_KAPPA)
  const double* kappaP_node;
  const double* wet;          // per node: wettingParam * surfaceArea (PF_CONTACT)
  double pressure[MINIM_MAXF];
  unsigned fix_mask;          // fixFluid bits
  int nvar;                   // variable (non-fixed) fluids
  double soft_coef;           // densityConst * sigmaMean * res^2
  double confine_coef[MINIM_MAXF];
  const double* ff_init;      // ndof (PF_CONFINE)
  double fmag[MINIM_MAXF];
  double fnorm[MINIM_MAXF][3];
  double total_volume2;       // sum nodeVol^2 (PF_VOLUME)
  double vol_target[MINIM_MAXF];  // PF_UVOL: target volumes
  double vol_coef;            // PF_UVOL: volConst * sigmaMean / res^4
  int pf_dist;                // L2 prefetch distance of the stencil sweep (0 = none)
};

struct PotBAH {
  int nvert, nbar, nhinge;
  const int2* bars;           // sorted by colour
  const double2* bar_par;     // {k, l0}
  const int4* hinges;         // sorted by colour
  const double2* hinge_par;   // {k, theta0}
  int nbar_colors, nhinge_colors;
  const int* bar_color_off;   // nbar_colors + 1 offsets
  const int* hinge_color_off;
  const unsigned char* node_el;  // per vertex: force/wall elements present
  int nforce;                 // 0, 3 or 3*nvert
  const double* force;
  int wall_on, wall_adh;
  double wall_eps, wall_sig;
};

// ---- minimiser ------------------------------------------------------------------
struct MinParams {
  int method;       // 0 lbfgs, 1 fire, 2 gd, 3 anneal
  int linesearch;   // 0 backtracking, 1 none
  int max_iter;
  int m;
  int precision;    // 0 mixed, 1 fp64, 2 fp32
  double tol;
  double max_step, init_step, dt_max, alpha;
  // Anneal
  double temp_init, displacement, cooling_rate;
  int max_rej;
  int ntsched;               // entries of tsched (0: temp_init / (1 + cooling_rate * iter))
  const double* tsched;      // device copy of the tabulated schedule
  unsigned long long seed;
};

enum RunStatus { ST_CONVERGED = 0, ST_MAXITER = 1, ST_NAN = 2, ST_TIMEOUT = 3,
                 ST_CANCELLED = 4, ST_RUNNING = 5 };

struct MinScalars {
  int status;
  int initialised;
  int iter;          // the reference's loop counter
  int ii;            // Lbfgs::_i
  int stage;         // 0: FP32 coordinates, 1: FP64 coordinates
  int xi, gi;        // which of X[2] / G[2] is current
  int evals;
  int fp64_iters;
  int stall;         // iterations since the best rms improved (stage 0)
  int nsteps;        // Fire::_nSteps; Anneal::_sinceAccepted
  int pbuf, ybuf;    // spare history buffers (direction / new y)
  int ybuf2;         // second spare y slot (stepped path, two trials per pass), or -1
  int exhausted_run; // consecutive line searches that found no Armijo point
  int switch_reason; // why the FP64 stage started: 1 converged in FP32,
                     // 2 line search exhausted twice, 3 stalled near tol
  int sidx[MINIM_MAXM], yidx[MINIM_MAXM];  // ring slot -> buffer
  double E;          // energy at the current coordinates
  double gg;         // g.g at the current coordinates
  double best_rms;
  double dt, a, dtmax, gnorm;  // Fire
  double rho[MINIM_MAXM], sigma[MINIM_MAXM], yy[MINIM_MAXM];
  // compact L-BFGS: SY[a][b] = s_a.y_b (slot indices; the part with a older
  // than or equal to b is used), YY[a][b] = y_a.y_b; column `pend` (the
  // newest pair) is filled by the next direction's first pass
  double SY[MINIM_MAXM][MINIM_MAXM], YY[MINIM_MAXM][MINIM_MAXM];
  int pend;
  int cool;          // iterations before a stalled run may re-enter FP64
  int fp64_fails;    // FP64 stages left on a stall (each doubles the next wait, up to 16x)
  int spare_;
  // set by the stepped FP32 path when it hands an iteration's end-of-
  // iteration bookkeeping (precision switch, convergence) to the kernel
  int resume, resume_exhausted;
  // work counters for the roofline: algorithmic HBM bytes of every vector
  // pass and evaluation, and Lennard-Jones pair interactions per precision
  double abytes, pairs32, pairs64;
  // device time (ns, block 0) in gradient evaluations, line-search trial
  // evaluations and L-BFGS direction passes
  double tphase[3];
  // batch kernels: %globaltimer when a CTA first took the instance and when
  // one last stored it (ns)
  unsigned long long t_first, t_last;
};

// K_PF1 is the kernel variant for a binary PhaseField with none of the
// optional terms except pressure (chosen by the host; same results).
enum Kind { K_LJ = 0, K_PF = 1, K_BAH = 2, K_PF1 = 3 };

struct InstDesc {
  int kind;
  int ndof;
  PotLJ lj;
  PotPF pf;
  PotBAH bah;
  MinParams mp;
  const unsigned char* fixed;  // per-dof fixed flags, or NULL
  float* X32[2];
  double* X64[2];
  float* G[2];
  // stepped path, two trials per pass: the second trial's point and gradient
  // (exchanged with X32[1 - xi] / G[1 - gi] when it is accepted), or NULL
  float* X32s;
  float* Gs;
  int hstride;     // floats between history buffers (ndof rounded up to 64)
  float* Sb;       // (m + 1) * hstride: ring of directions (s = sigma * S)
  float* Yb;       // (m + 1) * hstride
  float* V;        // Fire velocity
  double* GA;      // FP64 gradient accumulator (BarAndHinge scatter), or NULL
  double* xres;    // resident FP64 coordinates: read at start, written at the end
  MinScalars* st;
  int stage_bytes; // grid launches: bytes of each shared staging buffer (0 = none)
  int pf_dist;     // vector passes: L2 prefetch distance in sweep steps (0 = none)
};

// Bounded software grid barrier state (one per cooperative launch).
struct GridSyncState {
  unsigned int count;
  unsigned int gen;
  int err;                // set when a barrier wait gave up
  unsigned int limit_ms;  // bound of every wait (0: 5 s)
};

// ---- kernel entry points (engine.cu) ---------------------------------------------
enum Op { OP_MINIMISE = 0, OP_EVAL = 1, OP_CONSTRAIN = 2, OP_EVAL_STAGE = 3, OP_LJ_PAIRS = 4 };

struct EvalIO {      // OP_EVAL / OP_CONSTRAIN on one instance, FP64 in/out
  const double* x;   // coordinates (device), ndof
  double* g;         // gradient out (device) or NULL
  double* e;         // energy out (device, 1 double) or NULL
  double* v;         // OP_CONSTRAIN: vector constrained in place
  // OP_EVAL_STAGE (and the one-CTA evaluation kernel): one evaluation by a
  // minimiser stage's own potential kernels at x + t p, the gradient stored
  // as the minimiser stores it (FP32, constrained) into g32, or an
  // energy-only evaluation when g32 is NULL
  int stage;         // 0: FP32 coordinates x32; 1: FP64 coordinates x (FP64-stage arithmetic)
  float t32;
  double t64;
  const float* x32;
  const float* p;    // direction (FP32 in both stages), or NULL
  float* g32;
  // OP_LJ_PAIRS: the pairs i < j within the cutoff at x32 (at most cap)
  int2* pairs;
  int* npairs;
  int cap;
};

}  // namespace mg

extern "C" {
// Launchers, one set per potential kind (engine_{lj,pf,bah}.cu).  Each
// returns a cudaError_t value.
#define MG_DECLARE_LAUNCHERS(NAME)                                                              \
  int mg_launch_batch_##NAME(const mg::InstDesc* d_insts, int ninst, int* d_counter,             \
                             int slice_iters, int threads, int blocks, size_t smem, void* stream); \
  int mg_launch_grid_##NAME(const mg::InstDesc* d_inst, int op, const mg::EvalIO* d_io,           \
                            int slice_iters, mg::GridSyncState* d_bar, double* d_partials,       \
                            int threads, int blocks, size_t smem, void* stream);                 \
  int mg_occupancy_##NAME(int grid, int threads, size_t smem, int* blocks_per_sm);              \
  int mg_launch_cta_eval_##NAME(const mg::InstDesc* d_inst, const mg::EvalIO* d_io, int threads,  \
                                size_t smem, void* stream);                                    \
  int mg_launch_cbatch_##NAME(const mg::InstDesc* d_insts, int ninst, int* d_counter, int slice_iters, \
                              int threads, int csize, int clusters, size_t smem, void* stream);   \
  int mg_cluster_occupancy_##NAME(int threads, int csize, size_t smem, int* clusters);
MG_DECLARE_LAUNCHERS(lj)
MG_DECLARE_LAUNCHERS(pf)
MG_DECLARE_LAUNCHERS(bah)
MG_DECLARE_LAUNCHERS(pf1)
// engine_misc.cu: FP64 <-> FP32 vector conversion on a stream
int mg_convert(const void* src, void* dst, size_t n, int to_float, void* stream);
// engine_misc.cu: one block waits, with the grid barrier's bounded wait, for
// an arrival count that nothing reaches; *bar must be zeroed with its
// limit_ms set.  The kernel returns when the wait gives up (bar->err = 1).
int mg_wait_probe(mg::GridSyncState* bar, void* stream);
// stepped.cu: up to `slice` FP32 L-BFGS iterations (history m) of a binary
// PhaseField instance as one launch of the graph of its shape (cached per
// process); dual: the workspace has the spare buffers for two trials per
// pass; hd: the host's copy of the descriptor (buffer addresses for the
// trial pass's tensor maps).  Returns a cudaError_t.
int mg_stepped_pf1_run(mg::InstDesc* d, const mg::InstDesc* hd, mg::MinScalars* st, int m, const int* grid,
                       int nsm, int slice, int dual, void* stream, double* kernels);
void mg_stepped_free_all();
// stepped.cu: one line-stencil pass outside the graph (kernel checks)
int mg_stepped_lines_probe(const mg::InstDesc* d, const int* grid, int mode, const float* X, const float* P,
                           const float* Go, float t, float* Xa, float* Ga, float* Ya, float* Xb, float* Gb,
                           float* Yb, double* part, int max_rows, int nsm, int* rows, void* stream);
// stepped.cu: the same two-trial pass through tensor-map tiles
int mg_stepped_lines_tma_probe(const mg::InstDesc* d, const int* grid, const float* X, const float* P,
                               const float* Go, float t, float* Xa, float* Ga, float* Ya, float* Xb, float* Gb,
                               float* Yb, double* part, int max_rows, int nsm, int* rows, void* stream);
}
