/*
 * minim_gpu.h -- C ABI of the GB300-native minimisation engine.
 *
 * Plain C types only: pointers, sizes, ints and doubles.  Every function
 * returns an int status (MINIM_GPU_OK == 0) and records a message that
 * minim_gpu_last_error() returns.  Kernels never trap: per-instance failures
 * come back as a result status word.
 *
 * What each entry point replaces in the reference C++ library (paths are
 * relative to the minim source tree):
 *   minim_gpu_instance_create   State::State(pot, coords)       src/State.cpp:12-26
 *                               + Potential::init/initLocal     src/potentials/LjNd.cpp:12-26,
 *                                 src/potentials/PhaseField.cpp:137-235,
 *                                 src/potentials/PhaseFieldUnstructured.cpp:114-308,
 *                                 src/potentials/BarAndHinge.cpp:16-248
 *   minim_gpu_energy_gradient   State::energy/gradient/energyGradient
 *                                                               src/State.cpp:134-192
 *   minim_gpu_instance_set_coords / get_coords
 *                               State::coords(in) / coords()    src/State.cpp:282-288
 *   minim_gpu_instance_set_fixed
 *                               Potential::setConstraints(iFix) src/Potential.cpp:80-84
 *   minim_gpu_apply_constraints State::applyConstraints         src/State.cpp:321-323
 *   minim_gpu_minimise          Minimiser::minimise(state)      src/Minimiser.cpp:27-38
 *                               with Lbfgs/Fire/GradDescent/Anneal
 *                                                               src/minimisers/{Lbfgs,Fire,GradDescent,Anneal}.cpp
 *   minim_gpu_batch_*           (no counterpart: many States minimised together)
 *   minim_gpu_server_*          (no counterpart: continuous batching of requests)
 */
#ifndef MINIM_GPU_H
#define MINIM_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MINIM_GPU_ABI_VERSION 2

/* ---- call status ------------------------------------------------------ */
enum {
  MINIM_GPU_OK = 0,
  MINIM_GPU_ERR_INVALID = 1,   /* bad argument (reference: std::invalid_argument) */
  MINIM_GPU_ERR_RUNTIME = 2,   /* reference: std::runtime_error */
  MINIM_GPU_ERR_CUDA = 3,      /* a CUDA call failed */
  MINIM_GPU_ERR_OOM = 4,       /* device allocation failed */
  MINIM_GPU_ERR_NO_DEVICE = 5, /* no usable sm_103 device */
  MINIM_GPU_ERR_BUSY = 6       /* request not finished / not known */
};

/* ---- per-instance result status (device status word) ------------------- */
enum {
  MINIM_RES_CONVERGED = 0,  /* checkConvergence() became true */
  MINIM_RES_MAXITER = 1,    /* loop ran iter = 0..maxIter without converging */
  MINIM_RES_NAN = 2,        /* a non-finite energy or gradient was produced */
  MINIM_RES_TIMEOUT = 3,    /* a device wait gave up (bounded barrier) */
  MINIM_RES_CANCELLED = 4,  /* cancelled by the caller before completion */
  MINIM_RES_RUNNING = 5,    /* still in progress (serving) */
  MINIM_RES_REJECTED = 6    /* could not be admitted (does not fit in memory) */
};

/* ---- potential kinds ---------------------------------------------------- */
/* MINIM_GPU_PFU is PhaseFieldUnstructured (include/potentials/
 * PhaseFieldUnstructured.h), the element form of the same model: it takes a
 * minim_gpu_pf_params with that class's meaning (fixed volume as an energy
 * penalty, DENSITY_FIXED as the Nth fluid computed from the others). */
enum { MINIM_GPU_LJ = 0, MINIM_GPU_PF = 1, MINIM_GPU_BAH = 2, MINIM_GPU_PFU = 3 };

/* LjNd(nDim, sigma, epsilon): include/potentials/LjNd.h:22-24.  cutoff has
 * no counterpart in the reference, which sums every pair: 0 (the default)
 * keeps every pair; rc > 0 keeps the pairs with r^2 < rc^2, r^2 evaluated
 * in FP64 ((dx^2 + dy^2) + dz^2, one rounding per operation) of the
 * coordinates the evaluation sees, found through a device cell list. */
typedef struct {
  int ndim;         /* 2 or 3 */
  double sigma;     /* default 1 */
  double epsilon;   /* default 1 */
  double cutoff;    /* 0 = every pair (the reference) */
} minim_gpu_lj_params;

/* PhaseField (MODEL_BASIC): include/potentials/PhaseField.h:13-69.
 * Arrays may be NULL with count 0 to take the reference defaults. */
enum { MINIM_PF_DENSITY_HARD = 0, MINIM_PF_DENSITY_SOFT = 1,
       MINIM_PF_DENSITY_NONE = 2, MINIM_PF_DENSITY_FIXED = 3 };
typedef struct {
  int grid[3];                  /* setGridSize */
  int nfluid;                   /* setNFluid (default 1) */
  double resolution;            /* setResolution (default 1) */
  int n_interface_size;         /* 0 (default = resolution), or nfluid */
  const double* interface_size;
  int n_surface_tension;        /* 1, nfluid, or ngrid*nfluid (per node) */
  const double* surface_tension;
  int density_constraint;       /* MINIM_PF_DENSITY_* (default hard) */
  double density_const;         /* default 1 */
  int volume_fixed;             /* setVolumeFixed / setVolume */
  double vol_const;             /* default 0.01 (PF: unused; PFU: the volume penalty's strength) */
  const double* volume;         /* nfluid target volumes, or NULL = initial volumes */
  const double* pressure;       /* nfluid, or NULL (= 0) */
  const char* solid;            /* ngrid (0/1), or NULL (= no solid) */
  int n_contact_angle;          /* 0, ngrid, or ngrid*nfluid */
  const double* contact_angle;  /* degrees */
  const double* force;          /* nfluid*3, or NULL (setForce) */
  const char* fix_fluid;        /* nfluid, or NULL (setFixFluid) */
  const double* confinement;    /* nfluid, or NULL (setConfinement) */
} minim_gpu_pf_params;

/* BarAndHinge: include/potentials/BarAndHinge.h:10-60.
 * Topology comes either from a triangulation (setTriangulation) or from
 * explicit bond/hinge lists (setBondList/setHingeList, with stride >= 2 / 4;
 * entries after the first 2 / 4 are the adjacent-triangle vertices / bond
 * index used only by the thickness-based rigidities). */
typedef struct {
  int ntri; const int* tris;                     /* 3 per triangle */
  int nbond; const int* bonds; int bond_stride;  /* optional explicit bonds */
  int nhinge; const int* hinges; int hinge_stride;
  double modulus;                                /* default 1 */
  double poisson_ratio;                          /* default 0.3 */
  int n_thickness; const double* thickness;      /* 0, 1 or nvert */
  int n_kbond; const double* kbond;              /* 0, 1 or nbond */
  int n_khinge; const double* khinge;            /* 0, 1 or nhinge */
  int n_length0; const double* length0;          /* 0 (from coords), 1 or nbond */
  int n_theta0; const double* theta0;            /* 0 (from coords), 1 or nhinge */
  int n_force; const double* force;              /* 0, 3 or 3*nvert */
  int wall_on, wall_adhesion;
  double wall_epsilon;                           /* default 1e-12 */
  double wall_sigma;                             /* default 1e-5 */
} minim_gpu_bah_params;

/* ---- minimisers ---------------------------------------------------------- */
enum { MINIM_LBFGS = 0, MINIM_FIRE = 1, MINIM_GD = 2, MINIM_ANNEAL = 3 };
enum { MINIM_LS_BACKTRACKING = 0, MINIM_LS_NONE = 1 };
/* Precision of the coordinates while minimising.  MIXED runs FP32
 * coordinates/gradients with FP64 reductions, then switches to FP64
 * coordinates for the final polish; FP64 runs FP64 coordinates throughout;
 * FP32 never switches. */
enum { MINIM_PREC_MIXED = 0, MINIM_PREC_FP64 = 1, MINIM_PREC_FP32 = 2 };

typedef struct {
  int method;        /* MINIM_LBFGS / MINIM_FIRE / MINIM_GD */
  int linesearch;    /* MINIM_LS_*; reference default: backtracking, except Fire(dtMax) */
  int max_iter;      /* Minimiser::maxIter (default 100000) */
  double tol;        /* State::convergence; < 0 takes the potential's default */
  int m;             /* Lbfgs::setM (default 5) */
  double max_step;   /* Lbfgs::setMaxStep (default 0 = off) */
  double init_step;  /* Lbfgs::setInitStep (default 1) */
  double dt_max;     /* Fire dtMax (0 = estimate 0.1/sqrt|g| at start) */
  double alpha;      /* GradDescent::setAlpha (default 0.1) */
  int precision;     /* MINIM_PREC_* (Anneal always runs FP64 coordinates) */
  /* Anneal(tempInit, displacement), include/minimisers/Anneal.h:9-44.  Each
   * iteration moves every coordinate by displacement * U(-1, 1) from the
   * last accepted state and accepts by the Metropolis rule at
   * T = temp_init / (1 + cooling_rate * iter), or T = temp_schedule[iter]
   * (clamped to the last entry) when a schedule is given -- a
   * setCoolingSchedule function tabulated by the caller.  The random numbers
   * are a counter-based hash of (seed, iter, index): the same seed gives the
   * same run (the reference seeds rand() with time(0) + rank). */
  double temp_init;         /* default 1 */
  double displacement;      /* default 0.1 */
  double cooling_rate;      /* setCoolingRate (default 1) */
  int max_rejections;       /* setMaxRejections (default 0: runs max_iter + 1 iterations) */
  int n_temp_schedule;      /* 0, or entries of temp_schedule */
  const double* temp_schedule;  /* read during the call that uses it (batch: batch_add copies it) */
  uint64_t seed;
} minim_gpu_minimiser_params;

typedef struct {
  int status;           /* MINIM_RES_* */
  int iter;             /* Minimiser::iter after minimise() (reference meaning) */
  int fp64_iters;       /* iterations run with FP64 coordinates */
  int evals;            /* potential evaluations (energy-only and energy+gradient) */
  double energy;        /* energy at the returned coordinates */
  double rms;           /* sqrt(g.g/ndof) at the returned coordinates (Anneal: 0, no gradient) */
  double dt_max;        /* Fire: the dtMax used (estimated when 0 was passed) */
  double latency_ms;    /* serving: submit -> completion wall time */
  double run_ms;        /* batches and serving: device time from the first slice's start to the
                           last slice's end of this instance (0 for single-instance calls) */
} minim_gpu_result;

/* Measurement of the last minimise / batch call, taken by the library on the
 * stream it launches on: CUDA events around every kernel launch. */
typedef struct {
  double kernel_ms;     /* summed device time of the minimiser kernel launches */
  double wall_ms;       /* host wall time of the call */
  int64_t launches;     /* minimiser kernel launches in the call */
  double abytes;        /* algorithmic HBM bytes of the work done (all instances) */
  double pairs32;       /* Lennard-Jones pair interactions in FP32 */
  double pairs64;       /* ... and in FP64 */
  int64_t iterations;   /* minimiser iterations (all instances) */
  int64_t fp64_iterations; /* ... of which with FP64 coordinates */
  /* instances whose FP64 stage started because: [1] FP32 converged, [2] the
   * line search failed twice in a row, [3] the gradient stalled near tol */
  int64_t switches[4];
  /* device time in gradient evaluations, line-search trial evaluations and
   * L-BFGS direction passes (single-instance calls; summed over instances
   * for batches) */
  double phase_ms[3];
  /* batch and server calls: device time the autotuner spent timing
   * candidate launch shapes before the run (not in kernel_ms) */
  double tune_ms;
} minim_gpu_run_stats;

typedef struct minim_gpu_instance_s* minim_gpu_handle;
typedef struct minim_gpu_batch_s* minim_gpu_batch;
typedef struct minim_gpu_server_s* minim_gpu_server;

/* ---- library ------------------------------------------------------------ */
int minim_gpu_abi_version(void);
int minim_gpu_last_error(char* buf, size_t len);
/* Fills defaults equal to the reference's constructors and setters. */
void minim_gpu_default_minimiser(int method, minim_gpu_minimiser_params* out);
void minim_gpu_default_pf(minim_gpu_pf_params* out);
void minim_gpu_default_bah(minim_gpu_bah_params* out);
/* Number of potential/minimiser kernel launches issued by this process. */
int64_t minim_gpu_launch_count(void);
/* Statistics of the most recent minimise / batch_run call. */
int minim_gpu_last_run_stats(minim_gpu_run_stats* out);

/* ---- single instances ------------------------------------------------------ */
/* Copies the host arrays into device-owned buffers; the caller keeps its own.
 * params points at minim_gpu_{lj,pf,bah}_params according to kind. */
int minim_gpu_instance_create(int kind, const void* params, const double* x0,
                              size_t ndof, minim_gpu_handle* out);
int minim_gpu_instance_destroy(minim_gpu_handle h);
int minim_gpu_instance_ndof(minim_gpu_handle h, size_t* ndof);
/* The potential's own default convergence (PhaseField: 1e-8*sigma*res^2). */
int minim_gpu_instance_default_tol(minim_gpu_handle h, double* tol);
int minim_gpu_instance_set_coords(minim_gpu_handle h, const double* x);
int minim_gpu_instance_get_coords(minim_gpu_handle h, double* x);
/* Fixed degrees of freedom: gradient (and step) components forced to 0. */
int minim_gpu_instance_set_fixed(minim_gpu_handle h, const int* idof, size_t n);
/* Energy and constrained gradient at x (x == NULL: the resident coordinates).
 * e and g may each be NULL, as in the reference. */
int minim_gpu_energy_gradient(minim_gpu_handle h, const double* x, double* e, double* g);
/* In-place State::applyConstraints on a host vector of length ndof. */
int minim_gpu_apply_constraints(minim_gpu_handle h, double* v);
/* Device-resident minimisation of one instance using the whole GPU; on
 * return the instance holds the minimised coordinates. */
int minim_gpu_minimise(minim_gpu_handle h, const minim_gpu_minimiser_params* mp,
                       minim_gpu_result* res);

/* ---- batches: many instances in one persistent launch --------------------- */
int minim_gpu_batch_create(minim_gpu_batch* out);
int minim_gpu_batch_add(minim_gpu_batch b, minim_gpu_handle h,
                        const minim_gpu_minimiser_params* mp);
/* threads_per_cta > 0 runs every instance on one CTA of that many threads;
 * 0 = autotuned: each instance's launch shape -- threads per CTA and CTAs per
 * instance (one CTA, or a thread-block cluster of 2, 4 or 8 CTAs on as many
 * SMs for large instances) -- depends only on its own potential kind, size
 * bucket, method and precision (never on the rest of the batch), chosen the
 * first time that key is seen in the process by timing every candidate on a
 * short slice of copies of the batch's instances of that key
 * (MINIM_GPU_TUNE=0: a fixed size rule instead; MINIM_GPU_TUNE_CACHE=file
 * keeps the choices across processes).  results has one entry per added
 * instance. */
int minim_gpu_batch_run(minim_gpu_batch b, int threads_per_cta, minim_gpu_result* results);
/* As minim_gpu_batch_run with one launch shape for every instance:
 * threads_per_cta (32 .. 512, a multiple of 32; Lennard-Jones at most 256)
 * and ctas CTAs per instance (1 .. 8; more than 1 runs each instance on a
 * thread-block cluster of that many CTAs). */
int minim_gpu_batch_run_shape(minim_gpu_batch b, int threads_per_cta, int ctas, minim_gpu_result* results);
/* The autotuner's choices so far (no counterpart in the reference): up to
 * cap rows of 8 ints {potential kind (MINIM_GPU_*), size bucket, method,
 * precision, threads per CTA, CTAs per instance, measured (1) or read from
 * the cache file (0), times recorded}, and per row 8 doubles: the measured
 * slice time of each candidate in ms -- one-CTA candidates on the batch's
 * sample of the key, cluster candidates on its largest instance alone,
 * followed (when there are cluster candidates) by the chosen one-CTA
 * shape's time on that instance (ms may be NULL).  *n receives the number
 * of rows. */
int minim_gpu_tune_table(int cap, int* rows, double* ms, int* n);
int minim_gpu_batch_destroy(minim_gpu_batch b);

/* ---- serving: continuous batching ------------------------------------------ */
typedef struct {
  size_t max_bytes;     /* device memory budget for resident instances (0 = 50% free) */
  int max_slots;        /* maximum concurrently resident instances (0 = 4096) */
  int slice_iters;      /* iterations each resident instance runs per step (0 = 64) */
  int threads_per_cta;  /* 0 = autotuned */
} minim_gpu_server_config;

int minim_gpu_server_create(const minim_gpu_server_config* cfg, minim_gpu_server* out);
/* Queue a request; it is admitted once slots and memory allow. */
int minim_gpu_server_submit(minim_gpu_server s, int kind, const void* params,
                            const double* x0, size_t ndof,
                            const minim_gpu_minimiser_params* mp, uint64_t* request_id);
/* One scheduling step: admit queued requests, run one slice on every
 * resident instance, retire the finished ones.  Reports what is resident
 * and what is still queued. */
int minim_gpu_server_step(minim_gpu_server s, int* n_resident, int* n_queued);
/* Completed requests since the last call (ids and results), at most max. */
int minim_gpu_server_poll(minim_gpu_server s, uint64_t* ids, minim_gpu_result* res,
                          int max, int* n_done);
/* Copy out a completed request's coordinates and release it. */
int minim_gpu_server_take(minim_gpu_server s, uint64_t id, double* x, size_t ndof);
int minim_gpu_server_cancel(minim_gpu_server s, uint64_t id);
int minim_gpu_server_destroy(minim_gpu_server s);

/* ---- set-up introspection (host only; no GPU needed) ------------------------
 * These expose the host-side set-up so it can be compared with the reference
 * library: BarAndHinge elements in the order of BarAndHinge::init
 * (src/potentials/BarAndHinge.cpp:16-67; topology of computeBondList /
 * computeHingeList, lines 70-147), the greedy element colouring used by the
 * gradient scatter, and PhaseField::init/initLocal products (kappa, kappaP,
 * nodeVol, surfaceArea; src/potentials/PhaseField.cpp:78-235). */
int minim_gpu_bah_elements(const minim_gpu_bah_params* q, const double* x0, size_t ndof, int cap,
                           int* nbar, int* bars, double* bar_par, int* nhinge, int* hinges,
                           double* hinge_par);
int minim_gpu_bah_colouring(const minim_gpu_bah_params* q, const double* x0, size_t ndof,
                            int* nbar_colors, int* nhinge_colors, int* valid);
/* The BarAndHinge elements an instance evaluates, in its colour order (no
 * counterpart in the reference; for checking the set-up, which runs on the
 * device for a triangulation unless MINIM_GPU_BAH_DEVICE_SETUP=0): bars (2
 * per bar) with {k, l0}, hinges (4 per hinge) with {k, theta0}, at most cap
 * of each; colour offsets (ncolors + 1 entries, at most 65); on_device = 1
 * when the device built them.  Elements whose coordinates are all fixed are
 * not included. */
int minim_gpu_instance_bah_arrays(minim_gpu_handle h, int cap, int* nbar, int* bars, double* bar_par,
                                  int* nbar_colors, int* bar_off, int* nhinge, int* hinges,
                                  double* hinge_par, int* nhinge_colors, int* hinge_off, int* on_device);
/* kind: MINIM_GPU_PF or MINIM_GPU_PFU.  kernel_variant: 1 = general
 * PhaseField kernel, 3 = binary kernel without optional terms. */
int minim_gpu_pf_setup(int kind, const minim_gpu_pf_params* q, const double* x0, size_t ndof, double* kappa,
                       double* kappaP, int* nk, double* node_vol, double* surface_area,
                       int* kernel_variant);

/* ---- kernel checks (no counterpart in the reference) ----------------------
 * One energy (and gradient) evaluation by the potential kernels that a
 * minimisation runs in a given stage, at the point x + t p, so that those
 * kernels can be checked one evaluation at a time against an FP64
 * evaluation of the same point (the reference's State::energyGradient,
 * src/State.cpp:134-192, is FP64 throughout).  path:
 *   MINIM_EVAL_FP32_GRID   FP32 coordinates, the single-instance kernels (whole GPU)
 *   MINIM_EVAL_FP32_CTA    FP32 coordinates, the batch kernels (one CTA per instance)
 *   MINIM_EVAL_FP64S_GRID  FP64 coordinates with the FP64 stage's arithmetic
 *                          (double-float where the minimiser uses it), whole GPU
 *   MINIM_EVAL_FP64S_CTA   the same on one CTA
 *   MINIM_EVAL_LINES       the line stencil of the stepped L-BFGS graph (binary
 *                          PhaseField without optional terms, nz % 4 == 0): two
 *                          trials in one pass, at t and at t/2
 *   MINIM_EVAL_LINES_TMA   the same pass with its lines brought into shared
 *                          memory as tensor-map tiles (nz % 32 == 0, nz <= 256,
 *                          ny % 4 == 0, ny >= 8); g is required
 * x (ndof) is rounded to FP32 on the FP32 paths; p (ndof, or NULL for the
 * point x itself) is rounded to FP32, as the minimiser's directions are.
 * The FP32 paths form the point as x32 + fl(t32 * p32) (the line stencil as
 * one fused multiply-add), the FP64 paths as x + t * p.  g receives the
 * gradient as the minimiser stores it (FP32 values, constraints applied);
 * g == NULL runs the energy-only evaluation (the line-search trial kernels).
 * For the two line-stencil paths, e and g (if given) hold two evaluations, at t then at
 * t/2 (2 and 2 * ndof entries), and xt (optional, 2 * ndof) receives the two
 * points as the stencil formed them; on the other paths xt must be NULL. */
enum { MINIM_EVAL_FP32_GRID = 0, MINIM_EVAL_FP32_CTA = 1, MINIM_EVAL_FP64S_GRID = 2,
       MINIM_EVAL_FP64S_CTA = 3, MINIM_EVAL_LINES = 4, MINIM_EVAL_LINES_TMA = 5 };
int minim_gpu_eval_kernel(minim_gpu_handle h, int path, const double* x, const double* p, double t,
                          double* e, double* g, double* xt);

/* The pairs i < j that the FP32 stage of a Lennard-Jones instance with a
 * cutoff evaluates at x (rounded to FP32), from the device cell list (no
 * counterpart in the reference): up to cap pairs (2 ints each) sorted by
 * (i, j) into pairs, the total into *npairs.  For checking the pair set
 * against a CPU enumeration with the same FP64 r^2 of the same FP32 values. */
int minim_gpu_lj_cutoff_pairs(minim_gpu_handle h, const double* x, int cap, int* pairs, int* npairs);

/* Failure detection check (no counterpart in the reference): one block
 * runs the device barrier's bounded wait on an arrival count that nothing
 * reaches, with its limit set to limit_ms (1 .. 60000).  The wait gives up,
 * records the error the host reads, and the kernel returns: *timed_out = 1,
 * *elapsed_ms = the kernel's device time.  The same bound (5 s) protects
 * every wait of the single-instance kernels, whose minimisations then end
 * with status MINIM_RES_TIMEOUT. */
int minim_gpu_wait_probe(int limit_ms, int* timed_out, double* elapsed_ms);

/* ---- allocation-free minimisation (no counterpart in the reference) ------
 * Minimises one Lennard-Jones cluster (LjNd energy, the given minimiser) in
 * one CTA without allocating any memory: for callers that cannot call the
 * device allocator -- code embedded in a runtime whose caching allocator
 * already holds the GPU's memory, or a loop that must stay out of the
 * driver's allocator.  x_dev (device memory, ndof doubles) holds the start
 * and receives the minimum; the workspace is a fixed 1 MiB device array
 * inside this library, at most 3072 degrees of freedom (1024 particles in
 * 3-D; larger calls return MINIM_GPU_ERR_INVALID).  Work is queued on
 * `stream` (a cudaStream_t, NULL = legacy default stream) and the call
 * returns after synchronising that stream.  The first call on a device (with
 * that device current) looks up the array's device address.  All calls
 * share the one array: calls that overlap on
 * the GPU race and must be serialised by the caller.  The tolerance
 * mp->tol < 0 means 1e-6.  Results equal minim_gpu_batch_run with 256
 * threads per CTA. */
int minim_gpu_lj_minimise_noalloc(const minim_gpu_lj_params* p, double* x_dev, size_t ndof,
                                  const minim_gpu_minimiser_params* mp, minim_gpu_result* res,
                                  void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MINIM_GPU_H */
