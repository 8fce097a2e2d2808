// capi.cpp -- host runtime behind include/minim_gpu.h.
//
// One process, one GPU (the current CUDA device, which must be sm_103).
// Device memory comes from the stream-ordered pool (cudaMallocAsync with a
// release threshold that keeps freed blocks cached), so admitting and
// retiring thousands of instances does not hit the driver allocator.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "engine.h"
#include "minim_gpu.h"
#include "setup.h"
#include "topology.h"

using namespace mg;

namespace {

thread_local std::string g_err;
std::atomic<int64_t> g_launches{0};
minim_gpu_run_stats g_stats{};
std::recursive_mutex g_mu;

struct ApiError {
  int code;
  std::string msg;
};

#define CK(call)                                                                              \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess)                                                                    \
      throw ApiError{e_ == cudaErrorMemoryAllocation ? MINIM_GPU_ERR_OOM : MINIM_GPU_ERR_CUDA, \
                     std::string(#call) + ": " + cudaGetErrorString(e_)};                     \
  } while (0)

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

// ---- device ------------------------------------------------------------------
struct Dev {
  int ok = 0;
  int id = 0;
  int nsm = 0;
  std::string why;
  cudaStream_t s = nullptr;             // runtime stream (allocations, copies)
  cudaStream_t ks[8] = {};              // batch launch streams (one per launch group)
};

Dev& dev() {
  static Dev d;
  static bool inited = false;
  if (inited) return d;
  inited = true;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    d.why = "no CUDA device";
    return d;
  }
  cudaGetDevice(&d.id);
  cudaDeviceProp p;
  cudaGetDeviceProperties(&p, d.id);
  if (!(p.major == 10 && p.minor == 3)) {
    d.why = std::string("the kernels are built for sm_103a; device is sm_") + std::to_string(p.major) +
            std::to_string(p.minor);
    return d;
  }
  d.nsm = p.multiProcessorCount;
  cudaStreamCreateWithFlags(&d.s, cudaStreamNonBlocking);
  for (auto& k : d.ks) cudaStreamCreateWithFlags(&k, cudaStreamNonBlocking);
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, d.id) == cudaSuccess) {
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  d.ok = 1;
  return d;
}

Dev& need_dev() {
  Dev& d = dev();
  if (!d.ok) throw ApiError{MINIM_GPU_ERR_NO_DEVICE, "minim_gpu: " + d.why};
  return d;
}

void* dalloc(size_t bytes) {
  if (bytes == 0) bytes = 256;
  void* p = nullptr;
  CK(cudaMallocAsync(&p, bytes, need_dev().s));
  return p;
}
void dfree(void* p) {
  if (p) cudaFreeAsync(p, dev().s);
}
template <typename T>
T* upload(const std::vector<T>& v) {
  if (v.empty()) return nullptr;
  T* p = (T*)dalloc(v.size() * sizeof(T));
  CK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, dev().s));
  return p;
}

// ---- kernel table ---------------------------------------------------------------
struct Kern {
  int (*batch)(const InstDesc*, int, int*, int, int, int, size_t, void*);
  int (*grid)(const InstDesc*, int, const EvalIO*, int, GridSyncState*, double*, int, int, size_t, void*);
  int (*occ)(int, int, size_t, int*);
  int (*cta_eval)(const InstDesc*, const EvalIO*, int, size_t, void*);
  int (*cbatch)(const InstDesc*, int, int*, int, int, int, int, size_t, void*);
  int (*cocc)(int, int, size_t, int*);
};
#define MG_KERN(N)                                                                              \
  Kern {                                                                                        \
    mg_launch_batch_##N, mg_launch_grid_##N, mg_occupancy_##N, mg_launch_cta_eval_##N,          \
        mg_launch_cbatch_##N, mg_cluster_occupancy_##N                                          \
  }
Kern kern(int kk) {
  switch (kk) {
    case K_LJ: return MG_KERN(lj);
    case K_PF: return MG_KERN(pf);
    case K_BAH: return MG_KERN(bah);
    default: return MG_KERN(pf1);
  }
}
#undef MG_KERN
// Lennard-Jones shared memory: 1536 particles of 4 doubles (the tiles of the
// generic pair loop), or positions and eight warps' force accumulators of
// up to 416 particles (the dealt FP32 evaluation)
const size_t kLjTileBytes = 1536 * 32;
// dynamic shared memory of a one-CTA (or cluster) batch launch of these
// instances with this many threads: the largest need among them
size_t group_smem(int kk, const InstDesc* d, int n, int threads) {
  if (kk != K_LJ) return 0;
  size_t s = 0;
  for (int i = 0; i < n; i++) s = std::max(s, lj_smem_bytes(d[i].lj.np, threads));
  return s;
}
// Grid launches of the grid-sized potentials can stream the minimiser's
// vector passes through a ring of kStages shared-memory stages of
// MINIM_GPU_STAGE_KB kilobytes each (at most 50; 4 x 22.5 KB keeps two
// blocks of 256 threads per SM).  The default, 0, reads global memory
// directly with L2 prefetch one sweep step ahead, which measures faster.
const int kStages = 4;
int stage_bytes_cfg() {
  static const int v = [] {
    const char* e = std::getenv("MINIM_GPU_STAGE_KB");
    double kb = e ? std::atof(e) : 0.0;
    kb = kb < 0 ? 0 : (kb > 50 ? 50 : kb);
    return ((int)(kb * 1024) / 256) * 256;
  }();
  return v;
}
int grid_stage_bytes(int kk) { return kk == K_LJ ? 0 : stage_bytes_cfg(); }
// The FP32 stage of L-BFGS on a large binary PhaseField runs as a graph of
// phase kernels (stepped.cu) unless MINIM_GPU_STEPPED=0.
bool stepped_cfg() {
  static const bool v = [] {
    const char* e = std::getenv("MINIM_GPU_STEPPED");
    return !(e && e[0] == '0');
  }();
  return v;
}
// The stepped graph's line-search trials evaluate two consecutive trials of
// the backtracking sequence per pass unless MINIM_GPU_TRIAL_PAIRS=0.
bool dual_cfg() {
  static const bool v = [] {
    const char* e = std::getenv("MINIM_GPU_TRIAL_PAIRS");
    return !(e && e[0] == '0');
  }();
  return v;
}
// BarAndHinge instances given by a triangulation are set up on the device
// (topology.cu) unless MINIM_GPU_BAH_DEVICE_SETUP=0.
bool bah_device_cfg() {
  static const bool v = [] {
    const char* e = std::getenv("MINIM_GPU_BAH_DEVICE_SETUP");
    return !(e && e[0] == '0');
  }();
  return v;
}
// L2 prefetch distance of the grid launches' sweeps, in sweep steps
// (MINIM_GPU_PREFETCH, default 1; 0 disables it).
int prefetch_cfg() {
  static const int v = [] {
    const char* e = std::getenv("MINIM_GPU_PREFETCH");
    const int d = e ? std::atoi(e) : 1;
    return d < 0 ? 0 : (d > 8 ? 8 : d);
  }();
  return v;
}
size_t grid_smem(int kk) { return kk == K_LJ ? kLjTileBytes : kStages * (size_t)stage_bytes_cfg(); }

// ---- workspace layout --------------------------------------------------------------
struct WsLayout {
  size_t x32[2], x64[2], g[2], x32s, gs, S, Y, V, total, hstride;
  int nS, nY;
  bool fp64;
  size_t sched;  // Anneal's tabulated temperatures
  int nsched;
};
size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }
// dual: the stepped path's spare buffers for two line-search trials per pass
// (a point, a gradient and one more y slot)
WsLayout ws_layout(size_t n, const minim_gpu_minimiser_params& mp, bool dual = false) {
  WsLayout L{};
  size_t o = 0;
  auto take = [&](size_t bytes) { size_t r = o; o += align256(bytes); return r; };
  L.fp64 = mp.precision != MINIM_PREC_FP32 || mp.method == MINIM_ANNEAL;
  L.nS = mp.method == MINIM_LBFGS ? mp.m + 1 : (mp.method == MINIM_FIRE ? 1 : 0);
  L.nY = mp.method == MINIM_LBFGS ? mp.m + 1 + (dual ? 1 : 0) : 0;
  for (int k = 0; k < 2; k++) L.x32[k] = take(n * 4);
  L.x32s = dual ? take(n * 4) : (size_t)-1;
  L.gs = dual ? take(n * 4) : (size_t)-1;
  for (int k = 0; k < 2; k++) L.x64[k] = L.fp64 ? take(n * 8) : (size_t)-1;
  for (int k = 0; k < 2; k++) L.g[k] = take(n * 4);
  L.hstride = (n + 63) & ~(size_t)63;
  // the direction pass addresses history slots with 32-bit float4 offsets
  if ((size_t)(L.nS > L.nY ? L.nS : L.nY) * L.hstride >= ((size_t)1 << 33))
    throw ApiError{MINIM_GPU_ERR_INVALID, "instance too large for the history layout"};
  L.S = L.nS ? take((size_t)L.nS * L.hstride * 4) : (size_t)-1;
  L.Y = L.nY ? take((size_t)L.nY * L.hstride * 4) : (size_t)-1;
  L.V = mp.method == MINIM_FIRE ? take(n * 4) : (size_t)-1;
  L.nsched = (mp.method == MINIM_ANNEAL && mp.n_temp_schedule > 0) ? mp.n_temp_schedule : 0;
  L.sched = L.nsched ? take((size_t)L.nsched * 8) : (size_t)-1;
  L.total = o;
  return L;
}
void ws_apply(InstDesc& d, char* base, const WsLayout& L) {
  for (int k = 0; k < 2; k++) {
    d.X32[k] = (float*)(base + L.x32[k]);
    d.X64[k] = L.fp64 ? (double*)(base + L.x64[k]) : nullptr;
    d.G[k] = (float*)(base + L.g[k]);
  }
  d.X32s = L.x32s != (size_t)-1 ? (float*)(base + L.x32s) : nullptr;
  d.Gs = L.gs != (size_t)-1 ? (float*)(base + L.gs) : nullptr;
  d.hstride = (int)L.hstride;
  d.Sb = L.nS ? (float*)(base + L.S) : nullptr;
  d.Yb = L.nY ? (float*)(base + L.Y) : nullptr;
  d.V = L.V != (size_t)-1 ? (float*)(base + L.V) : nullptr;
}
// after ws_apply and to_mp: Anneal's temperature table into the workspace
void ws_sched(InstDesc& d, char* base, const WsLayout& L, const std::vector<double>& sched, cudaStream_t s) {
  d.mp.ntsched = 0;
  d.mp.tsched = nullptr;
  if (!L.nsched || sched.empty()) return;
  CK(cudaMemcpyAsync(base + L.sched, sched.data(), (size_t)L.nsched * 8, cudaMemcpyHostToDevice, s));
  d.mp.tsched = (const double*)(base + L.sched);
  d.mp.ntsched = L.nsched;
}
std::vector<double> sched_of(const minim_gpu_minimiser_params& mp) {
  if (mp.method != MINIM_ANNEAL || mp.n_temp_schedule <= 0) return {};
  return std::vector<double>(mp.temp_schedule, mp.temp_schedule + mp.n_temp_schedule);
}

void check_mp(const minim_gpu_minimiser_params& mp) {
  if (mp.method < 0 || mp.method > 3) throw ApiError{MINIM_GPU_ERR_INVALID, "unknown minimiser method"};
  if (mp.method == MINIM_ANNEAL && (mp.n_temp_schedule < 0 || (mp.n_temp_schedule > 0 && !mp.temp_schedule)))
    throw ApiError{MINIM_GPU_ERR_INVALID, "Anneal: invalid temperature schedule"};
  if (mp.linesearch != MINIM_LS_BACKTRACKING && mp.linesearch != MINIM_LS_NONE)
    throw ApiError{MINIM_GPU_ERR_INVALID, "Invalid line search method."};
  if (mp.method == MINIM_LBFGS && (mp.m < 1 || mp.m > MINIM_MAXM))
    throw ApiError{MINIM_GPU_ERR_INVALID, "Lbfgs: m must be between 1 and 16 on the device"};
  if (mp.precision < 0 || mp.precision > 2) throw ApiError{MINIM_GPU_ERR_INVALID, "unknown precision"};
}

MinParams to_mp(const minim_gpu_minimiser_params& q, double tol) {
  MinParams p{};
  p.method = q.method;
  p.linesearch = q.linesearch;
  p.max_iter = q.max_iter;
  p.m = q.method == MINIM_LBFGS ? q.m : 0;
  p.precision = q.precision;
  p.tol = tol;
  p.max_step = q.max_step;
  p.init_step = q.init_step;
  p.dt_max = q.dt_max;
  p.alpha = q.alpha;
  if (q.method == MINIM_ANNEAL) {
    p.precision = MINIM_PREC_FP64;  // the Metropolis test compares FP64 energies
    p.temp_init = q.temp_init;
    p.displacement = q.displacement;
    p.cooling_rate = q.cooling_rate;
    p.max_rej = q.max_rejections;
    p.seed = q.seed;
  }
  return p;
}

MinScalars fresh_scalars() {
  MinScalars s;
  std::memset(&s, 0, sizeof s);
  s.status = ST_RUNNING;
  s.pend = -1;
  return s;
}

void fill_result(minim_gpu_result* r, const MinScalars& s, size_t n) {
  std::memset(r, 0, sizeof *r);
  r->status = s.status;
  r->iter = s.iter;
  r->fp64_iters = s.fp64_iters;
  r->evals = s.evals;
  r->energy = s.E;
  r->rms = std::sqrt(s.gg / (double)n);
  r->dt_max = s.dtmax;
  r->run_ms = (s.t_last > s.t_first && s.t_first) ? (double)(s.t_last - s.t_first) * 1e-6 : 0.0;
}

}  // namespace

// ---------------------------------------------------------------------------
// Instances
// ---------------------------------------------------------------------------
struct minim_gpu_instance_s {
  int kind = 0;
  int kk = 0;        // kernel kind
  size_t n = 0;
  InstDesc d{};      // potential part + resident pointers
  std::vector<void*> owned;
  double default_tol = 1e-6;
  BahHost bah;
  BahTopoDev bah_topo;   // device-built elements (bah_dev), before filtering and colouring
  bool bah_dev = false;
  std::vector<unsigned char> fixed;
  size_t pot_bytes = 0;
  // grid-launch resources (lazy)
  InstDesc* d_desc = nullptr;
  EvalIO* d_io = nullptr;
  GridSyncState* d_bar = nullptr;
  double* d_partials = nullptr;
  size_t partials_bytes = 0;
  double* d_tmp = nullptr;   // n doubles: API coordinates / vectors
  double* d_g = nullptr;     // n doubles: API gradient
  double* d_e = nullptr;
  int gblocks = 0, gthreads = 256;
  // single-instance workspace (lazy)
  void* ws = nullptr;
  size_t ws_bytes = 0;
  MinScalars* d_st = nullptr;

  void* own(void* p) {
    if (p) owned.push_back(p);
    return p;
  }
  template <typename T>
  T* own_upload(const std::vector<T>& v) {
    T* p = upload(v);
    own(p);
    pot_bytes += v.size() * sizeof(T);
    return p;
  }
  ~minim_gpu_instance_s() {
    for (void* p : owned) dfree(p);
    dfree(ws);
  }
};

namespace {

void upload_bah_arrays(minim_gpu_instance_s* h) {
  PotBAH& P = h->d.bah;
  if (h->bah_dev) {
    BahColouredDev C;
    const int rc = mg_bah_colour_device(&h->bah_topo, h->fixed.empty() ? nullptr : h->fixed.data(), &C, dev().s);
    if (rc == MG_TOPO_CUDA) throw ApiError{MINIM_GPU_ERR_CUDA, "BarAndHinge device colouring failed"};
    if (rc == MG_TOPO_OK) {
      P.nvert = h->bah.nvert;
      P.nbar = C.nbar;
      P.nhinge = C.nhinge;
      P.bars = (int2*)h->own(C.bars);
      P.bar_par = (double2*)h->own(C.bpar);
      P.hinges = (int4*)h->own(C.hinges);
      P.hinge_par = (double2*)h->own(C.hpar);
      P.nbar_colors = C.nbar_colors;
      P.nhinge_colors = C.nhinge_colors;
      P.bar_color_off = (int*)h->own(C.bar_off);
      P.hinge_color_off = (int*)h->own(C.hinge_off);
      P.node_el = (unsigned char*)h->own(C.node_el);
      P.nforce = (int)h->bah.force.size();
      P.force = h->own_upload(h->bah.force);
      P.wall_on = h->bah.wall_on;
      P.wall_adh = h->bah.wall_adh;
      P.wall_eps = h->bah.wall_eps;
      P.wall_sig = h->bah.wall_sig;
      return;
    }
    // more colours than the device colouring handles: continue on the host
    // from the device-built elements
    const BahTopoDev& T = h->bah_topo;
    std::vector<int2> b2(T.nbar);
    std::vector<int4> h4(T.nhinge);
    std::vector<double2> bp(T.nbar), hp(T.nhinge);
    CK(cudaMemcpyAsync(b2.data(), T.bars, b2.size() * sizeof(int2), cudaMemcpyDeviceToHost, dev().s));
    CK(cudaMemcpyAsync(bp.data(), T.bpar, bp.size() * sizeof(double2), cudaMemcpyDeviceToHost, dev().s));
    CK(cudaMemcpyAsync(h4.data(), T.hinges, h4.size() * sizeof(int4), cudaMemcpyDeviceToHost, dev().s));
    CK(cudaMemcpyAsync(hp.data(), T.hpar, hp.size() * sizeof(double2), cudaMemcpyDeviceToHost, dev().s));
    CK(cudaStreamSynchronize(dev().s));
    for (size_t i = 0; i < b2.size(); i++) {
      h->bah.bars.insert(h->bah.bars.end(), {b2[i].x, b2[i].y});
      h->bah.bpar.insert(h->bah.bpar.end(), {bp[i].x, bp[i].y});
    }
    for (size_t i = 0; i < h4.size(); i++) {
      h->bah.hinges.insert(h->bah.hinges.end(), {h4[i].x, h4[i].y, h4[i].z, h4[i].w});
      h->bah.hpar.insert(h->bah.hpar.end(), {hp[i].x, hp[i].y});
    }
    h->bah_dev = false;
  }
  BahDevArrays A = bah_arrays(h->bah, h->fixed);
  P.nvert = h->bah.nvert;
  P.nbar = (int)A.bars.size();
  P.nhinge = (int)A.hinges.size();
  P.bars = h->own_upload(A.bars);
  P.bar_par = h->own_upload(A.bpar);
  P.hinges = h->own_upload(A.hinges);
  P.hinge_par = h->own_upload(A.hpar);
  P.nbar_colors = (int)A.bar_off.size() - 1;
  P.nhinge_colors = (int)A.hinge_off.size() - 1;
  P.bar_color_off = h->own_upload(A.bar_off);
  P.hinge_color_off = h->own_upload(A.hinge_off);
  P.node_el = h->own_upload(A.node_el);
  P.nforce = (int)h->bah.force.size();
  P.force = h->own_upload(h->bah.force);
  P.wall_on = h->bah.wall_on;
  P.wall_adh = h->bah.wall_adh;
  P.wall_eps = h->bah.wall_eps;
  P.wall_sig = h->bah.wall_sig;
}

minim_gpu_instance_s* create_instance(int kind, const void* params, const double* x0, size_t ndof) {
  need_dev();
  if (!params || !x0 || ndof == 0) throw ApiError{MINIM_GPU_ERR_INVALID, "null parameters or empty coordinates"};
  if (ndof > 0x7fffffffULL) throw ApiError{MINIM_GPU_ERR_INVALID, "too many degrees of freedom"};
  auto h = new minim_gpu_instance_s();
  try {
    h->kind = kind;
    h->n = ndof;
    h->d.kind = kind;
    h->d.ndof = (int)ndof;
    if (kind == MINIM_GPU_LJ) {
      auto q = (const minim_gpu_lj_params*)params;
      if (q->ndim < 2 || q->ndim > 3 || ndof % q->ndim)
        throw ApiError{MINIM_GPU_ERR_INVALID, "LjNd: Length of coords must be a multiple of the number of dimensions."};
      h->kk = K_LJ;
      h->d.lj.ndim = q->ndim;
      h->d.lj.np = (int)(ndof / q->ndim);
      h->d.lj.s6 = std::pow(q->sigma, 6);
      h->d.lj.eps = q->epsilon;
      if (!(q->cutoff >= 0) || std::isinf(q->cutoff))
        throw ApiError{MINIM_GPU_ERR_INVALID, "LjNd: the cutoff must be a finite value >= 0."};
      if (q->cutoff > 0) {
        // cell-list scratch: a hash table of at least 2N buckets
        int hb = 6;
        while (((size_t)1 << hb) < 2 * (size_t)h->d.lj.np) hb++;
        h->d.lj.rc2 = q->cutoff * q->cutoff;
        h->d.lj.inv_cs = 1.0 / (q->cutoff * (1.0 + 1e-3));
        h->d.lj.hbits = hb;
        h->d.lj.cells = (int*)h->own(dalloc(lj_cell_ints(h->d.lj.np, hb) * sizeof(int)));
      }
    } else if (kind == MINIM_GPU_PF || kind == MINIM_GPU_PFU) {
      PfHost H = setup_pf(*(const minim_gpu_pf_params*)params, x0, ndof, kind == MINIM_GPU_PFU);
      h->kk = H.kernel_kind;
      h->default_tol = H.default_tol;
      h->d.pf = H.pot;
      h->d.pf.aux = h->own_upload(H.aux);
      h->d.pf.wet = h->own_upload(H.wet);
      h->d.pf.kappa_node = h->own_upload(H.kappa_node);
      h->d.pf.kappaP_node = h->own_upload(H.kappaP_node);
      h->d.pf.ff_init = h->own_upload(H.ff_init);
    } else if (kind == MINIM_GPU_BAH) {
      h->kk = K_BAH;
      const auto* q = (const minim_gpu_bah_params*)params;
      if (ndof % 3) throw ApiError{MINIM_GPU_ERR_INVALID, "BarAndHinge: coordinates must be 3 per vertex"};
      bool built = false;
      if (bah_device_cfg() && q->ntri > 0 && q->nbond == 0 && q->nhinge == 0) {
        char msg[256] = {0};
        const int rc = mg_bah_topology_device(q, x0, (int)(ndof / 3), &h->bah_topo, dev().s, msg, (int)sizeof msg);
        if (rc == MG_TOPO_INVALID) throw ApiError{MINIM_GPU_ERR_INVALID, msg};
        if (rc == MG_TOPO_CUDA) throw ApiError{MINIM_GPU_ERR_CUDA, "BarAndHinge device set-up failed"};
        if (rc == MG_TOPO_OK) {
          h->own(h->bah_topo.bars);
          h->own(h->bah_topo.bpar);
          h->own(h->bah_topo.hinges);
          h->own(h->bah_topo.hpar);
          h->bah = BahHost{};
          h->bah.nvert = (int)(ndof / 3);
          bah_scalars(*q, h->bah);
          h->bah_dev = true;
          built = true;
        }
      }
      if (!built) h->bah = setup_bah(*q, x0, ndof);
      upload_bah_arrays(h);
      h->d.GA = (double*)h->own(dalloc(ndof * sizeof(double)));
    } else {
      throw ApiError{MINIM_GPU_ERR_INVALID, "unknown potential kind"};
    }
    h->d.kind = kind;
    h->d.xres = (double*)h->own(dalloc(ndof * sizeof(double)));
    CK(cudaMemcpyAsync(h->d.xres, x0, ndof * sizeof(double), cudaMemcpyHostToDevice, dev().s));
    CK(cudaStreamSynchronize(dev().s));
  } catch (...) {
    delete h;
    throw;
  }
  return h;
}

void ensure_grid(minim_gpu_instance_s* h) {
  Dev& D = need_dev();
  if (h->d_desc) return;
  int per_sm = 0;
  CK((cudaError_t)kern(h->kk).occ(1, h->gthreads, grid_smem(h->kk), &per_sm));
  if (per_sm < 1) throw ApiError{MINIM_GPU_ERR_CUDA, "grid kernel does not fit on an SM"};
  h->gblocks = D.nsm * per_sm;
  h->d_desc = (InstDesc*)h->own(dalloc(sizeof(InstDesc)));
  h->d_io = (EvalIO*)h->own(dalloc(sizeof(EvalIO)));
  h->d_bar = (GridSyncState*)h->own(dalloc(sizeof(GridSyncState)));
  h->partials_bytes = (2 * (size_t)h->gblocks * 64 + 2 * 64) * sizeof(double) + (size_t)h->gblocks * 4;
  h->d_partials = (double*)h->own(dalloc(h->partials_bytes));
  h->d_e = (double*)h->own(dalloc(sizeof(double)));
  h->d_tmp = (double*)h->own(dalloc(h->n * sizeof(double)));
  h->d_g = (double*)h->own(dalloc(h->n * sizeof(double)));
}

void launch_grid(minim_gpu_instance_s* h, int op, int slice) {
  Dev& D = need_dev();
  CK(cudaMemsetAsync(h->d_bar, 0, sizeof(GridSyncState), D.s));
  // barrier flags and epochs restart at 0 in every launch
  const size_t flag_off = (2 * (size_t)h->gblocks * 64 + 2 * 64) * sizeof(double);
  CK(cudaMemsetAsync((char*)h->d_partials + flag_off, 0, h->partials_bytes - flag_off, D.s));
  CK((cudaError_t)kern(h->kk).grid(h->d_desc, op, h->d_io, slice, h->d_bar, h->d_partials, h->gthreads,
                                    h->gblocks, grid_smem(h->kk), D.s));
  g_launches++;
}

int grid_error(minim_gpu_instance_s* h) {
  GridSyncState b;
  CK(cudaMemcpyAsync(&b, h->d_bar, sizeof b, cudaMemcpyDeviceToHost, dev().s));
  CK(cudaStreamSynchronize(dev().s));
  return b.err;
}

void do_eval(minim_gpu_instance_s* h, const double* x, double* e, double* g) {
  Dev& D = need_dev();
  ensure_grid(h);
  const double* xd = h->d.xres;
  if (x) {
    CK(cudaMemcpyAsync(h->d_tmp, x, h->n * sizeof(double), cudaMemcpyHostToDevice, D.s));
    xd = h->d_tmp;
  }
  EvalIO io{};
  io.x = xd;
  io.g = g ? h->d_g : nullptr;
  io.e = h->d_e;
  InstDesc d = h->d;
  d.fixed = h->d.fixed;
  CK(cudaMemcpyAsync(h->d_desc, &d, sizeof d, cudaMemcpyHostToDevice, D.s));
  CK(cudaMemcpyAsync(h->d_io, &io, sizeof io, cudaMemcpyHostToDevice, D.s));
  launch_grid(h, OP_EVAL, 0);
  double ev = 0;
  CK(cudaMemcpyAsync(&ev, h->d_e, sizeof(double), cudaMemcpyDeviceToHost, D.s));
  if (g) CK(cudaMemcpyAsync(g, h->d_g, h->n * sizeof(double), cudaMemcpyDeviceToHost, D.s));
  CK(cudaStreamSynchronize(D.s));
  if (grid_error(h)) throw ApiError{MINIM_GPU_ERR_RUNTIME, "device barrier timed out"};
  if (e) *e = ev;
}

int rule_threads(int kk, const InstDesc& d);

// One evaluation by a minimiser stage's own potential kernels (the checks of
// minim_gpu_eval_kernel).  Temporary buffers come from the caching pool.
void do_eval_kernel(minim_gpu_instance_s* h, int path, const double* x, const double* p, double t, double* e,
                    double* g, double* xt) {
  Dev& D = need_dev();
  if (path < MINIM_EVAL_FP32_GRID || path > MINIM_EVAL_LINES_TMA || !x)
    throw ApiError{MINIM_GPU_ERR_INVALID, "minim_gpu_eval_kernel: invalid path or null coordinates"};
  const bool tma = path == MINIM_EVAL_LINES_TMA;
  const bool lines = path == MINIM_EVAL_LINES || tma;
  if (xt && !lines)
    throw ApiError{MINIM_GPU_ERR_INVALID, "minim_gpu_eval_kernel: xt is only returned by the line stencil"};
  if (lines && h->kk != K_PF1)
    throw ApiError{MINIM_GPU_ERR_INVALID, "minim_gpu_eval_kernel: the line stencil runs binary PhaseField "
                                          "instances without optional terms only"};
  if (tma && !g) throw ApiError{MINIM_GPU_ERR_INVALID, "minim_gpu_eval_kernel: the TMA line stencil needs g"};
  if (tma) {
    const int* n = h->d.pf.n;
    if (n[2] % 32 || n[2] > 256 || n[1] % 4 || n[1] < 8 || n[0] < 3)
      throw ApiError{MINIM_GPU_ERR_INVALID, "minim_gpu_eval_kernel: the grid does not take the TMA line stencil"};
  }
  ensure_grid(h);
  const size_t n = h->n, vb = align256(n * sizeof(float));
  // x32, p32, g32, two scratch vectors, and the line stencil's Xa Ga Ya Xb Gb Yb Go
  const int nvec = lines ? 12 : 5;
  const int max_rows = 16 * D.nsm;
  char* buf = (char*)dalloc(nvec * vb + (size_t)max_rows * MINIM_WIDE * sizeof(double));
  auto vec = [&](int k) { return (float*)(buf + (size_t)k * vb); };
  float* x32 = vec(0);
  float* p32 = p ? vec(1) : nullptr;
  float* g32 = g ? vec(2) : nullptr;
  try {
    CK(cudaMemcpyAsync(h->d_tmp, x, n * sizeof(double), cudaMemcpyHostToDevice, D.s));
    CK((cudaError_t)mg_convert(h->d_tmp, x32, n, 1, D.s));
    std::vector<float> ph;
    if (p) {
      ph.resize(n);
      for (size_t i = 0; i < n; i++) ph[i] = (float)p[i];
      CK(cudaMemcpyAsync(p32, ph.data(), n * sizeof(float), cudaMemcpyHostToDevice, D.s));
    }
    double ev[2] = {0.0, 0.0};
    std::vector<float> gh;
    if (lines) {
      // trials of a direction: both gradients are written, so a zero
      // direction stands in for p == NULL
      if (!p32) {
        p32 = vec(1);
        CK(cudaMemsetAsync(p32, 0, n * sizeof(float), D.s));
      }
      float* Go = vec(11);
      CK(cudaMemsetAsync(Go, 0, n * sizeof(float), D.s));
      CK(cudaMemcpyAsync(h->d_desc, &h->d, sizeof(InstDesc), cudaMemcpyHostToDevice, D.s));
      double* part = (double*)(buf + nvec * vb);
      int rows = 0;
      const int mode = g ? 3 : 0;
      if (tma)
        CK((cudaError_t)mg_stepped_lines_tma_probe(h->d_desc, h->d.pf.n, x32, p32, Go, (float)t, vec(5), vec(6),
                                                   vec(7), vec(8), vec(9), vec(10), part, max_rows, D.nsm, &rows,
                                                   D.s));
      else
        CK((cudaError_t)mg_stepped_lines_probe(h->d_desc, h->d.pf.n, mode, x32, p32, Go, (float)t, vec(5),
                                               vec(6), vec(7), vec(8), vec(9), vec(10), part, max_rows, D.nsm,
                                               &rows, D.s));
      g_launches++;
      std::vector<double> hp((size_t)rows * MINIM_WIDE);
      CK(cudaMemcpyAsync(hp.data(), part, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, D.s));
      if (g || xt) gh.resize(4 * n);
      if (g) {
        CK(cudaMemcpyAsync(gh.data(), vec(6), n * sizeof(float), cudaMemcpyDeviceToHost, D.s));
        CK(cudaMemcpyAsync(gh.data() + n, vec(9), n * sizeof(float), cudaMemcpyDeviceToHost, D.s));
      }
      if (xt && g) {
        CK(cudaMemcpyAsync(gh.data() + 2 * n, vec(5), n * sizeof(float), cudaMemcpyDeviceToHost, D.s));
        CK(cudaMemcpyAsync(gh.data() + 3 * n, vec(8), n * sizeof(float), cudaMemcpyDeviceToHost, D.s));
      }
      CK(cudaStreamSynchronize(D.s));
      // rows: {E, g.g, P.y, y.y, E2, ...} (mode 3) or {E} (mode 0), summed in block order
      for (int r = 0; r < rows; r++) {
        ev[0] += hp[(size_t)r * MINIM_WIDE];
        if (mode == 3) ev[1] += hp[(size_t)r * MINIM_WIDE + 4];
      }
      if (e) {
        e[0] = ev[0];
        if (mode == 3) e[1] = ev[1];
      }
      if (g)
        for (size_t i = 0; i < 2 * n; i++) g[i] = gh[i];
      if (xt) {
        if (!g) throw ApiError{MINIM_GPU_ERR_INVALID, "minim_gpu_eval_kernel: the energy-only pass forms no point"};
        for (size_t i = 0; i < 2 * n; i++) xt[i] = gh[2 * n + i];
      }
      dfree(buf);
      return;
    }
    InstDesc d = h->d;
    d.X32[0] = vec(3);  // scratch of the double-float sweeps
    d.X32[1] = vec(4);
    d.mp = MinParams{};
    d.mp.method = MINIM_LBFGS;
    EvalIO io{};
    io.x = h->d_tmp;
    io.e = h->d_e;
    io.stage = (path == MINIM_EVAL_FP64S_GRID || path == MINIM_EVAL_FP64S_CTA) ? 1 : 0;
    io.t32 = (float)t;
    io.t64 = t;
    io.x32 = x32;
    io.p = p32;
    io.g32 = g32;
    CK(cudaMemcpyAsync(h->d_desc, &d, sizeof d, cudaMemcpyHostToDevice, D.s));
    CK(cudaMemcpyAsync(h->d_io, &io, sizeof io, cudaMemcpyHostToDevice, D.s));
    if (path == MINIM_EVAL_FP32_GRID || path == MINIM_EVAL_FP64S_GRID) {
      launch_grid(h, OP_EVAL_STAGE, 0);
    } else {
      const int thr = rule_threads(h->kk, h->d);
      CK((cudaError_t)kern(h->kk).cta_eval(h->d_desc, h->d_io, thr, group_smem(h->kk, &h->d, 1, thr), D.s));
      g_launches++;
    }
    CK(cudaMemcpyAsync(&ev[0], h->d_e, sizeof(double), cudaMemcpyDeviceToHost, D.s));
    if (g) {
      gh.resize(n);
      CK(cudaMemcpyAsync(gh.data(), g32, n * sizeof(float), cudaMemcpyDeviceToHost, D.s));
    }
    CK(cudaStreamSynchronize(D.s));
    if ((path == MINIM_EVAL_FP32_GRID || path == MINIM_EVAL_FP64S_GRID) && grid_error(h))
      throw ApiError{MINIM_GPU_ERR_RUNTIME, "device barrier timed out"};
    if (e) e[0] = ev[0];
    if (g)
      for (size_t i = 0; i < n; i++) g[i] = gh[i];
  } catch (...) {
    cudaStreamSynchronize(D.s);
    dfree(buf);
    throw;
  }
  dfree(buf);
}

void do_minimise(minim_gpu_instance_s* h, const minim_gpu_minimiser_params& mp, minim_gpu_result* res) {
  Dev& D = need_dev();
  check_mp(mp);
  ensure_grid(h);
  const double tol = mp.tol >= 0 ? mp.tol : h->default_tol;
  // the FP32 stage of a large binary PhaseField L-BFGS runs as the stepped graph
  const bool stepped_ok = stepped_cfg() && h->kk == K_PF1 && mp.method == MINIM_LBFGS &&
                          mp.precision != MINIM_PREC_FP64 && h->d.fixed == nullptr && h->n >= ((size_t)1 << 18);
  // two trials per pass; its graph sets up the line search in the first
  // pass's controller, which has no step cap (Lbfgs::setMaxStep)
  const bool dual = stepped_ok && dual_cfg() && mp.max_step == 0;
  WsLayout L = ws_layout(h->n, mp, dual);
  const size_t need = L.total + align256(sizeof(MinScalars));
  if (need > h->ws_bytes) {
    dfree(h->ws);
    h->ws = dalloc(need);
    h->ws_bytes = need;
  }
  InstDesc d = h->d;
  ws_apply(d, (char*)h->ws, L);
  d.mp = to_mp(mp, tol);
  ws_sched(d, (char*)h->ws, L, sched_of(mp), D.s);
  d.stage_bytes = grid_stage_bytes(h->kk);
  d.pf_dist = prefetch_cfg();
  d.pf.pf_dist = d.pf_dist;
  h->d_st = (MinScalars*)((char*)h->ws + L.total);
  d.st = h->d_st;
  MinScalars s = fresh_scalars();
  s.ybuf2 = dual ? mp.m + 1 : -1;
  CK(cudaMemcpyAsync(h->d_st, &s, sizeof s, cudaMemcpyHostToDevice, D.s));
  CK(cudaMemcpyAsync(h->d_desc, &d, sizeof d, cudaMemcpyHostToDevice, D.s));
  int slice = 64;
  const double t0 = now_ms();
  minim_gpu_run_stats stats{};
  cudaEvent_t ev0, ev1;
  CK(cudaEventCreate(&ev0));
  CK(cudaEventCreate(&ev1));
  const bool stepped = stepped_ok && L.total < ((size_t)1 << 34);  // signed 32-bit float4 offsets across the workspace
  if (stepped) {
    // iteration 0 (set-up) on the persistent kernel, then the FP32 stage as
    // graph launches until it hands over (precision switch, convergence,
    // NaN) or stops
    CK(cudaEventRecord(ev0, D.s));
    launch_grid(h, OP_MINIMISE, 1);
    CK(cudaEventRecord(ev1, D.s));
    CK(cudaMemcpyAsync(&s, h->d_st, sizeof s, cudaMemcpyDeviceToHost, D.s));
    CK(cudaStreamSynchronize(D.s));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, ev0, ev1));
    stats.kernel_ms += ms;
    stats.launches++;
    if (grid_error(h)) s.status = ST_TIMEOUT;
    while (s.status == ST_RUNNING && s.stage == 0 && !s.resume) {
      const int it0 = s.iter;
      double kernels = 0;
      CK(cudaEventRecord(ev0, D.s));
      CK((cudaError_t)mg_stepped_pf1_run(h->d_desc, &d, h->d_st, mp.m, h->d.pf.n, D.nsm, 4096, dual ? 1 : 0, D.s, &kernels));
      CK(cudaEventRecord(ev1, D.s));
      CK(cudaMemcpyAsync(&s, h->d_st, sizeof s, cudaMemcpyDeviceToHost, D.s));
      CK(cudaStreamSynchronize(D.s));
      CK(cudaEventElapsedTime(&ms, ev0, ev1));
      stats.kernel_ms += ms;
      stats.launches += (int64_t)kernels;
      g_launches += (int64_t)kernels;
      if ((s.iter == it0 && !s.resume) || s.iter > mp.max_iter) break;  // not eligible, or done
    }
  }
  for (; s.status == ST_RUNNING;) {
    CK(cudaEventRecord(ev0, D.s));
    launch_grid(h, OP_MINIMISE, slice);
    CK(cudaEventRecord(ev1, D.s));
    CK(cudaMemcpyAsync(&s, h->d_st, sizeof s, cudaMemcpyDeviceToHost, D.s));
    CK(cudaStreamSynchronize(D.s));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, ev0, ev1));
    stats.kernel_ms += ms;
    stats.launches++;
    if (s.status != ST_RUNNING) break;
    if (grid_error(h)) {
      s.status = ST_TIMEOUT;
      break;
    }
    slice = std::min(slice * 2, 4096);
  }
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  stats.wall_ms = now_ms() - t0;
  stats.abytes = s.abytes;
  stats.pairs32 = s.pairs32;
  stats.pairs64 = s.pairs64;
  stats.iterations = s.iter + (s.status == ST_CONVERGED ? 1 : 0);
  stats.fp64_iterations = s.fp64_iters;
  for (int k = 0; k < 3; k++) stats.phase_ms[k] = s.tphase[k] * 1e-6;
  if (s.switch_reason > 0 && s.switch_reason < 4) stats.switches[s.switch_reason]++;
  g_stats = stats;
  if (res) fill_result(res, s, h->n);
}

template <class F>
int guarded(F&& f) {
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  try {
    f();
    return MINIM_GPU_OK;
  } catch (const ApiError& e) {
    g_err = e.msg;
    return e.code;
  } catch (const SetupError& e) {
    g_err = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    g_err = "host allocation failed";
    return MINIM_GPU_ERR_OOM;
  } catch (const std::exception& e) {
    g_err = e.what();
    return MINIM_GPU_ERR_RUNTIME;
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Batches
// ---------------------------------------------------------------------------
struct minim_gpu_batch_s {
  std::vector<minim_gpu_handle> inst;
  std::vector<minim_gpu_minimiser_params> mp;
  std::vector<std::vector<double>> sched;  // Anneal schedules, copied at batch_add
};

namespace {

double cost_of(const InstDesc& d, int kk) {
  if (kk == K_LJ) return (double)d.lj.np * d.lj.np;
  if (kk == K_BAH) return (double)d.bah.nbar + 4.0 * d.bah.nhinge + d.ndof;
  return (double)d.ndof;
}

// ---- launch shapes and the autotuner ----------------------------------------------
// An instance's batch launch shape (threads per CTA) is a function of its
// own kernel kind, size bucket, method and precision only -- never of the
// rest of the batch -- so that its result is the same alone and in any mix.
// The shape of a (kind, bucket, method, precision) key is chosen the first
// time the key is seen in the process: every candidate runs a short slice
// of the same instances (copies of their coordinates and state; the
// workspace is not yet in use) and the fastest is kept.  MINIM_GPU_TUNE=0
// takes the size rule instead; MINIM_GPU_TUNE_CACHE names a file that keeps
// the choices across processes (keyed by the device name and the driver).
int size_bucket(int kk, const InstDesc& d) {
  if (kk == K_LJ) {
    static const int edges[] = {32, 64, 96, 128, 192, 256, 384, 512, 768, 1024, 1536};
    int b = 0;
    while (b < 11 && d.lj.np > edges[b]) b++;
    return b;
  }
  static const double edges[] = {4096, 16384, 65536, 262144, 1048576};
  const double sz = kk == K_BAH ? (double)d.bah.nvert * 3 : (double)d.ndof;
  int b = 0;
  while (b < 5 && sz > edges[b]) b++;
  return b;
}

// A batch launch shape: threads per CTA and CTAs per instance (a
// thread-block cluster of that many CTAs, on as many SMs; 1 = one CTA).
struct Shape {
  int threads, csize;
  bool operator==(const Shape& o) const { return threads == o.threads && csize == o.csize; }
};

// The size rule: Lennard-Jones 64 / 128 / 256 threads by cluster size; the
// grid-sized kinds 512 (one CTA per SM at 128 registers a thread: sixteen
// warps to hide the stencil's and the element gathers' latency); one CTA
// per instance.
Shape rule_shape(int kk, const InstDesc& d) {
  if (kk == K_LJ) return {d.lj.np <= 96 ? 64 : (d.lj.np <= 192 ? 128 : 256), 1};
  return {512, 1};
}
int rule_threads(int kk, const InstDesc& d) { return rule_shape(kk, d).threads; }

// Candidates of a key: one CTA per instance with each thread count, and for
// large instances (Lennard-Jones above 512 particles, grid-sized kinds above
// 16k degrees of freedom) clusters of 2, 4 and 8 CTAs.
std::vector<Shape> shape_candidates(int kk, int bucket) {
  if (kk == K_LJ) {
    std::vector<Shape> c = {{64, 1}, {128, 1}, {256, 1}};
    if (bucket >= 8) c.insert(c.end(), {{256, 2}, {256, 4}, {256, 8}});
    return c;
  }
  std::vector<Shape> c = {{256, 1}, {512, 1}};
  if (bucket >= 2) c.insert(c.end(), {{512, 2}, {512, 4}, {512, 8}});
  return c;
}
constexpr int kMaxCand = 8;

struct TuneKey {
  int kk, bucket, method, prec;
  bool operator==(const TuneKey& o) const {
    return kk == o.kk && bucket == o.bucket && method == o.method && prec == o.prec;
  }
};
struct TuneEntry {
  TuneKey key;
  Shape shape;
  double ms[kMaxCand];  // measured time per candidate (0: not measured)
  int from_file;
};
std::vector<TuneEntry> g_tune;
bool g_tune_loaded = false;
double g_tune_ms = 0;  // device time spent tuning in the last batch call

TuneKey tune_key(int kk, const InstDesc& d) {
  return {kk, size_bucket(kk, d), d.mp.method, d.mp.precision};
}

std::string tune_device_tag() {
  cudaDeviceProp p;
  int drv = 0;
  cudaGetDeviceProperties(&p, dev().id);
  cudaDriverGetVersion(&drv);
  std::string tag = std::string(p.name) + "/" + std::to_string(drv);
  for (auto& c : tag)
    if (c == ' ') c = '_';
  return tag;
}

void tune_load() {
  if (g_tune_loaded) return;
  g_tune_loaded = true;
  const char* fn = std::getenv("MINIM_GPU_TUNE_CACHE");
  if (!fn || !*fn) return;
  FILE* f = std::fopen(fn, "r");
  if (!f) return;
  const std::string tag = tune_device_tag();
  char dev_tag[256];
  TuneEntry e{};
  while (std::fscanf(f, "%255s %d %d %d %d %d %d", dev_tag, &e.key.kk, &e.key.bucket, &e.key.method,
                     &e.key.prec, &e.shape.threads, &e.shape.csize) == 7) {
    if (tag != dev_tag) continue;
    bool ok = false;
    for (const Shape& c : shape_candidates(e.key.kk, e.key.bucket)) ok |= c == e.shape;
    if (!ok) continue;
    e.from_file = 1;
    g_tune.push_back(e);
  }
  std::fclose(f);
}

void tune_save(const TuneEntry& e) {
  const char* fn = std::getenv("MINIM_GPU_TUNE_CACHE");
  if (!fn || !*fn) return;
  FILE* f = std::fopen(fn, "a");
  if (!f) return;
  std::fprintf(f, "%s %d %d %d %d %d %d\n", tune_device_tag().c_str(), e.key.kk, e.key.bucket, e.key.method,
               e.key.prec, e.shape.threads, e.shape.csize);
  std::fclose(f);
}

bool tune_enabled() {
  const char* e = std::getenv("MINIM_GPU_TUNE");
  return !(e && e[0] == '0');
}

const TuneEntry* tune_find(const TuneKey& k) {
  for (auto& e : g_tune)
    if (e.key == k) return &e;
  return nullptr;
}

// Resident blocks (csize 1) or clusters (csize > 1) of a shape, 0 when it
// does not fit.
int shape_slots(int kk, const Shape& sh, size_t smem) {
  Dev& D = need_dev();
  if (sh.csize == 1) {
    int per_sm = 0;
    CK((cudaError_t)kern(kk).occ(0, sh.threads, smem, &per_sm));
    return per_sm * D.nsm;
  }
  int clusters = 0;
  const cudaError_t e = (cudaError_t)kern(kk).cocc(sh.threads, sh.csize, smem, &clusters);
  if (e != cudaSuccess) {
    cudaGetLastError();  // a cluster shape the device cannot hold: not a candidate
    return 0;
  }
  return clusters;
}

// One batch launch of instances [d_insts, +ninst) with a shape on a stream.
void launch_shape(int kk, const Shape& sh, const InstDesc* d_insts, int ninst, int* counter, int slice, int slots,
                  size_t smem, cudaStream_t s) {
  const int n = std::min(ninst, slots);
  if (sh.csize == 1)
    CK((cudaError_t)kern(kk).batch(d_insts, ninst, counter, slice, sh.threads, n, smem, s));
  else
    CK((cudaError_t)kern(kk).cbatch(d_insts, ninst, counter, slice, sh.threads, sh.csize, n, smem, s));
  g_launches++;
}

// Times every candidate shape on a short slice of the given fresh
// instances (at most two per SM of them, largest first) and records the
// fastest for the key.
void tune_measure(const TuneKey& key, const std::vector<InstDesc>& sample) {
  Dev& D = need_dev();
  const int ns = (int)sample.size();
  const char* it_env = std::getenv("MINIM_GPU_TUNE_ITERS");
  const int iters = it_env ? std::max(1, std::atoi(it_env)) : 12;
  // trial copies: the coordinates (written back by an instance that stops
  // within the slice) and fresh state records
  size_t xbytes = 0;
  std::vector<size_t> xo(ns);
  for (int i = 0; i < ns; i++) {
    xo[i] = xbytes;
    xbytes += align256((size_t)sample[i].ndof * sizeof(double));
  }
  char* xcopy = (char*)dalloc(xbytes);
  MinScalars* st = (MinScalars*)dalloc(ns * sizeof(MinScalars));
  InstDesc* dd = (InstDesc*)dalloc(ns * sizeof(InstDesc));
  int* counter = (int*)dalloc(sizeof(int));
  std::vector<InstDesc> trial(sample);
  for (int i = 0; i < ns; i++) {
    trial[i].xres = (double*)(xcopy + xo[i]);
    trial[i].st = st + i;
    CK(cudaMemcpyAsync(trial[i].xres, sample[i].xres, sample[i].ndof * sizeof(double), cudaMemcpyDeviceToDevice,
                       D.s));
  }
  CK(cudaMemcpyAsync(dd, trial.data(), ns * sizeof(InstDesc), cudaMemcpyHostToDevice, D.s));
  std::vector<MinScalars> fresh(ns, fresh_scalars());
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  TuneEntry ent{};
  ent.key = key;
  // the slice on the first `count` instances of the sample with a shape:
  // two runs, the second timed (the first loads the kernel)
  auto time_shape = [&](const Shape& sh, int count) -> float {
    const size_t smem = group_smem(key.kk, sample.data(), count, sh.threads);
    const int slots = shape_slots(key.kk, sh, smem);
    if (slots < 1) return -1.f;
    float ms = 0;
    for (int rep = 0; rep < 2; rep++) {
      CK(cudaMemcpyAsync(st, fresh.data(), ns * sizeof(MinScalars), cudaMemcpyHostToDevice, D.s));
      CK(cudaMemsetAsync(counter, 0, sizeof(int), D.s));
      CK(cudaEventRecord(e0, D.s));
      launch_shape(key.kk, sh, dd, count, counter, iters, slots, smem, D.s);
      CK(cudaEventRecord(e1, D.s));
      CK(cudaEventSynchronize(e1));
      CK(cudaEventElapsedTime(&ms, e0, e1));
      g_tune_ms += ms;
    }
    return ms;
  };
  // one CTA per instance: the shape that runs the sample fastest
  double best = 1e300;
  const std::vector<Shape> cand = shape_candidates(key.kk, key.bucket);
  bool clusters = false;
  for (size_t c = 0; c < cand.size() && c < (size_t)kMaxCand; c++) {
    if (cand[c].csize > 1) {
      clusters = true;
      continue;
    }
    const float ms = time_shape(cand[c], ns);
    if (ms < 0) continue;
    ent.ms[c] = ms;
    if (ms < best) {
      best = ms;
      ent.shape = cand[c];
    }
  }
  // Large instances: a batch's makespan is at least its largest instance's
  // time on its CTAs, so the cluster shapes are judged by the slice time of
  // the sample's largest instance alone; the largest cluster whose parallel
  // efficiency t(1) / (C t(C)) is at least 1/2 is taken.  (The one-CTA
  // shape's time of that instance is kept after the candidates' times.)
  if (clusters && ent.shape.threads > 0) {
    const float t1 = time_shape(ent.shape, 1);
    if (cand.size() < (size_t)kMaxCand) ent.ms[cand.size()] = t1;
    for (size_t c = 0; c < cand.size() && c < (size_t)kMaxCand; c++) {
      if (cand[c].csize == 1) continue;
      const float tc = time_shape(cand[c], 1);
      if (tc <= 0) continue;
      ent.ms[c] = tc;
      if (t1 > 0 && t1 >= 0.5 * cand[c].csize * tc && cand[c].csize > ent.shape.csize) ent.shape = cand[c];
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  dfree(xcopy);
  dfree(st);
  dfree(dd);
  dfree(counter);
  if (ent.shape.threads == 0) throw ApiError{MINIM_GPU_ERR_CUDA, "batch kernel does not fit on an SM"};
  g_tune.push_back(ent);
  tune_save(ent);
}

// The launch shape of every instance: the caller's thread count (one CTA per
// instance), else the tuned (or, with tuning off, the rule's) shape of its
// key.  Keys not yet tuned are measured on their fresh instances.
std::vector<Shape> batch_shapes(const std::vector<InstDesc>& descs, const std::vector<int>& kks,
                                const std::vector<char>& fresh, Shape force) {
  const int n = (int)descs.size();
  std::vector<Shape> sh(n, force);
  if (force.threads > 0) return sh;
  const bool tune = tune_enabled();
  if (tune) tune_load();
  std::vector<TuneKey> keys(n);
  for (int i = 0; i < n; i++) keys[i] = tune_key(kks[i], descs[i]);
  if (tune) {
    for (int i = 0; i < n; i++) {
      if (tune_find(keys[i]) || !fresh[i]) continue;
      // every fresh instance of this key, largest first, at most two per SM
      std::vector<int> idx;
      for (int j = i; j < n; j++)
        if (fresh[j] && keys[j] == keys[i]) idx.push_back(j);
      std::stable_sort(idx.begin(), idx.end(),
                       [&](int a, int b) { return cost_of(descs[a], kks[a]) > cost_of(descs[b], kks[b]); });
      if ((int)idx.size() > 2 * need_dev().nsm) idx.resize(2 * need_dev().nsm);
      std::vector<InstDesc> sample;
      for (int j : idx) sample.push_back(descs[j]);
      tune_measure(keys[i], sample);
    }
  }
  for (int i = 0; i < n; i++) {
    const TuneEntry* e = tune ? tune_find(keys[i]) : nullptr;
    sh[i] = e ? e->shape : rule_shape(kks[i], descs[i]);
  }
  return sh;
}

// Runs the given instances with the batch kernels: one launch per (kernel
// kind, shape) group, the groups concurrently on their own streams.
// descs[i].st must point into d_st; fresh[i] marks instances not yet started
// (the autotuner may run trial slices on copies of those).  Returns when all
// launches are done.
void run_batch(std::vector<InstDesc>& descs, const std::vector<int>& kks, MinScalars* d_st,
               const std::vector<MinScalars>& st_init, int slice, Shape force, const std::vector<char>& fresh) {
  Dev& D = need_dev();
  const int n = (int)descs.size();
  if (n == 0) return;
  g_tune_ms = 0;
  const std::vector<Shape> shp = batch_shapes(descs, kks, fresh, force);
  if (!st_init.empty())
    CK(cudaMemcpyAsync(d_st, st_init.data(), n * sizeof(MinScalars), cudaMemcpyHostToDevice, D.s));
  // group by kernel kind and shape, largest first within a group (LPT)
  std::vector<int> order(n);
  for (int i = 0; i < n; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    if (kks[a] != kks[b]) return kks[a] < kks[b];
    if (shp[a].csize != shp[b].csize) return shp[a].csize > shp[b].csize;
    if (shp[a].threads != shp[b].threads) return shp[a].threads < shp[b].threads;
    return cost_of(descs[a], kks[a]) > cost_of(descs[b], kks[b]);
  });
  std::vector<InstDesc> sorted(n);
  for (int i = 0; i < n; i++) sorted[i] = descs[order[i]];
  // Every group's launch configuration first: the occupancy query loads a
  // kernel that has not run yet in this process, and loading one while
  // another kernel runs waits for it (lazy module loading), which would
  // serialise the groups' launches.
  struct Launch {
    int kk, i0, i1, slots;
    Shape sh;
    size_t smem;
  };
  std::vector<Launch> launches;
  for (int i0 = 0; i0 < n;) {
    const int kk = kks[order[i0]];
    const Shape sh = shp[order[i0]];
    int i1 = i0;
    while (i1 < n && kks[order[i1]] == kk && shp[order[i1]] == sh) i1++;
    const size_t smem = group_smem(kk, sorted.data() + i0, i1 - i0, sh.threads);
    const int slots = shape_slots(kk, sh, smem);
    if (slots < 1) throw ApiError{MINIM_GPU_ERR_CUDA, "batch kernel does not fit on an SM"};
    launches.push_back({kk, i0, i1, slots, sh, smem});
    i0 = i1;
  }
  InstDesc* d_descs = (InstDesc*)dalloc(n * sizeof(InstDesc));
  int* d_counters = (int*)dalloc(launches.size() * sizeof(int));
  CK(cudaMemcpyAsync(d_descs, sorted.data(), n * sizeof(InstDesc), cudaMemcpyHostToDevice, D.s));
  CK(cudaMemsetAsync(d_counters, 0, launches.size() * sizeof(int), D.s));
  cudaEvent_t ready, t_end;
  CK(cudaEventCreate(&ready));
  CK(cudaEventCreate(&t_end));
  CK(cudaEventRecord(ready, D.s));
  std::vector<cudaEvent_t> done;
  for (size_t g = 0; g < launches.size(); g++) {
    const Launch& L = launches[g];
    cudaStream_t ks = D.ks[g % 8];
    CK(cudaStreamWaitEvent(ks, ready, 0));
    launch_shape(L.kk, L.sh, d_descs + L.i0, L.i1 - L.i0, d_counters + g, slice, L.slots, L.smem, ks);
    cudaEvent_t ev;
    CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    CK(cudaEventRecord(ev, ks));
    done.push_back(ev);
  }
  for (auto ev : done) {
    CK(cudaStreamWaitEvent(D.s, ev, 0));
    cudaEventDestroy(ev);
  }
  CK(cudaEventRecord(t_end, D.s));
  CK(cudaEventSynchronize(t_end));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, ready, t_end));
  g_stats.kernel_ms = ms;
  g_stats.launches = (int64_t)done.size();
  g_stats.tune_ms = g_tune_ms;
  cudaEventDestroy(ready);
  cudaEventDestroy(t_end);
  dfree(d_descs);
  dfree(d_counters);
}

}  // namespace

// ---------------------------------------------------------------------------
// Server (continuous batching)
// ---------------------------------------------------------------------------
namespace {
struct Request {
  uint64_t id = 0;
  minim_gpu_instance_s* inst = nullptr;
  minim_gpu_minimiser_params mp{};
  std::vector<double> sched;  // Anneal schedule, copied at submit
  double tol = 0;
  int state = 0;  // 0 queued, 1 resident, 2 done
  int slot = -1;
  void* ws = nullptr;
  size_t bytes = 0;
  double t_submit = 0, t_done = 0;
  minim_gpu_result res{};
  bool polled = false;
};
}  // namespace

struct minim_gpu_server_s {
  minim_gpu_server_config cfg{};
  uint64_t next_id = 1;
  std::unordered_map<uint64_t, Request> reqs;
  std::deque<uint64_t> queue;
  std::vector<uint64_t> slots;    // slot -> request id (0 = free)
  std::vector<uint64_t> done;     // finished, not yet polled
  size_t bytes_in_use = 0;
  MinScalars* d_st = nullptr;     // one per slot
  std::vector<InstDesc> descs;    // per slot (valid where resident)
  ~minim_gpu_server_s() {
    for (auto& kv : reqs) {
      dfree(kv.second.ws);
      delete kv.second.inst;
    }
    dfree(d_st);
  }
};

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

int minim_gpu_abi_version(void) { return MINIM_GPU_ABI_VERSION; }

// Sets the calling thread's last-error message (for entry points defined in
// other translation units).
void mg_set_last_error(const char* msg) { g_err = msg ? msg : ""; }

int minim_gpu_last_error(char* buf, size_t len) {
  if (buf && len) {
    std::strncpy(buf, g_err.c_str(), len - 1);
    buf[len - 1] = 0;
  }
  return (int)g_err.size();
}

int64_t minim_gpu_launch_count(void) { return g_launches.load(); }

int minim_gpu_last_run_stats(minim_gpu_run_stats* out) {
  return guarded([&] { *out = g_stats; });
}

void minim_gpu_default_minimiser(int method, minim_gpu_minimiser_params* p) {
  std::memset(p, 0, sizeof *p);
  p->method = method;
  p->linesearch = MINIM_LS_BACKTRACKING;
  p->max_iter = 100000;
  p->tol = -1;
  p->m = 5;
  p->max_step = 0;
  p->init_step = 1;
  p->dt_max = 0;
  p->alpha = 0.1;
  p->precision = MINIM_PREC_MIXED;
  p->temp_init = 1;
  p->displacement = 0.1;
  p->cooling_rate = 1;
}

void minim_gpu_default_pf(minim_gpu_pf_params* p) {
  std::memset(p, 0, sizeof *p);
  p->grid[0] = p->grid[1] = p->grid[2] = 1;
  p->nfluid = 1;
  p->resolution = 1;
  p->density_constraint = MINIM_PF_DENSITY_HARD;
  p->density_const = 1;
  p->vol_const = 0.01;
}

void minim_gpu_default_bah(minim_gpu_bah_params* p) {
  std::memset(p, 0, sizeof *p);
  p->bond_stride = 2;
  p->hinge_stride = 4;
  p->modulus = 1;
  p->poisson_ratio = 0.3;
  p->wall_epsilon = 1e-12;
  p->wall_sigma = 1e-5;
}

int minim_gpu_instance_create(int kind, const void* params, const double* x0, size_t ndof,
                              minim_gpu_handle* out) {
  return guarded([&] {
    if (!out) throw ApiError{MINIM_GPU_ERR_INVALID, "null output handle"};
    *out = create_instance(kind, params, x0, ndof);
  });
}

int minim_gpu_instance_destroy(minim_gpu_handle h) {
  return guarded([&] { delete h; });
}

int minim_gpu_instance_ndof(minim_gpu_handle h, size_t* n) {
  return guarded([&] { *n = h->n; });
}

int minim_gpu_instance_default_tol(minim_gpu_handle h, double* tol) {
  return guarded([&] { *tol = h->default_tol; });
}

int minim_gpu_instance_set_coords(minim_gpu_handle h, const double* x) {
  return guarded([&] {
    CK(cudaMemcpyAsync(h->d.xres, x, h->n * sizeof(double), cudaMemcpyHostToDevice, need_dev().s));
    CK(cudaStreamSynchronize(dev().s));
  });
}

int minim_gpu_instance_get_coords(minim_gpu_handle h, double* x) {
  return guarded([&] {
    CK(cudaMemcpyAsync(x, h->d.xres, h->n * sizeof(double), cudaMemcpyDeviceToHost, need_dev().s));
    CK(cudaStreamSynchronize(dev().s));
  });
}

int minim_gpu_instance_set_fixed(minim_gpu_handle h, const int* idof, size_t n) {
  return guarded([&] {
    std::vector<unsigned char> f(h->n, 0);
    for (size_t i = 0; i < n; i++) {
      if (idof[i] < 0 || (size_t)idof[i] >= h->n) throw ApiError{MINIM_GPU_ERR_INVALID, "fixed dof out of range"};
      f[idof[i]] = 1;
    }
    h->fixed = n ? f : std::vector<unsigned char>();
    h->d.fixed = h->own_upload(h->fixed);
    if (h->kind == MINIM_GPU_BAH) upload_bah_arrays(h);
    CK(cudaStreamSynchronize(dev().s));
  });
}

int minim_gpu_energy_gradient(minim_gpu_handle h, const double* x, double* e, double* g) {
  return guarded([&] { do_eval(h, x, e, g); });
}

int minim_gpu_eval_kernel(minim_gpu_handle h, int path, const double* x, const double* p, double t, double* e,
                          double* g, double* xt) {
  return guarded([&] {
    if (!h) throw ApiError{MINIM_GPU_ERR_INVALID, "null handle"};
    do_eval_kernel(h, path, x, p, t, e, g, xt);
  });
}

int minim_gpu_apply_constraints(minim_gpu_handle h, double* v) {
  return guarded([&] {
    Dev& D = need_dev();
    ensure_grid(h);
    CK(cudaMemcpyAsync(h->d_tmp, v, h->n * sizeof(double), cudaMemcpyHostToDevice, D.s));
    EvalIO io{};
    io.v = h->d_tmp;
    CK(cudaMemcpyAsync(h->d_desc, &h->d, sizeof(InstDesc), cudaMemcpyHostToDevice, D.s));
    CK(cudaMemcpyAsync(h->d_io, &io, sizeof io, cudaMemcpyHostToDevice, D.s));
    launch_grid(h, OP_CONSTRAIN, 0);
    CK(cudaMemcpyAsync(v, h->d_tmp, h->n * sizeof(double), cudaMemcpyDeviceToHost, D.s));
    CK(cudaStreamSynchronize(D.s));
  });
}

int minim_gpu_minimise(minim_gpu_handle h, const minim_gpu_minimiser_params* mp, minim_gpu_result* res) {
  return guarded([&] {
    if (!mp) throw ApiError{MINIM_GPU_ERR_INVALID, "null minimiser parameters"};
    do_minimise(h, *mp, res);
  });
}

int minim_gpu_batch_create(minim_gpu_batch* out) {
  return guarded([&] { *out = new minim_gpu_batch_s(); });
}

int minim_gpu_batch_add(minim_gpu_batch b, minim_gpu_handle h, const minim_gpu_minimiser_params* mp) {
  return guarded([&] {
    if (!b || !h || !mp) throw ApiError{MINIM_GPU_ERR_INVALID, "null argument"};
    check_mp(*mp);
    b->inst.push_back(h);
    b->mp.push_back(*mp);
    b->sched.push_back(sched_of(*mp));
  });
}

namespace {
void batch_run_shape(minim_gpu_batch b, Shape force, minim_gpu_result* results) {
  {
    Dev& D = need_dev();
    const int n = (int)b->inst.size();
    if (n == 0) return;
    std::vector<WsLayout> L(n);
    std::vector<size_t> off(n);
    size_t total = 0;
    for (int i = 0; i < n; i++) {
      L[i] = ws_layout(b->inst[i]->n, b->mp[i]);
      off[i] = total;
      total += L[i].total;
    }
    char* arena = (char*)dalloc(total);
    MinScalars* d_st = (MinScalars*)dalloc(n * sizeof(MinScalars));
    std::vector<InstDesc> descs(n);
    std::vector<int> kks(n);
    for (int i = 0; i < n; i++) {
      InstDesc d = b->inst[i]->d;
      ws_apply(d, arena + off[i], L[i]);
      const double tol = b->mp[i].tol >= 0 ? b->mp[i].tol : b->inst[i]->default_tol;
      d.mp = to_mp(b->mp[i], tol);
      ws_sched(d, arena + off[i], L[i], b->sched[i], D.s);
      d.st = d_st + i;
      descs[i] = d;
      kks[i] = b->inst[i]->kk;
    }
    std::vector<MinScalars> st(n, fresh_scalars());
    const double t0 = now_ms();
    run_batch(descs, kks, d_st, st, 0x7fffffff, force, std::vector<char>(n, 1));
    CK(cudaMemcpyAsync(st.data(), d_st, n * sizeof(MinScalars), cudaMemcpyDeviceToHost, D.s));
    CK(cudaStreamSynchronize(D.s));
    g_stats.wall_ms = now_ms() - t0;
    g_stats.abytes = g_stats.pairs32 = g_stats.pairs64 = 0;
    g_stats.iterations = 0;
    g_stats.fp64_iterations = 0;
    for (auto& k : g_stats.switches) k = 0;
    for (auto& k : g_stats.phase_ms) k = 0;
    for (auto& s : st) {
      for (int k = 0; k < 3; k++) g_stats.phase_ms[k] += s.tphase[k] * 1e-6;
      g_stats.fp64_iterations += s.fp64_iters;
      if (s.switch_reason > 0 && s.switch_reason < 4) g_stats.switches[s.switch_reason]++;
      g_stats.abytes += s.abytes;
      g_stats.pairs32 += s.pairs32;
      g_stats.pairs64 += s.pairs64;
      g_stats.iterations += s.iter + (s.status == ST_CONVERGED ? 1 : 0);
    }
    dfree(arena);
    dfree(d_st);
    if (results)
      for (int i = 0; i < n; i++) fill_result(&results[i], st[i], b->inst[i]->n);
  }
}
}  // namespace

int minim_gpu_lj_cutoff_pairs(minim_gpu_handle h, const double* x, int cap, int* pairs, int* npairs) {
  return guarded([&] {
    if (!h || !x || cap < 0 || (cap > 0 && !pairs) || !npairs)
      throw ApiError{MINIM_GPU_ERR_INVALID, "minim_gpu_lj_cutoff_pairs: invalid arguments"};
    if (h->kk != K_LJ || !(h->d.lj.rc2 > 0))
      throw ApiError{MINIM_GPU_ERR_INVALID, "minim_gpu_lj_cutoff_pairs: not a Lennard-Jones instance with a cutoff"};
    Dev& D = need_dev();
    ensure_grid(h);
    const size_t n = h->n;
    const size_t xb = align256(n * sizeof(float));
    char* buf = (char*)dalloc(xb + 256 + (size_t)std::max(cap, 1) * sizeof(int2));
    float* x32 = (float*)buf;
    int* cnt = (int*)(buf + xb);
    int2* out = (int2*)(buf + xb + 256);
    try {
      CK(cudaMemcpyAsync(h->d_tmp, x, n * sizeof(double), cudaMemcpyHostToDevice, D.s));
      CK((cudaError_t)mg_convert(h->d_tmp, x32, n, 1, D.s));
      CK(cudaMemsetAsync(cnt, 0, sizeof(int), D.s));
      EvalIO io{};
      io.x32 = x32;
      io.pairs = out;
      io.npairs = cnt;
      io.cap = cap;
      CK(cudaMemcpyAsync(h->d_desc, &h->d, sizeof(InstDesc), cudaMemcpyHostToDevice, D.s));
      CK(cudaMemcpyAsync(h->d_io, &io, sizeof io, cudaMemcpyHostToDevice, D.s));
      launch_grid(h, OP_LJ_PAIRS, 0);
      int total = 0;
      CK(cudaMemcpyAsync(&total, cnt, sizeof(int), cudaMemcpyDeviceToHost, D.s));
      CK(cudaStreamSynchronize(D.s));
      if (grid_error(h)) throw ApiError{MINIM_GPU_ERR_RUNTIME, "device barrier timed out"};
      const int k = std::min(total, cap);
      std::vector<int2> hp(k);
      if (k) CK(cudaMemcpyAsync(hp.data(), out, k * sizeof(int2), cudaMemcpyDeviceToHost, D.s));
      CK(cudaStreamSynchronize(D.s));
      std::sort(hp.begin(), hp.end(),
                [](const int2& a, const int2& b) { return a.x != b.x ? a.x < b.x : a.y < b.y; });
      for (int i = 0; i < k; i++) {
        pairs[2 * i] = hp[i].x;
        pairs[2 * i + 1] = hp[i].y;
      }
      *npairs = total;
    } catch (...) {
      cudaStreamSynchronize(D.s);
      dfree(buf);
      throw;
    }
    dfree(buf);
  });
}

int minim_gpu_wait_probe(int limit_ms, int* timed_out, double* elapsed_ms) {
  return guarded([&] {
    Dev& D = need_dev();
    if (limit_ms < 1 || limit_ms > 60000) throw ApiError{MINIM_GPU_ERR_INVALID, "limit_ms must be 1 .. 60000"};
    GridSyncState* bar = (GridSyncState*)dalloc(sizeof(GridSyncState));
    GridSyncState h{};
    h.limit_ms = (unsigned)limit_ms;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaMemcpyAsync(bar, &h, sizeof h, cudaMemcpyHostToDevice, D.s));
    CK(cudaEventRecord(e0, D.s));
    CK((cudaError_t)mg_wait_probe(bar, D.s));
    g_launches++;
    CK(cudaEventRecord(e1, D.s));
    CK(cudaMemcpyAsync(&h, bar, sizeof h, cudaMemcpyDeviceToHost, D.s));
    CK(cudaStreamSynchronize(D.s));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    dfree(bar);
    if (timed_out) *timed_out = h.err != 0;
    if (elapsed_ms) *elapsed_ms = ms;
  });
}

int minim_gpu_batch_run(minim_gpu_batch b, int threads, minim_gpu_result* results) {
  return guarded([&] { batch_run_shape(b, Shape{threads, 1}, results); });
}

int minim_gpu_batch_run_shape(minim_gpu_batch b, int threads_per_cta, int ctas, minim_gpu_result* results) {
  return guarded([&] {
    if (threads_per_cta < 32 || threads_per_cta % 32 || threads_per_cta > 512 || ctas < 1 || ctas > 8)
      throw ApiError{MINIM_GPU_ERR_INVALID, "minim_gpu_batch_run_shape: threads_per_cta 32..512 (a multiple of 32), ctas 1..8"};
    for (auto* h : b->inst)
      if (h->kk == K_LJ && threads_per_cta > 256)
        throw ApiError{MINIM_GPU_ERR_INVALID, "minim_gpu_batch_run_shape: Lennard-Jones takes at most 256 threads per CTA"};
    batch_run_shape(b, Shape{threads_per_cta, ctas}, results);
  });
}

int minim_gpu_tune_table(int cap, int* rows, double* ms, int* n) {
  return guarded([&] {
    const int k = (int)g_tune.size();
    if (n) *n = k;
    for (int i = 0; i < k && i < cap; i++) {
      const TuneEntry& e = g_tune[i];
      const int kind = e.key.kk == K_LJ ? MINIM_GPU_LJ : (e.key.kk == K_BAH ? MINIM_GPU_BAH : MINIM_GPU_PF);
      const std::vector<Shape> cs = shape_candidates(e.key.kk, e.key.bucket);
      bool cl = false;
      for (const Shape& c : cs) cl |= c.csize > 1;
      // with cluster candidates, the one-CTA shape's time of the largest
      // instance follows the candidates' times
      const int cand = (int)cs.size() + (cl ? 1 : 0);
      const int row[8] = {kind, e.key.bucket, e.key.method, e.key.prec, e.shape.threads, e.shape.csize,
                          e.from_file ? 0 : 1, e.from_file ? 0 : cand};
      if (rows) std::memcpy(rows + 8 * i, row, sizeof row);
      if (ms)
        for (int c = 0; c < kMaxCand; c++) ms[kMaxCand * i + c] = e.ms[c];
    }
  });
}

int minim_gpu_batch_destroy(minim_gpu_batch b) {
  return guarded([&] { delete b; });
}

int minim_gpu_server_create(const minim_gpu_server_config* cfg, minim_gpu_server* out) {
  return guarded([&] {
    need_dev();
    auto s = new minim_gpu_server_s();
    if (cfg) s->cfg = *cfg;
    if (s->cfg.max_slots <= 0) s->cfg.max_slots = 4096;
    if (s->cfg.slice_iters <= 0) s->cfg.slice_iters = 64;
    if (s->cfg.max_bytes == 0) {
      size_t fr = 0, tot = 0;
      cudaMemGetInfo(&fr, &tot);
      s->cfg.max_bytes = fr / 2;
    }
    s->slots.assign(s->cfg.max_slots, 0);
    s->descs.resize(s->cfg.max_slots);
    s->d_st = (MinScalars*)dalloc(s->cfg.max_slots * sizeof(MinScalars));
    *out = s;
  });
}

int minim_gpu_server_submit(minim_gpu_server s, int kind, const void* params, const double* x0, size_t ndof,
                            const minim_gpu_minimiser_params* mp, uint64_t* request_id) {
  return guarded([&] {
    if (!mp) throw ApiError{MINIM_GPU_ERR_INVALID, "null minimiser parameters"};
    check_mp(*mp);
    Request r;
    r.id = s->next_id++;
    r.inst = create_instance(kind, params, x0, ndof);
    r.mp = *mp;
    r.sched = sched_of(*mp);
    r.tol = mp->tol >= 0 ? mp->tol : r.inst->default_tol;
    r.bytes = ws_layout(ndof, *mp).total;
    r.t_submit = now_ms();
    if (r.bytes + r.inst->pot_bytes > s->cfg.max_bytes) {
      r.state = 2;
      r.res.status = MINIM_RES_REJECTED;
      r.t_done = r.t_submit;
      s->done.push_back(r.id);
    } else {
      s->queue.push_back(r.id);
    }
    if (request_id) *request_id = r.id;
    s->reqs.emplace(r.id, r);
  });
}

int minim_gpu_server_step(minim_gpu_server s, int* n_resident, int* n_queued) {
  return guarded([&] {
    Dev& D = need_dev();
    // admit
    std::vector<int> admitted;
    int free_slot = 0;
    while (!s->queue.empty()) {
      Request& r = s->reqs[s->queue.front()];
      if (r.state != 0) {  // cancelled while queued
        s->queue.pop_front();
        continue;
      }
      if (s->bytes_in_use + r.bytes > s->cfg.max_bytes) break;
      while (free_slot < s->cfg.max_slots && s->slots[free_slot]) free_slot++;
      if (free_slot >= s->cfg.max_slots) break;
      s->queue.pop_front();
      WsLayout L = ws_layout(r.inst->n, r.mp);
      r.ws = dalloc(L.total);
      r.slot = free_slot;
      r.state = 1;
      s->slots[free_slot] = r.id;
      s->bytes_in_use += r.bytes;
      InstDesc d = r.inst->d;
      ws_apply(d, (char*)r.ws, L);
      d.mp = to_mp(r.mp, r.tol);
      ws_sched(d, (char*)r.ws, L, r.sched, D.s);
      d.st = s->d_st + free_slot;
      s->descs[free_slot] = d;
      admitted.push_back(free_slot);
    }
    for (int slot : admitted) {
      MinScalars st = fresh_scalars();
      CK(cudaMemcpyAsync(s->d_st + slot, &st, sizeof st, cudaMemcpyHostToDevice, D.s));
    }
    // one slice on every resident instance
    std::vector<InstDesc> descs;
    std::vector<int> kks, slot_of;
    std::vector<char> fresh;
    for (int k = 0; k < s->cfg.max_slots; k++) {
      if (!s->slots[k]) continue;
      descs.push_back(s->descs[k]);
      kks.push_back(s->reqs[s->slots[k]].inst->kk);
      slot_of.push_back(k);
      fresh.push_back(std::find(admitted.begin(), admitted.end(), k) != admitted.end());
    }
    if (!descs.empty()) {
      run_batch(descs, kks, s->d_st, {}, s->cfg.slice_iters, Shape{s->cfg.threads_per_cta, 1}, fresh);
      std::vector<MinScalars> st(s->cfg.max_slots);
      CK(cudaMemcpyAsync(st.data(), s->d_st, s->cfg.max_slots * sizeof(MinScalars), cudaMemcpyDeviceToHost, D.s));
      CK(cudaStreamSynchronize(D.s));
      const double t = now_ms();
      for (int k : slot_of) {
        if (st[k].status == ST_RUNNING) continue;
        Request& r = s->reqs[s->slots[k]];
        fill_result(&r.res, st[k], r.inst->n);
        r.t_done = t;
        r.res.latency_ms = t - r.t_submit;
        r.state = 2;
        dfree(r.ws);
        r.ws = nullptr;
        s->bytes_in_use -= r.bytes;
        s->slots[k] = 0;
        r.slot = -1;
        s->done.push_back(r.id);
      }
    }
    int res_n = 0;
    for (auto id : s->slots) res_n += id != 0;
    if (n_resident) *n_resident = res_n;
    if (n_queued) *n_queued = (int)s->queue.size();
  });
}

int minim_gpu_server_poll(minim_gpu_server s, uint64_t* ids, minim_gpu_result* res, int max, int* n_done) {
  return guarded([&] {
    int k = 0;
    while (k < max && !s->done.empty()) {
      const uint64_t id = s->done.front();
      s->done.erase(s->done.begin());
      Request& r = s->reqs[id];
      r.polled = true;
      if (ids) ids[k] = id;
      if (res) res[k] = r.res;
      k++;
    }
    if (n_done) *n_done = k;
  });
}

int minim_gpu_server_take(minim_gpu_server s, uint64_t id, double* x, size_t ndof) {
  return guarded([&] {
    auto it = s->reqs.find(id);
    if (it == s->reqs.end() || it->second.state != 2) throw ApiError{MINIM_GPU_ERR_BUSY, "request not finished"};
    Request& r = it->second;
    if (x) {
      if (ndof != r.inst->n) throw ApiError{MINIM_GPU_ERR_INVALID, "wrong coordinate count"};
      CK(cudaMemcpyAsync(x, r.inst->d.xres, ndof * sizeof(double), cudaMemcpyDeviceToHost, dev().s));
      CK(cudaStreamSynchronize(dev().s));
    }
    delete r.inst;
    s->reqs.erase(it);
  });
}

int minim_gpu_server_cancel(minim_gpu_server s, uint64_t id) {
  return guarded([&] {
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) throw ApiError{MINIM_GPU_ERR_BUSY, "unknown request"};
    Request& r = it->second;
    if (r.state == 2) return;
    if (r.state == 1) {
      s->slots[r.slot] = 0;
      dfree(r.ws);
      r.ws = nullptr;
      s->bytes_in_use -= r.bytes;
      r.slot = -1;
    }
    r.state = 2;
    r.res.status = MINIM_RES_CANCELLED;
    r.t_done = now_ms();
    r.res.latency_ms = r.t_done - r.t_submit;
    s->done.push_back(id);
  });
}

int minim_gpu_server_destroy(minim_gpu_server s) {
  return guarded([&] { delete s; });
}

// ---- host-only set-up introspection (no GPU needed) -------------------------
int minim_gpu_bah_elements(const minim_gpu_bah_params* q, const double* x0, size_t ndof, int cap, int* nbar,
                           int* bars, double* bar_par, int* nhinge, int* hinges, double* hinge_par) {
  return guarded([&] {
    BahHost B = setup_bah(*q, x0, ndof);
    const int nb = (int)(B.bars.size() / 2), nh = (int)(B.hinges.size() / 4);
    *nbar = nb;
    *nhinge = nh;
    if (nb <= cap) {
      std::memcpy(bars, B.bars.data(), B.bars.size() * sizeof(int));
      std::memcpy(bar_par, B.bpar.data(), B.bpar.size() * sizeof(double));
    }
    if (nh <= cap) {
      std::memcpy(hinges, B.hinges.data(), B.hinges.size() * sizeof(int));
      std::memcpy(hinge_par, B.hpar.data(), B.hpar.size() * sizeof(double));
    }
  });
}

int minim_gpu_bah_colouring(const minim_gpu_bah_params* q, const double* x0, size_t ndof, int* nbar_colors,
                            int* nhinge_colors, int* valid) {
  return guarded([&] {
    BahHost B = setup_bah(*q, x0, ndof);
    BahDevArrays A = bah_arrays(B, {});
    *nbar_colors = (int)A.bar_off.size() - 1;
    *nhinge_colors = (int)A.hinge_off.size() - 1;
    // every colour must be vertex-disjoint
    int ok = 1;
    std::vector<int> seen(B.nvert, -1);
    for (int c = 0; c < *nbar_colors && ok; c++)
      for (int e = A.bar_off[c]; e < A.bar_off[c + 1] && ok; e++)
        for (int v : {A.bars[e].x, A.bars[e].y}) {
          if (seen[v] == c) ok = 0;
          seen[v] = c;
        }
    std::fill(seen.begin(), seen.end(), -1);
    for (int c = 0; c < *nhinge_colors && ok; c++)
      for (int e = A.hinge_off[c]; e < A.hinge_off[c + 1] && ok; e++)
        for (int v : {A.hinges[e].x, A.hinges[e].y, A.hinges[e].z, A.hinges[e].w}) {
          if (seen[v] == c) ok = 0;
          seen[v] = c;
        }
    *valid = ok;
  });
}

int minim_gpu_instance_bah_arrays(minim_gpu_handle h, int cap, int* nbar, int* bars, double* bar_par,
                                  int* nbar_colors, int* bar_off, int* nhinge, int* hinges, double* hinge_par,
                                  int* nhinge_colors, int* hinge_off, int* on_device) {
  return guarded([&] {
    if (!h || h->kind != MINIM_GPU_BAH) throw ApiError{MINIM_GPU_ERR_INVALID, "not a BarAndHinge instance"};
    const PotBAH& P = h->d.bah;
    *nbar = P.nbar;
    *nhinge = P.nhinge;
    *nbar_colors = P.nbar_colors;
    *nhinge_colors = P.nhinge_colors;
    *on_device = h->bah_dev ? 1 : 0;
    if (P.nbar > cap || P.nhinge > cap || P.nbar_colors > 64 || P.nhinge_colors > 64) return;
    Dev& D = need_dev();
    std::vector<int2> b2(P.nbar);
    std::vector<int4> h4(P.nhinge);
    std::vector<double2> bp(P.nbar), hp(P.nhinge);
    if (P.nbar) {
      CK(cudaMemcpyAsync(b2.data(), P.bars, b2.size() * sizeof(int2), cudaMemcpyDeviceToHost, D.s));
      CK(cudaMemcpyAsync(bp.data(), P.bar_par, bp.size() * sizeof(double2), cudaMemcpyDeviceToHost, D.s));
    }
    if (P.nhinge) {
      CK(cudaMemcpyAsync(h4.data(), P.hinges, h4.size() * sizeof(int4), cudaMemcpyDeviceToHost, D.s));
      CK(cudaMemcpyAsync(hp.data(), P.hinge_par, hp.size() * sizeof(double2), cudaMemcpyDeviceToHost, D.s));
    }
    CK(cudaMemcpyAsync(bar_off, P.bar_color_off, (P.nbar_colors + 1) * sizeof(int), cudaMemcpyDeviceToHost, D.s));
    CK(cudaMemcpyAsync(hinge_off, P.hinge_color_off, (P.nhinge_colors + 1) * sizeof(int), cudaMemcpyDeviceToHost,
                       D.s));
    CK(cudaStreamSynchronize(D.s));
    for (int i = 0; i < P.nbar; i++) {
      bars[2 * i] = b2[i].x;
      bars[2 * i + 1] = b2[i].y;
      bar_par[2 * i] = bp[i].x;
      bar_par[2 * i + 1] = bp[i].y;
    }
    for (int i = 0; i < P.nhinge; i++) {
      hinges[4 * i] = h4[i].x;
      hinges[4 * i + 1] = h4[i].y;
      hinges[4 * i + 2] = h4[i].z;
      hinges[4 * i + 3] = h4[i].w;
      hinge_par[2 * i] = hp[i].x;
      hinge_par[2 * i + 1] = hp[i].y;
    }
  });
}

int minim_gpu_pf_setup(int kind, const minim_gpu_pf_params* q, const double* x0, size_t ndof, double* kappa,
                       double* kappaP, int* nk, double* node_vol, double* surface_area, int* kernel_variant) {
  return guarded([&] {
    if (kind != MINIM_GPU_PF && kind != MINIM_GPU_PFU) throw ApiError{MINIM_GPU_ERR_INVALID, "not a phase-field kind"};
    PfHost H = setup_pf(*q, x0, ndof, kind == MINIM_GPU_PFU);
    *nk = (int)H.kappa.size();
    if (kappa) std::memcpy(kappa, H.kappa.data(), H.kappa.size() * sizeof(double));
    if (kappaP) std::memcpy(kappaP, H.kappaP.data(), H.kappaP.size() * sizeof(double));
    // empty per-node arrays: no solid, every node bulk
    const size_t ng = (size_t)H.pot.ngrid;
    const double r3 = std::pow(q->resolution, 3);
    if (node_vol) {
      if (H.node_vol.empty()) std::fill(node_vol, node_vol + ng, r3);
      else std::memcpy(node_vol, H.node_vol.data(), ng * sizeof(double));
    }
    if (surface_area) {
      if (H.surface_area.empty()) std::fill(surface_area, surface_area + ng, 0.0);
      else std::memcpy(surface_area, H.surface_area.data(), ng * sizeof(double));
    }
    if (kernel_variant) *kernel_variant = H.kernel_kind;
  });
}

}  // extern "C"
