// engine.cu -- the two persistent kernels and their launchers.
//
//   batch_kernel : one CTA per instance.  CTAs pull instance indices from a
//                  global counter (largest instances first, set by the host),
//                  run that instance's minimisation for up to `slice`
//                  iterations entirely on chip, store its state and pull the
//                  next.  No CTA ever waits on another.
//   grid_kernel  : one instance on the whole GPU (cooperative launch, bounded
//                  software grid barrier); also serves the FP64 energy /
//                  gradient and constraint calls of the C ABI.
#pragma once
#include "minimiser.cuh"

namespace mg {

// WR: rows of the wide-reduction scratch, one per warp of the block
template <int WR = 8>
struct SharedScalars {
  double red[(32 + 1) * MINIM_MAXRED];
  double wide[WR * MINIM_WIDE];
  double wout[MINIM_WIDE];
  double SY[MINIM_MAXM * MINIM_MAXM], YY[MINIM_MAXM * MINIM_MAXM];
  float coefS[MINIM_MAXM], coefY[MINIM_MAXM];
  long long boff[2 * MINIM_MAXM];
  double rho[MINIM_MAXM], sig[MINIM_MAXM], yy[MINIM_MAXM], alpha[MINIM_MAXM];
  int sidx[MINIM_MAXM], yidx[MINIM_MAXM];
  unsigned long long mbar[MINIM_NSTAGE], mbar_empty[MINIM_NSTAGE];
  int stage_err;
  int next, ok, last;
};

__device__ __forceinline__ void copy_desc(InstDesc* dst, const InstDesc* src) {
  const int nw = (int)(sizeof(InstDesc) / sizeof(int));
  const int* s = reinterpret_cast<const int*>(src);
  int* d = reinterpret_cast<int*>(dst);
  for (int i = threadIdx.x; i < nw; i += blockDim.x) d[i] = s[i];
}

template <class Team, int KIND, class SS>
__device__ void setup_runner(Runner<Team, KIND>& R, SS& S, const InstDesc& in) {
  R.n = in.ndof;
  R.rho = S.rho; R.sig = S.sig; R.yy = S.yy; R.alpha = S.alpha;
  R.sidx = S.sidx; R.yidx = S.yidx;
  R.SY = S.SY; R.YY = S.YY; R.wout = S.wout; R.coefS = S.coefS; R.coefY = S.coefY;
  R.boff = S.boff;
  R.mbar = S.mbar;
  R.mbar_empty = S.mbar_empty;
  R.stage_err = &S.stage_err;
  R.sq = 0u;
}

// The grid-sized kinds run 512-thread blocks (one per SM at 128 registers a
// thread); Lennard-Jones keeps up to 256 threads and MG_LJ_MINB or more
// blocks per SM (the register budget of its FP32 pair loops).
#ifndef MG_LJ_MINB
#define MG_LJ_MINB 2
#endif
template <int KIND>
__global__ void __launch_bounds__(KIND == K_LJ ? 256 : 512, KIND == K_LJ ? MG_LJ_MINB : 1)
batch_kernel(const InstDesc* __restrict__ insts, int ninst, int* counter, int slice, int lj_tile) {
  __shared__ SharedScalars<KIND == K_LJ ? 8 : 16> S;
  __shared__ __align__(16) InstDesc s_in;
  extern __shared__ __align__(16) unsigned char dyn[];
  for (;;) {
    if (threadIdx.x == 0) S.next = atomicAdd(counter, 1);
    __syncthreads();
    const int k = S.next;
    if (k >= ninst) break;
    copy_desc(&s_in, &insts[k]);
    __syncthreads();
    if (threadIdx.x == 0 && s_in.st->t_first == 0) s_in.st->t_first = globaltimer_ns();
    CtaTeam tm{S.red, S.wide};
    Runner<CtaTeam, KIND> R{tm, s_in, dyn, lj_tile};
    setup_runner(R, S, s_in);
    R.load(*s_in.st);
    R.run(slice);
    R.store(*s_in.st);
    if (threadIdx.x == 0) s_in.st->t_last = globaltimer_ns();
  }
}

// The batch path with one instance per thread-block cluster: the cluster's
// CTAs (on as many SMs) share the instance's every phase through the cluster
// team.  Rank 0 pulls instance indices from the counter and the others read
// the index from its shared memory; every CTA leaves the loop after the same
// cluster barrier, so no CTA exits while another may still read its shared
// memory.
template <int KIND>
__global__ void __launch_bounds__(KIND == K_LJ ? 256 : 512, 1)
cluster_batch_kernel(const InstDesc* __restrict__ insts, int ninst, int* counter, int slice, int lj_tile) {
  __shared__ SharedScalars<KIND == K_LJ ? 8 : 16> S;
  __shared__ __align__(16) InstDesc s_in;
  __shared__ double xch[2 * MINIM_WIDE];
  __shared__ int next;
  extern __shared__ __align__(16) unsigned char dyn[];
  auto cl = cooperative_groups::this_cluster();
  const bool lead = cl.block_rank() == 0;
  for (;;) {
    if (lead && threadIdx.x == 0) next = atomicAdd(counter, 1);
    cl.sync();
    const int k = *cl.map_shared_rank(&next, 0);
    // every CTA has read the index before the leader draws the next one
    cl.sync();
    if (k >= ninst) break;
    copy_desc(&s_in, &insts[k]);
    __syncthreads();
    if (lead && threadIdx.x == 0 && s_in.st->t_first == 0) s_in.st->t_first = globaltimer_ns();
    ClusterTeam tm{S.red, S.wide, xch, 0};
    Runner<ClusterTeam, KIND> R{tm, s_in, dyn, lj_tile};
    setup_runner(R, S, s_in);
    R.load(*s_in.st);
    R.run(slice);
    R.store(*s_in.st);
    if (lead && threadIdx.x == 0) s_in.st->t_last = globaltimer_ns();
  }
}

template <class Team, int KIND>
__device__ void eval_op(Runner<Team, KIND>& R, Team& tm, const InstDesc& in, const EvalIO& io) {
  CView<double> cv{io.x, nullptr, 0.0};
  StoreEmit64 em{io.g, in.fixed};
  const bool want_g = io.g != nullptr;
  const double ep = R.template pot_eval<double, false>(cv, nullptr, em, true, want_g);
  if constexpr (KIND == K_PF) {
    if (want_g && (in.pf.flags & PF_VOLUME)) {
      tm.sync();
      pf_volume_project<double>(tm, in.pf, io.g);
    }
  }
  double v[1] = {ep};
  tm.reduce(v);
  if (io.e && tm.block0() && threadIdx.x == 0) *io.e = v[0];
}

// One evaluation by a minimiser stage's potential kernels (the arithmetic
// and the reduction of grad_eval / energy_at) at x + t p, for checking them
// against an FP64 evaluation.
template <class Team, int KIND>
__device__ void eval_stage_op(Runner<Team, KIND>& R, Team& tm, const InstDesc& in, const EvalIO& io) {
  const bool want_g = io.g32 != nullptr;
  FusedEmit em{io.g32, nullptr, nullptr, nullptr, in.fixed};
  double ep;
  if (io.stage == 0) {
    CView<float> cv{io.x32, io.p, io.t32};
    ep = R.template pot_eval<float>(cv, nullptr, em, true, want_g);
  } else {
    CView<double> cv{io.x, io.p, io.t64};
    ep = R.template pot_eval<double>(cv, nullptr, em, true, want_g);
  }
  if constexpr (KIND == K_PF) {
    if (want_g && (in.pf.flags & PF_VOLUME)) {
      tm.sync();
      pf_volume_project<float>(tm, in.pf, io.g32);
    }
  }
  double v[1] = {ep};
  if (io.stage == 0) {
    float ps[1], pc[1];
    to_pair(ep, ps[0], pc[0]);
    tm.template reduce_pairs<1>(ps, pc, v);
  } else {
    tm.reduce(v);
  }
  if (io.e && tm.block0() && threadIdx.x == 0) *io.e = v[0];
}

// eval_stage_op on one CTA: the batch kernels' team (Lennard-Jones clusters
// take the symmetric tile path there)
template <int KIND>
__global__ void __launch_bounds__(KIND == K_LJ ? 256 : 512, KIND == K_LJ ? 2 : 1)
cta_eval_kernel(const InstDesc* __restrict__ inst, const EvalIO* io, int lj_tile) {
  __shared__ SharedScalars<KIND == K_LJ ? 8 : 16> S;
  __shared__ __align__(16) InstDesc s_in;
  extern __shared__ __align__(16) unsigned char dyn[];
  copy_desc(&s_in, inst);
  __syncthreads();
  CtaTeam tm{S.red, S.wide};
  Runner<CtaTeam, KIND> R{tm, s_in, dyn, lj_tile};
  setup_runner(R, S, s_in);
  eval_stage_op(R, tm, s_in, *io);
}

template <class Team, int KIND>
__device__ void constrain_op(Team& tm, const InstDesc& in, const EvalIO& io) {
  double* v = io.v;
  // PhaseFieldUnstructured::init replaces the constraint list, so fixed
  // degrees of freedom set on the state come after its own constraints
  bool fixed_last = false;
  if constexpr (KIND == K_PF) fixed_last = (in.pf.flags & PF_UNSTR) != 0;
  if (in.fixed && !fixed_last)
    for (int i = tm.tid(); i < in.ndof; i += tm.nthr())
      if (in.fixed[i]) v[i] = 0.0;
  if constexpr (KIND == K_PF) {
    if (in.pf.flags & (PF_FIXFLUID | PF_HARD)) {
      tm.sync();
      pf_local_constrain<double>(tm, in.pf, v);
    }
    if (in.pf.flags & PF_VOLUME) {
      tm.sync();
      pf_volume_project<double>(tm, in.pf, v);
    }
  }
  if (in.fixed && fixed_last) {
    tm.sync();
    for (int i = tm.tid(); i < in.ndof; i += tm.nthr())
      if (in.fixed[i]) v[i] = 0.0;
  }
}

template <int KIND>
__global__ void __launch_bounds__(256, 2)
grid_kernel(const InstDesc* __restrict__ inst, int op, const EvalIO* io, int slice,
            GridSyncState* bar, double* partials, int lj_tile) {
  __shared__ SharedScalars<> S;
  __shared__ __align__(16) InstDesc s_in;
  extern __shared__ __align__(16) unsigned char dyn[];
  copy_desc(&s_in, inst);
  if (threadIdx.x == 0) {
    S.ok = 1;
    for (int k = 0; k < MINIM_NSTAGE; k++) {
      mbar_init(&S.mbar[k], 1);
      mbar_init(&S.mbar_empty[k], (blockDim.x + 31) >> 5);
    }
    S.stage_err = 0;
    mbar_init_fence();
  }
  __syncthreads();
  GridTeam tm{S.red,
              S.wide, bar, partials, 0, &S.ok, 0u};
  Runner<GridTeam, KIND> R{tm, s_in, dyn, lj_tile};
  setup_runner(R, S, s_in);
  if (op == OP_MINIMISE) {
    R.load(*s_in.st);
    R.run(slice);
    R.store(*s_in.st);
  } else if (op == OP_EVAL) {
    eval_op(R, tm, s_in, *io);
  } else if (op == OP_EVAL_STAGE) {
    eval_stage_op(R, tm, s_in, *io);
  } else if (op == OP_LJ_PAIRS) {
    if constexpr (KIND == K_LJ) {
      CView<float> cv{io->x32, nullptr, 0.f};
      NoEmit ne;
      lj_cells_eval<float>(tm, s_in.lj, cv, (float*)nullptr, &ne, false, false, io->pairs, io->npairs, io->cap);
    }
  } else {
    constrain_op<GridTeam, KIND>(tm, s_in, *io);
  }
}

}  // namespace mg

// Instantiates the kernels for one potential kind and defines its launchers
// (mg_launch_batch_<name>, mg_launch_grid_<name>, occupancy queries).
#define MG_DEFINE_LAUNCHERS(KIND, NAME)                                                          \
  /* opts the grid kernel in to more than 48 KB of dynamic shared memory */                      \
  static void mg_grid_smem_##NAME(size_t smem) {                                                  \
    static size_t done = 0;                                                                       \
    if (smem > done) {                                                                            \
      cudaFuncSetAttribute((const void*)mg::grid_kernel<KIND>,                                    \
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);               \
      done = smem;                                                                                \
    }                                                                                             \
  }                                                                                               \
  static void mg_batch_smem_##NAME(size_t smem) {                                                 \
    static size_t done = 0;                                                                       \
    if (smem > done) {                                                                            \
      cudaFuncSetAttribute((const void*)mg::batch_kernel<KIND>,                                   \
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);               \
      done = smem;                                                                                \
    }                                                                                             \
  }                                                                                               \
  extern "C" int mg_launch_batch_##NAME(const mg::InstDesc* d_insts, int ninst, int* d_counter,   \
                                        int slice_iters, int threads, int blocks, size_t smem,    \
                                        void* stream) {                                           \
    mg_batch_smem_##NAME(smem);                                                                   \
    const int tile = (int)(smem / sizeof(mg::D4));                                                \
    mg::batch_kernel<KIND><<<blocks, threads, smem, (cudaStream_t)stream>>>(                     \
        d_insts, ninst, d_counter, slice_iters, tile);                                            \
    return (int)cudaGetLastError();                                                               \
  }                                                                                               \
  extern "C" int mg_launch_grid_##NAME(const mg::InstDesc* d_inst, int op, const mg::EvalIO* d_io, \
                                       int slice_iters, mg::GridSyncState* d_bar,                 \
                                       double* d_partials, int threads, int blocks, size_t smem,  \
                                       void* stream) {                                            \
    int tile = (int)(smem / sizeof(mg::D4));                                                      \
    mg_grid_smem_##NAME(smem);                                                                    \
    void* args[] = {(void*)&d_inst, (void*)&op,         (void*)&d_io, (void*)&slice_iters,        \
                    (void*)&d_bar,  (void*)&d_partials, (void*)&tile};                            \
    return (int)cudaLaunchCooperativeKernel((const void*)mg::grid_kernel<KIND>, dim3(blocks),     \
                                            dim3(threads), args, smem, (cudaStream_t)stream);     \
  }                                                                                               \
  extern "C" int mg_launch_cta_eval_##NAME(const mg::InstDesc* d_inst, const mg::EvalIO* d_io,     \
                                           int threads, size_t smem, void* stream) {              \
    const int tile = (int)(smem / sizeof(mg::D4));                                                \
    const cudaError_t a = cudaFuncSetAttribute((const void*)mg::cta_eval_kernel<KIND>,            \
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
    if (a != cudaSuccess) return (int)a;                                                          \
    mg::cta_eval_kernel<KIND><<<1, threads, smem, (cudaStream_t)stream>>>(d_inst, d_io, tile);    \
    return (int)cudaGetLastError();                                                               \
  }                                                                                               \
  /* one instance per cluster of csize CTAs; blocks = clusters * csize */                          \
  extern "C" int mg_launch_cbatch_##NAME(const mg::InstDesc* d_insts, int ninst, int* d_counter,  \
                                         int slice_iters, int threads, int csize, int clusters,    \
                                         size_t smem, void* stream) {                              \
    const cudaError_t a = cudaFuncSetAttribute((const void*)mg::cluster_batch_kernel<KIND>,       \
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
    if (a != cudaSuccess) return (int)a;                                                          \
    cudaLaunchConfig_t cfg = {};                                                                  \
    cfg.gridDim = dim3(clusters * csize);                                                         \
    cfg.blockDim = dim3(threads);                                                                 \
    cfg.dynamicSmemBytes = smem;                                                                  \
    cfg.stream = (cudaStream_t)stream;                                                            \
    cudaLaunchAttribute at[1];                                                                    \
    at[0].id = cudaLaunchAttributeClusterDimension;                                               \
    at[0].val.clusterDim.x = csize;                                                               \
    at[0].val.clusterDim.y = 1;                                                                   \
    at[0].val.clusterDim.z = 1;                                                                   \
    cfg.attrs = at;                                                                               \
    cfg.numAttrs = 1;                                                                             \
    const int tile = (int)(smem / sizeof(mg::D4));                                                \
    return (int)cudaLaunchKernelEx(&cfg, mg::cluster_batch_kernel<KIND>, d_insts, ninst, d_counter, \
                                   slice_iters, tile);                                            \
  }                                                                                               \
  /* clusters of csize CTAs that can be resident at once */                                      \
  extern "C" int mg_cluster_occupancy_##NAME(int threads, int csize, size_t smem, int* clusters) { \
    const cudaError_t a = cudaFuncSetAttribute((const void*)mg::cluster_batch_kernel<KIND>,       \
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
    if (a != cudaSuccess) return (int)a;                                                          \
    cudaLaunchConfig_t cfg = {};                                                                  \
    cfg.gridDim = dim3(csize);                                                                    \
    cfg.blockDim = dim3(threads);                                                                 \
    cfg.dynamicSmemBytes = smem;                                                                  \
    cudaLaunchAttribute at[1];                                                                    \
    at[0].id = cudaLaunchAttributeClusterDimension;                                               \
    at[0].val.clusterDim.x = csize;                                                               \
    at[0].val.clusterDim.y = 1;                                                                   \
    at[0].val.clusterDim.z = 1;                                                                   \
    cfg.attrs = at;                                                                               \
    cfg.numAttrs = 1;                                                                             \
    return (int)cudaOccupancyMaxActiveClusters(clusters, (const void*)mg::cluster_batch_kernel<KIND>, &cfg); \
  }                                                                                               \
  extern "C" int mg_occupancy_##NAME(int grid, int threads, size_t smem, int* blocks_per_sm) {    \
    if (grid) mg_grid_smem_##NAME(smem);                                                          \
    else mg_batch_smem_##NAME(smem);                                                              \
    return grid ? (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(                             \
                      blocks_per_sm, mg::grid_kernel<KIND>, threads, smem)                        \
                : (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(                             \
                      blocks_per_sm, mg::batch_kernel<KIND>, threads, smem);                      \
  }
