// ref_shim.cpp -- extern "C" driver over the reference minim library's own
// public C++ API (State, Potential subclasses, Lbfgs/Fire/GradDescent/Anneal).
//
// Test infrastructure only: it is linked against the reference sources
// compiled unmodified by oracle/Makefile into oracle/_ref/, and is used to
// generate golden fixtures and to pin the C restatement (minim_oracle.c).
// It takes the same parameter structs as the GPU C ABI (include/minim_gpu.h)
// so a test can hand one description to the reference, the restatement and
// the GPU engine.
#include "minim.h"
#include "minim_gpu.h"

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

using namespace minim;
using std::vector;

namespace {

thread_local std::string g_err;

struct RefState {
  int kind;
  std::unique_ptr<State> state;
};

template <typename T>
vector<T> vec_of(const T* p, int n) {
  return (p && n > 0) ? vector<T>(p, p + n) : vector<T>();
}

int fail(const std::exception& e, int code) {
  g_err = e.what();
  return code;
}

std::unique_ptr<State> build(int kind, const void* params, const double* x0, size_t ndof,
                             const int* fixed, int nfixed) {
  vector<double> x(x0, x0 + ndof);
  vector<int> fix = vec_of(fixed, nfixed);
  if (kind == MINIM_GPU_LJ) {
    auto p = static_cast<const minim_gpu_lj_params*>(params);
    if (p->cutoff != 0) throw std::invalid_argument("the reference LjNd has no cutoff");
    LjNd pot(p->ndim, p->sigma, p->epsilon);
    if (!fix.empty()) pot.setConstraints(fix);
    return std::make_unique<State>(pot, x);
  }
  if (kind == MINIM_GPU_PF) {
    auto p = static_cast<const minim_gpu_pf_params*>(params);
    PhaseField pf;
    pf.setNFluid(p->nfluid);
    pf.setGridSize({p->grid[0], p->grid[1], p->grid[2]});
    pf.setResolution(p->resolution);
    if (p->n_interface_size > 0) pf.setInterfaceSize(vec_of(p->interface_size, p->n_interface_size));
    if (p->n_surface_tension > 0) pf.setSurfaceTension(vec_of(p->surface_tension, p->n_surface_tension));
    pf.densityConstraint = p->density_constraint;
    pf.densityConst = p->density_const;
    int ngrid = p->grid[0] * p->grid[1] * p->grid[2];
    if (p->volume_fixed) {
      if (p->volume) pf.setVolume(vec_of(p->volume, p->nfluid), p->vol_const);
      else pf.setVolumeFixed(true, p->vol_const);
    }
    if (p->pressure) pf.setPressure(vec_of(p->pressure, p->nfluid));
    if (p->solid) pf.setSolid(vec_of(p->solid, ngrid));
    if (p->n_contact_angle > 0) pf.setContactAngle(vec_of(p->contact_angle, p->n_contact_angle));
    if (p->force) {
      pf.force = vector<vector<double>>(p->nfluid, vector<double>(3));
      for (int f = 0; f < p->nfluid; f++)
        for (int d = 0; d < 3; d++) pf.force[f][d] = p->force[3 * f + d];
    }
    if (p->fix_fluid) pf.fixFluid = vec_of(p->fix_fluid, p->nfluid);
    if (p->confinement) pf.setConfinement(vec_of(p->confinement, p->nfluid));
    if (!fix.empty()) pf.setConstraints(fix);
    return std::make_unique<State>(pf, x);
  }
  if (kind == MINIM_GPU_PFU) {
    auto p = static_cast<const minim_gpu_pf_params*>(params);
    PhaseFieldUnstructured pf;
    pf.setNFluid(p->nfluid);
    pf.setGridSize({p->grid[0], p->grid[1], p->grid[2]});
    pf.setResolution(p->resolution);
    if (p->n_interface_size > 0) pf.setInterfaceSize(vec_of(p->interface_size, p->n_interface_size));
    if (p->n_surface_tension > 0) pf.setSurfaceTension(vec_of(p->surface_tension, p->n_surface_tension));
    pf.densityConstraint = p->density_constraint;
    pf.densityConst = p->density_const;
    int ngrid = p->grid[0] * p->grid[1] * p->grid[2];
    if (p->volume_fixed) {
      if (p->volume) pf.setVolume(vec_of(p->volume, p->nfluid), p->vol_const);
      else pf.setVolumeFixed(true, p->vol_const);
    }
    if (p->pressure) pf.setPressure(vec_of(p->pressure, p->nfluid));
    if (p->solid) pf.setSolid(vec_of(p->solid, ngrid));
    if (p->n_contact_angle > 0) pf.setContactAngle(vec_of(p->contact_angle, p->n_contact_angle));
    if (p->force) {
      pf.force = vector<vector<double>>(p->nfluid, vector<double>(3));
      for (int f = 0; f < p->nfluid; f++)
        for (int d = 0; d < 3; d++) pf.force[f][d] = p->force[3 * f + d];
    }
    if (p->fix_fluid) pf.fixFluid = vec_of(p->fix_fluid, p->nfluid);
    if (p->confinement) pf.setConfinement(vec_of(p->confinement, p->nfluid));
    // init() replaces the potential's constraint list, so fixed degrees of
    // freedom are added to the state's own copy afterwards
    auto st = std::make_unique<State>(pf, x);
    if (!fix.empty()) st->pot->setConstraints(fix);
    return st;
  }
  if (kind == MINIM_GPU_BAH) {
    auto p = static_cast<const minim_gpu_bah_params*>(params);
    BarAndHinge pot;
    if (p->ntri > 0) {
      vector<vector<int>> tris(p->ntri);
      for (int t = 0; t < p->ntri; t++) tris[t] = {p->tris[3 * t], p->tris[3 * t + 1], p->tris[3 * t + 2]};
      pot.setTriangulation(tris);
    }
    if (p->nbond > 0) {
      vector<vector<int>> b(p->nbond);
      for (int i = 0; i < p->nbond; i++) b[i] = vec_of(p->bonds + i * p->bond_stride, p->bond_stride);
      pot.setBondList(b);
    }
    if (p->nhinge > 0) {
      vector<vector<int>> h(p->nhinge);
      for (int i = 0; i < p->nhinge; i++) h[i] = vec_of(p->hinges + i * p->hinge_stride, p->hinge_stride);
      pot.setHingeList(h);
    }
    pot.setModulus(p->modulus);
    pot.poissonRatio = p->poisson_ratio;
    if (p->n_thickness > 0) pot.setThickness(vec_of(p->thickness, p->n_thickness));
    if (p->n_kbond > 0 || p->n_khinge > 0)
      pot.setRigidity(vec_of(p->kbond, p->n_kbond), vec_of(p->khinge, p->n_khinge));
    if (p->n_length0 > 0) pot.setLength0(vec_of(p->length0, p->n_length0));
    if (p->n_theta0 > 0) pot.setTheta0(vec_of(p->theta0, p->n_theta0));
    if (p->n_force > 0) pot.setForce(vec_of(p->force, p->n_force));
    pot.setWall(p->wall_on != 0);
    pot.setWallAdhesion(p->wall_adhesion != 0);
    pot.setWallParams(p->wall_epsilon, p->wall_sigma);
    if (!fix.empty()) pot.setConstraints(fix);
    return std::make_unique<State>(pot, x);
  }
  throw std::invalid_argument("ref_shim: unknown potential kind");
}

}  // namespace

extern "C" {

int ref_last_error(char* buf, size_t len) {
  if (buf && len) {
    std::strncpy(buf, g_err.c_str(), len - 1);
    buf[len - 1] = 0;
  }
  return (int)g_err.size();
}

void ref_set_num_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n > 0 ? n : 1);
#else
  (void)n;
#endif
}

int ref_create(int kind, const void* params, const double* x0, size_t ndof,
               const int* fixed, int nfixed, void** out) {
  try {
    auto rs = new RefState{kind, build(kind, params, x0, ndof, fixed, nfixed)};
    *out = rs;
    return 0;
  } catch (const std::invalid_argument& e) {
    return fail(e, MINIM_GPU_ERR_INVALID);
  } catch (const std::exception& e) {
    return fail(e, MINIM_GPU_ERR_RUNTIME);
  }
}

void ref_destroy(void* h) { delete static_cast<RefState*>(h); }

int ref_set_coords(void* h, const double* x) {
  auto rs = static_cast<RefState*>(h);
  rs->state->coords(vector<double>(x, x + rs->state->ndof));
  return 0;
}

int ref_get_coords(void* h, double* x) {
  auto rs = static_cast<RefState*>(h);
  auto c = rs->state->coords();
  std::memcpy(x, c.data(), c.size() * sizeof(double));
  return 0;
}

double ref_default_tol(void* h) { return static_cast<RefState*>(h)->state->convergence; }

// Energy via State::energy(coords), gradient via State::gradient(coords):
// the two calls the minimisers make (src/State.cpp:134-172).
int ref_energy_gradient(void* h, const double* x, double* e, double* g) {
  try {
    auto rs = static_cast<RefState*>(h);
    State& s = *rs->state;
    vector<double> xv = x ? vector<double>(x, x + s.ndof) : s.coords();
    if (e) *e = s.energy(xv);
    if (g) {
      auto gv = s.gradient(xv);
      std::memcpy(g, gv.data(), gv.size() * sizeof(double));
    }
    return 0;
  } catch (const std::exception& ex) {
    return fail(ex, MINIM_GPU_ERR_RUNTIME);
  }
}

int ref_apply_constraints(void* h, double* v) {
  auto rs = static_cast<RefState*>(h);
  State& s = *rs->state;
  vector<double> d(v, v + s.ndof);
  s.applyConstraints(d);
  std::memcpy(v, d.data(), d.size() * sizeof(double));
  return 0;
}

int ref_minimise(void* h, const minim_gpu_minimiser_params* mp, minim_gpu_result* res) {
  try {
    auto rs = static_cast<RefState*>(h);
    State& s = *rs->state;
    if (mp->tol >= 0) s.convergence = mp->tol;
    const char* ls = (mp->linesearch == MINIM_LS_NONE) ? "none" : "backtracking";
    int iter = 0;
    double dtmax = 0;
    if (mp->method == MINIM_LBFGS) {
      Lbfgs min;
      min.setM(mp->m).setMaxStep(mp->max_step).setInitStep(mp->init_step).setMaxIter(mp->max_iter);
      min.setLinesearch(ls);
      min.minimise(s);
      iter = min.iter;
    } else if (mp->method == MINIM_FIRE) {
      Fire min;
      min.dtMax = mp->dt_max;
      min.setMaxIter(mp->max_iter);
      min.setLinesearch(ls);
      min.minimise(s);
      iter = min.iter;
      dtmax = min.dtMax;
    } else if (mp->method == MINIM_GD) {
      GradDescent min;
      min.setAlpha(mp->alpha).setMaxIter(mp->max_iter);
      min.setLinesearch(ls);
      min.minimise(s);
      iter = min.iter;
    } else if (mp->method == MINIM_ANNEAL) {
      // Minimiser::minimise (src/Minimiser.cpp:27-38) spelled out, so that
      // rand() can be seeded after Anneal::init (which seeds it from the
      // clock): srand(seed), then the reference's own iterations
      Anneal min(mp->temp_init, mp->displacement);
      min.setCoolingRate(mp->cooling_rate).setMaxRejections(mp->max_rejections).setMaxIter(mp->max_iter);
      if (mp->n_temp_schedule > 0) {
        vector<double> tab(mp->temp_schedule, mp->temp_schedule + mp->n_temp_schedule);
        min.setCoolingSchedule([tab](int i) { return tab[i < (int)tab.size() ? i : (int)tab.size() - 1]; });
      }
      min.init(s);
      srand((unsigned)mp->seed);
      for (min.iter = 0; min.iter <= min.maxIter; min.iter++) {
        min.iteration(s);
        if (min.checkConvergence(s)) break;
      }
      iter = min.iter;
    } else {
      throw std::invalid_argument("ref_shim: unknown minimiser");
    }
    if (res) {
      std::memset(res, 0, sizeof(*res));
      double gg = 0;
      if (mp->method != MINIM_ANNEAL) {
        auto g = s.gradient();
        for (double v : g) gg += v * v;
      }
      res->rms = std::sqrt(gg / s.ndof);
      res->energy = s.energy();
      res->iter = iter;
      res->status = (iter <= mp->max_iter) ? MINIM_RES_CONVERGED : MINIM_RES_MAXITER;
      res->dt_max = dtmax;
    }
    return 0;
  } catch (const std::invalid_argument& e) {
    return fail(e, MINIM_GPU_ERR_INVALID);
  } catch (const std::exception& e) {
    return fail(e, MINIM_GPU_ERR_RUNTIME);
  }
}

// Elements of a BarAndHinge state in the reference's own order: bars
// (type 0: two nodes, {k, l0}), hinges (type 1: four nodes, {k, theta0}).
int ref_bah_elements(void* h, int cap, int* nbar, int* bars, double* bar_par,
                     int* nhinge, int* hinges, double* hinge_par) {
  auto rs = static_cast<RefState*>(h);
  int nb = 0, nh = 0;
  for (const auto& el : rs->state->pot->elements) {
    if (el.type == 0) {
      if (nb < cap) {
        bars[2 * nb] = el.idof[0] / 3;
        bars[2 * nb + 1] = el.idof[3] / 3;
        bar_par[2 * nb] = el.parameters[0];
        bar_par[2 * nb + 1] = el.parameters[1];
      }
      nb++;
    } else if (el.type == 1) {
      if (nh < cap) {
        for (int k = 0; k < 4; k++) hinges[4 * nh + k] = el.idof[3 * k] / 3;
        hinge_par[2 * nh] = el.parameters[0];
        hinge_par[2 * nh + 1] = el.parameters[1];
      }
      nh++;
    }
  }
  *nbar = nb;
  *nhinge = nh;
  return 0;
}

// PhaseField set-up products: kappa, kappaP (nParams each), nodeVol and
// surfaceArea (ngrid each).
int ref_pf_internals(void* h, double* kappa, double* kappaP, double* node_vol,
                     double* surface_area, int* nk) {
  auto rs = static_cast<RefState*>(h);
  if (rs->kind == MINIM_GPU_PFU) {
    // nodeVol is per degree of freedom after initLocal; no surfaceArea member
    auto& pf = static_cast<PhaseFieldUnstructured&>(*rs->state->pot);
    *nk = (int)pf.kappa.size();
    std::memcpy(kappa, pf.kappa.data(), pf.kappa.size() * sizeof(double));
    std::memcpy(kappaP, pf.kappaP.data(), pf.kappaP.size() * sizeof(double));
    for (int i = 0; i < pf.nGrid; i++) {
      node_vol[i] = pf.nodeVol[(size_t)i * pf.nFluid];
      surface_area[i] = 0;
    }
    return 0;
  }
  auto& pf = static_cast<PhaseField&>(*rs->state->pot);
  *nk = (int)pf.kappa.size();
  std::memcpy(kappa, pf.kappa.data(), pf.kappa.size() * sizeof(double));
  std::memcpy(kappaP, pf.kappaP.data(), pf.kappaP.size() * sizeof(double));
  std::memcpy(node_vol, pf.nodeVol.data(), pf.nodeVol.size() * sizeof(double));
  std::memcpy(surface_area, pf.surfaceArea.data(), pf.surfaceArea.size() * sizeof(double));
  return 0;
}

}  // extern "C"
