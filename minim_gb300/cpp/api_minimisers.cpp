// api_minimisers.cpp -- Lbfgs, Fire and GradDescent of the C++ API.
//
// deviceParams() describes the algorithm to the GPU engine (the path taken
// by minimise() for device potentials).  iteration() is the host loop used
// for host potentials and when a per-iteration callback is given; it follows
//   Lbfgs        src/minimisers/Lbfgs.cpp:34-133
//   Fire         src/minimisers/Fire.cpp:11-90
//   GradDescent  src/minimisers/GradDescent.cpp:11-46
//   line search  src/minimisers/linesearch.cpp:8-30
#include <cmath>

#include "minim.h"

namespace minim {

namespace {
// backtrackingLinesearch: Armijo with c = 0.5, tau = 0.5, at most 10 shrinks;
// the last (unevaluated) trial is taken when none passes.
double backtracking(State& state, vector<double>& step, double de0) {
  const double c = 0.5, tau = 0.5;
  double t = -c * de0;
  const double e0 = state.energy();
  double mult = 1;
  vector<double> x = state.blockCoords() + step;
  for (int i = 0; i < 10; i++) {
    const double e = state.energy(x);
    if (e0 - e >= t) break;
    step = step * tau;
    x = state.blockCoords() + step;
    mult *= tau;
    t *= tau;
  }
  state.blockCoords(x);
  return mult;
}
}  // namespace

// ---- Lbfgs ------------------------------------------------------------------------
Lbfgs& Lbfgs::setM(int m) {
  _m = m;
  return *this;
}
Lbfgs& Lbfgs::setMaxIter(int m) {
  Minimiser::setMaxIter(m);
  return *this;
}
Lbfgs& Lbfgs::setMaxStep(double s) {
  _maxStep = s;
  return *this;
}
Lbfgs& Lbfgs::setInitStep(double s) {
  _initStep = s;
  return *this;
}

bool Lbfgs::deviceParams(const State&, minim_gpu_minimiser_params* p) const {
  p->method = MINIM_LBFGS;
  p->m = _m;
  p->max_step = _maxStep;
  p->init_step = _initStep;
  return _m >= 1 && _m <= 16;
}

void Lbfgs::init(State&) {
  _s.assign(_m, {});
  _y.assign(_m, {});
  _rho.assign(_m, 0.0);
}

void Lbfgs::iteration(State& state) {
  if (iter == 0) {
    _g = state.procGradient();
    _i = 0;
  } else {
    _i++;
  }
  vector<double> step = getDirection(*state.comm);
  state.applyConstraints(step);
  double gs = state.comm->dotProduct(_g, step);
  if (gs > 0) {
    gs = -gs;
    step = -step;
  }
  if (linesearch == "backtracking") backtracking(state, step, gs);
  else state.blockCoords(state.blockCoords() + step);
  vector<double> gNew = state.procGradient();
  const vector<double> y = gNew - _g;
  const double sy = state.comm->dotProduct(step, y);
  if (sy != 0) {
    const int c = _i % _m;
    _s[c] = step;
    _y[c] = y;
    _rho[c] = 1 / sy;
  } else {
    _i--;
  }
  _g = gNew;
}

vector<double> Lbfgs::getDirection(const Communicator& comm) {
  vector<double> alpha(_m);
  const int mt = std::min(_m, _i);
  const int c = _i % _m;
  vector<double> step = -_g;
  if (_i == 0) {
    const double gn = comm.norm(_g);
    if (gn > 0) step *= _initStep / gn;
    return step;
  }
  for (int k1 = 0; k1 < mt; k1++) {
    const int k = (c - 1 - k1 + _m) % _m;
    alpha[k] = _rho[k] * comm.dotProduct(step, _s[k]);
    for (size_t j = 0; j < step.size(); j++) step[j] -= alpha[k] * _y[k][j];
  }
  const int kn = (c - 1 + _m) % _m;
  step *= 1 / (_rho[kn] * comm.dotProduct(_y[kn], _y[kn]));
  for (int k1 = 0; k1 < mt; k1++) {
    const int k = (c - mt + k1 + _m) % _m;
    const double beta = _rho[k] * comm.dotProduct(step, _y[k]);
    for (size_t j = 0; j < step.size(); j++) step[j] += (alpha[k] - beta) * _s[k][j];
  }
  if (_maxStep != 0) {
    const double ss = comm.norm(step);
    if (ss > _maxStep) step *= _maxStep / ss;
  }
  return step;
}

bool Lbfgs::checkConvergence(const State& state) {
  return std::sqrt(state.comm->dotProduct(_g, _g) / state.ndof) < state.convergence;
}

// ---- Fire ----------------------------------------------------------------------------
Fire::Fire(double dt) : dtMax(dt) { linesearch = "none"; }
Fire& Fire::setMaxIter(int m) {
  Minimiser::setMaxIter(m);
  return *this;
}
Fire& Fire::setDtMax(double dt) {
  dtMax = dt;
  return *this;
}

bool Fire::deviceParams(const State&, minim_gpu_minimiser_params* p) const {
  p->method = MINIM_FIRE;
  p->dt_max = dtMax;
  return true;
}

void Fire::init(State& state) {
  _v.assign(state.ndof, 0.0);
  if (dtMax != 0) return;
  _g = state.procGradient();
  _gNorm = std::sqrt(state.comm->dotProduct(_g, _g));
  if (_gNorm != 0) {
    dtMax = 0.1 / std::sqrt(_gNorm);
  } else {
    print("Warning: Unable to estimate dtMax parameter for FIRE.");
    dtMax = 1;
  }
}

void Fire::iteration(State& state) {
  if (iter == 0) {
    _dt = dtMax;
    _g = state.procGradient();
    _gNorm = std::sqrt(state.comm->dotProduct(_g, _g));
  }
  const double p = -state.comm->dotProduct(_v, _g);
  if (p > 0) {
    const double vNorm = std::sqrt(state.comm->dotProduct(_v, _v));
    _v = (1 - _a) * _v - (_a * vNorm / _gNorm + _dt) * _g;
    _nSteps++;
  } else {
    _v = -_dt * _g;
    _nSteps = 0;
  }
  if (p > 0 && _nSteps > _nMin) {
    _a *= _fA;
    _dt *= _fInc;
    if (_dt > dtMax) _dt = dtMax;
  } else if (p <= 0) {
    _a = _aStart;
    _dt *= _fDec;
  }
  vector<double> step = _dt * _v;
  state.applyConstraints(step);
  if (linesearch == "backtracking") {
    const double gs = state.comm->dotProduct(_g, step);
    backtracking(state, step, gs);
  } else {
    state.blockCoords(state.blockCoords() + step);
  }
  _g = state.procGradient();
  _gNorm = std::sqrt(state.comm->dotProduct(_g, _g));
}

bool Fire::checkConvergence(const State& state) { return _gNorm / std::sqrt((double)state.ndof) < state.convergence; }

// ---- GradDescent -------------------------------------------------------------------
GradDescent& GradDescent::setAlpha(double a) {
  _alpha = a;
  return *this;
}
GradDescent& GradDescent::setMaxIter(int m) {
  Minimiser::setMaxIter(m);
  return *this;
}

bool GradDescent::deviceParams(const State&, minim_gpu_minimiser_params* p) const {
  p->method = MINIM_GD;
  p->alpha = _alpha;
  return true;
}

void GradDescent::init(State& state) { _g.assign(state.ndof, 0.0); }

void GradDescent::iteration(State& state) {
  _g = state.procGradient();
  vector<double> step = -_alpha * _g;
  if (linesearch == "backtracking") {
    const double gs = state.comm->dotProduct(_g, step);
    backtracking(state, step, gs);
  } else {
    state.blockCoords(state.blockCoords() + step);
  }
}

bool GradDescent::checkConvergence(const State& state) {
  return std::sqrt(state.comm->dotProduct(_g, _g) / state.ndof) < state.convergence;
}

}  // namespace minim
