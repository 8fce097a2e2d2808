// api_minimisers.cpp -- Lbfgs, Fire, GradDescent and Anneal of the C++ API.
//
// deviceParams() describes the algorithm to the GPU engine (the path taken
// by minimise() for device potentials).  iteration() is the host loop used
// for host potentials and when a per-iteration callback is given; it follows
//   Lbfgs        src/minimisers/Lbfgs.cpp:34-133
//   Fire         src/minimisers/Fire.cpp:11-90
//   GradDescent  src/minimisers/GradDescent.cpp:11-46
//   Anneal       src/minimisers/Anneal.cpp:9-95
//   line search  src/minimisers/linesearch.cpp:8-30
#include <cmath>
#include <ctime>

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

// ---- Anneal ------------------------------------------------------------------------
namespace {
// the engine's random numbers (SplitMix64's output mix, Steele, Lea and Flood
// 2014, on a counter of (iteration, index) keyed by the seed)
uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}
double anneal_unit(uint64_t seed, int iter, uint32_t idx) {
  const uint64_t h = mix64(seed ^ mix64(((uint64_t)(uint32_t)iter << 32) | idx));
  return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}
uint64_t seed_of(uint64_t seed) { return seed ? seed : (uint64_t)std::time(nullptr) + (uint64_t)mpi.rank; }
}  // namespace

Anneal& Anneal::setDisplacement(double d) {
  displacement = d;
  return *this;
}
Anneal& Anneal::setTempInit(double t) {
  tempInit = t;
  return *this;
}
Anneal& Anneal::setCoolingRate(double r) {
  coolingRate = r;
  return *this;
}
Anneal& Anneal::setCoolingSchedule(std::function<double(int)> f) {
  coolingSchedule = f;
  return *this;
}
Anneal& Anneal::setMaxIter(int m) {
  Minimiser::setMaxIter(m);
  return *this;
}
Anneal& Anneal::setMaxRejections(int m) {
  maxRejections = m;
  return *this;
}
Anneal& Anneal::setSeed(uint64_t s) {
  seed = s;
  return *this;
}

bool Anneal::deviceParams(const State&, minim_gpu_minimiser_params* p) const {
  p->method = MINIM_ANNEAL;
  p->temp_init = tempInit;
  p->displacement = displacement;
  p->cooling_rate = coolingRate;
  p->max_rejections = maxRejections;
  p->seed = seed_of(seed);
  _table.clear();
  if (coolingSchedule) {
    const int n = (int)std::min<long long>((long long)maxIter + 1, 1LL << 24);
    _table.resize(n);
    for (int i = 0; i < n; i++) _table[i] = coolingSchedule(i);
    p->n_temp_schedule = n;
    p->temp_schedule = _table.data();
  }
  return true;
}

void Anneal::init(State& state) {
  _sinceAccepted = 0;
  _currentState = state.blockCoords();
  _currentE = state.energy();
  _seed = seed_of(seed);
}

void Anneal::iteration(State& state) {
  _temp = coolingSchedule ? coolingSchedule(iter) : tempInit / (1 + coolingRate * iter);
  vector<double> next(_currentState.size());
  for (size_t i = 0; i < next.size(); i++) {
    const double r = 2 * anneal_unit(_seed, iter, (uint32_t)i) - 1;
    next[i] = _currentState[i] + r * displacement;
  }
  state.blockCoords(next);
  const double e = state.energy();
  if (acceptMetropolis(e)) {
    _currentState = state.blockCoords();
    _currentE = e;
    _sinceAccepted = 0;
  } else {
    _sinceAccepted++;
  }
  if (checkConvergence(state) || iter == maxIter) state.blockCoords(_currentState);
}

bool Anneal::acceptMetropolis(double energy) {
  const double u = anneal_unit(_seed, iter, (uint32_t)_currentState.size());
  return energy < _currentE || u < std::exp((_currentE - energy) / _temp);
}

bool Anneal::checkConvergence(const State&) { return maxRejections > 0 && _sinceAccepted >= maxRejections; }

}  // namespace minim
