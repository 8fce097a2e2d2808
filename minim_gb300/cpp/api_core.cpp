// api_core.cpp -- Potential, State and Minimiser of the source-compatible C++
// API (include/minim/).  Behaviour follows the reference library:
//   Potential   src/Potential.cpp:10-162
//   State       src/State.cpp:12-328
//   Minimiser   src/Minimiser.cpp:9-69
// Device potentials route evaluations and whole minimisations through the C
// ABI (minim_gpu.h); host potentials run on the host as in the reference.
#include <cmath>
#include <iomanip>
#include <sstream>
#include <stdexcept>
#include <string>

#include "minim.h"

namespace minim {

Mpi mpi;

void throw_gpu(int rc) {
  if (rc == MINIM_GPU_OK) return;
  char buf[1024];
  minim_gpu_last_error(buf, sizeof buf);
  if (rc == MINIM_GPU_ERR_INVALID) throw std::invalid_argument(buf);
  throw std::runtime_error(buf);
}

// ---------------------------------------------------------------------------
// Potential
// ---------------------------------------------------------------------------
Potential::Potential(EFunc energy, GFunc gradient)
    : _energy(energy), _gradient(gradient), _energyGradient(nullptr) {}
Potential::Potential(EGFunc energyGradient)
    : _energy(nullptr), _gradient(nullptr), _energyGradient(energyGradient) {}

double Potential::energy(const vector<double>& coords) const {
  if (_energy) return _energy(coords);
  throw std::runtime_error("Potential: No energy function defined. If using parallel you must call energyGradient instead.");
}

vector<double> Potential::gradient(const vector<double>& coords) const {
  if (_gradient) return _gradient(coords);
  throw std::runtime_error("Potential: No gradient function defined. If using parallel you must call energyGradient instead.");
}

void Potential::energyGradient(const vector<double>& coords, const Communicator&, double* e,
                               vector<double>* g) const {
  if (_energyGradient) return _energyGradient(coords, e, g);
  if (e) *e = energy(coords);
  if (g) *g = gradient(coords);
}

State Potential::newState(const vector<double>& coords, const vector<int>& ranks) {
  return State(*this, coords, ranks);
}
State Potential::newState(int ndof, const vector<int>& ranks) {
  return newState(vector<double>(ndof), ranks);
}

Potential& Potential::setElements(vector<Element> e) {
  elements = e;
  return *this;
}
Potential& Potential::setElements(vector2d<int> idofs) {
  elements.clear();
  for (const auto& idof : idofs) elements.push_back({0, idof, {}});
  return *this;
}
Potential& Potential::setElements(vector2d<int> idofs, vector<int> types, vector2d<double> parameters) {
  elements.clear();
  for (size_t i = 0; i < idofs.size(); i++) elements.push_back({types[i], idofs[i], parameters[i]});
  return *this;
}

Potential& Potential::setConstraints(vector<int> iFix) {
  for (int i : iFix) constraints.push_back({{i}, nullptr, nullptr});
  return *this;
}
Potential& Potential::setConstraints(vector2d<int> idofs, vector<double> normal) {
  for (const auto& idof : idofs)
    constraints.push_back({idof, [normal](const vector<int>&, const vector<double>&) { return normal; }, nullptr});
  return *this;
}
Potential& Potential::setConstraints(vector2d<int> idofs, Constraint::NormalFn normal,
                                     Constraint::CorrectionFn correction) {
  for (const auto& idof : idofs) constraints.push_back({idof, normal, correction});
  return *this;
}

// Fixed dofs zeroed; for vector constraints the component of the step along
// the normal is removed; then the potential's specialised constraints.
void Potential::applyConstraints(const vector<double>& coords, const Communicator& comm,
                                 vector<double>& step) const {
  for (const auto& c : constraints) {
    if (c.idof.size() == 1) {
      step[c.idof[0]] = 0;
    } else {
      const vector<double> n = c.normal(coords);
      double nn = 0, gn = 0;
      for (size_t i = 0; i < n.size(); i++) {
        nn += n[i] * n[i];
        gn += step[c.idof[i]] * n[i];
      }
      for (size_t i = 0; i < n.size(); i++) step[c.idof[i]] -= gn * n[i] / nn;
    }
  }
  specialisedConstraints(coords, comm, step);
}

void Potential::correctConstraints(vector<double>& coords) const {
  for (const auto& c : constraints)
    if (c.correction) c.correction(c.idof, coords);
}

bool Potential::isFixed(int index) const {
  for (const auto& c : constraints)
    if (c.idof.size() == 1 && c.idof[0] == index) return true;
  return false;
}
vector<char> Potential::isFixed(const vector<int>& idx) const {
  vector<char> out(idx.size(), false);
  for (size_t i = 0; i < idx.size(); i++) out[i] = isFixed(idx[i]);
  return out;
}
vector<int> Potential::fixedDofs() const {
  vector<int> f;
  for (const auto& c : constraints)
    if (c.idof.size() == 1) f.push_back(c.idof[0]);
  return f;
}
bool Potential::hasNormalConstraints() const {
  for (const auto& c : constraints)
    if (c.idof.size() != 1) return true;
  return false;
}

std::unique_ptr<Communicator> Potential::newComm() const {
  if (potentialType() == UNSTRUCTURED && distributed)
    throw std::invalid_argument("Potential: You cannot create a State with a Potential that has already been distributed.");
  return std::make_unique<Communicator>();
}

Potential& Potential::setCommArray(vector<int> a) {
  commArray = a;
  return *this;
}

// ---------------------------------------------------------------------------
// State
// ---------------------------------------------------------------------------
State::State(const Potential& p, const vector<double>& coords, const vector<int>& ranks)
    : ndof(coords.size()), pot(p.clone()) {
  (void)ranks;
  pot->init(coords);
  convergence = pot->convergence;
  comm = pot->newComm();
  comm->setup(*pot, ndof, ranks);
  pot->initLocal(coords, *comm);
  _coords = coords;
  attachDevice();
}

void State::attachDevice() {
  dev_ = pot->createDevice(_coords);
  if (!dev_) return;
  const vector<int> fix = pot->fixedDofs();
  if (!fix.empty()) throw_gpu(minim_gpu_instance_set_fixed(dev_, fix.data(), fix.size()));
}

State::State(const State& s)
    : ndof(s.ndof), convergence(s.convergence), pot(s.pot->clone()), comm(s.comm->clone()),
      usesThisProc(s.usesThisProc), isFailed(s.isFailed), _coords(s._coords) {
  attachDevice();
}

State& State::operator=(const State& s) {
  if (this == &s) return *this;
  if (dev_) minim_gpu_instance_destroy(dev_);
  dev_ = nullptr;
  ndof = s.ndof;
  convergence = s.convergence;
  pot = s.pot->clone();
  comm = s.comm->clone();
  usesThisProc = s.usesThisProc;
  isFailed = s.isFailed;
  _coords = s._coords;
  attachDevice();
  return *this;
}

State::~State() {
  if (dev_) minim_gpu_instance_destroy(dev_);
}

namespace {
// host evaluation: basicEG / elementEG (src/State.cpp:48-79)
void host_eg(const Potential& pot, const Communicator& comm, const vector<double>& x, double* e,
             vector<double>* g) {
  if (e) *e = 0;
  if (g) *g = vector<double>(x.size());
  if (pot.potentialType() == Potential::UNSTRUCTURED) {
    for (const auto& el : pot.elements) pot.elementEnergyGradient(x, el, e, g);
    pot.blockEnergyGradient(x, comm, e, g);
  } else {
    pot.energyGradient(x, comm, e, g);
  }
  if (g) pot.applyConstraints(x, comm, *g);
}

// host-side vector constraints a device potential may carry
void host_normals(const Potential& pot, const vector<double>& x, vector<double>& v) {
  for (const auto& c : pot.constraints) {
    if (c.idof.size() == 1) continue;
    const vector<double> n = c.normal(x);
    double nn = 0, gn = 0;
    for (size_t i = 0; i < n.size(); i++) {
      nn += n[i] * n[i];
      gn += v[c.idof[i]] * n[i];
    }
    for (size_t i = 0; i < n.size(); i++) v[c.idof[i]] -= gn * n[i] / nn;
  }
}
}  // namespace

void State::energyGradient(const vector<double>& x, double* e, vector<double>* g) const {
  if (!usesThisProc) return;
  if (dev_) {
    if (g) g->assign(ndof, 0.0);
    throw_gpu(minim_gpu_energy_gradient(dev_, x.data(), e, g ? g->data() : nullptr));
    if (g && pot->hasNormalConstraints()) host_normals(*pot, x, *g);
    return;
  }
  host_eg(*pot, *comm, x, e, g);
}

double State::energy(const vector<double>& x) const {
  if (!usesThisProc) return 0;
  double e = 0;
  energyGradient(x, &e, nullptr);
  return e;
}
vector<double> State::gradient(const vector<double>& x) const {
  if (!usesThisProc) return {};
  vector<double> g;
  energyGradient(x, nullptr, &g);
  return g;
}
double State::energy() const { return energy(_coords); }
vector<double> State::gradient() const { return gradient(_coords); }
void State::energyGradient(double* e, vector<double>* g) const { energyGradient(_coords, e, g); }

double State::blockEnergy() const { return energy(); }
double State::blockEnergy(const vector<double>& x) const { return energy(x); }
vector<double> State::blockGradient() const { return gradient(); }
vector<double> State::blockGradient(const vector<double>& x) const { return gradient(x); }
void State::blockEnergyGradient(double* e, vector<double>* g) const { energyGradient(e, g); }
void State::blockEnergyGradient(const vector<double>& x, double* e, vector<double>* g) const {
  energyGradient(x, e, g);
}
double State::procEnergy() const { return energy(); }
double State::procEnergy(const vector<double>& x) const { return energy(x); }
vector<double> State::procGradient() const { return gradient(); }
vector<double> State::procGradient(const vector<double>& x) const { return gradient(x); }
void State::procEnergyGradient(double* e, vector<double>* g) const { energyGradient(e, g); }
void State::procEnergyGradient(const vector<double>& x, double* e, vector<double>* g) const {
  energyGradient(x, e, g);
}
double State::allEnergy() const { return energy(); }
vector<double> State::allGradient() const { return gradient(); }
void State::allEnergyGradient(double* e, vector<double>* g) const { energyGradient(e, g); }
vector<double> State::allCoords() const { return _coords; }

double State::operator[](int i) { return _coords[i]; }
vector<double> State::coords() const { return _coords; }
void State::coords(const vector<double>& in) { _coords = in; }
const vector<double>& State::blockCoords() const { return _coords; }
void State::blockCoords(const vector<double>& in) { _coords = in; }

double State::componentEnergy(int component) const {
  double e = 0;
  for (const auto& el : pot->elements)
    if (el.type == component) pot->elementEnergyGradient(_coords, el, &e, nullptr);
  return e;
}

void State::applyConstraints(vector<double>& data) const {
  if (dev_) {
    throw_gpu(minim_gpu_apply_constraints(dev_, data.data()));
    if (pot->hasNormalConstraints()) host_normals(*pot, _coords, data);
    return;
  }
  pot->applyConstraints(_coords, *comm, data);
}

// ---------------------------------------------------------------------------
// Minimiser
// ---------------------------------------------------------------------------
Minimiser& Minimiser::setMaxIter(int m) {
  maxIter = m;
  return *this;
}

Minimiser& Minimiser::setLinesearch(std::string method) {
  if (method != "backtracking" && method != "none") throw std::invalid_argument("Invalid line search method.");
  linesearch = method;
  return *this;
}

Minimiser& Minimiser::setPrecision(std::string p) {
  if (p != "mixed" && p != "fp64" && p != "fp32") throw std::invalid_argument("Invalid precision.");
  precision = p;
  return *this;
}

bool Minimiser::deviceMinimise(State& state) {
  minim_gpu_minimiser_params p;
  minim_gpu_default_minimiser(MINIM_LBFGS, &p);
  if (!deviceParams(state, &p)) return false;
  if (state.pot->hasNormalConstraints()) return false;
  p.linesearch = linesearch == "none" ? MINIM_LS_NONE : MINIM_LS_BACKTRACKING;
  p.max_iter = maxIter;
  p.tol = state.convergence;
  p.precision = precision == "fp64" ? MINIM_PREC_FP64 : (precision == "fp32" ? MINIM_PREC_FP32 : MINIM_PREC_MIXED);
  throw_gpu(minim_gpu_instance_set_coords(state.device(), state._coords.data()));
  throw_gpu(minim_gpu_minimise(state.device(), &p, &lastResult));
  throw_gpu(minim_gpu_instance_get_coords(state.device(), state._coords.data()));
  iter = lastResult.iter;
  deviceDone(lastResult);
  // a device failure (non-finite values, a device wait that gave up) is the
  // reference's failure flag, State::failed() (src/State.cpp:326-328)
  if (lastResult.status == MINIM_RES_NAN || lastResult.status == MINIM_RES_TIMEOUT) state.failed();
  return true;
}

std::vector<double> Minimiser::minimise(State& state, std::function<void(int, State&)> adjustState) {
  if (!state.usesThisProc) return {};
  if (!adjustState && state.device() && deviceMinimise(state)) return state.coords();
  init(state);
  for (iter = 0; iter <= maxIter; iter++) {
    if (adjustState) adjustState(iter, state);
    if (state.isFailed) break;
    iteration(state);
    if (checkConvergence(state)) break;
  }
  return state.coords();
}

std::vector<double> Minimiser::minimise(State& state, std::string logType) {
  std::function<void(int, State&)> logFn = nullptr;
  const size_t div = logType.find('-');
  if (div < logType.length()) {
    const std::string fields = logType.substr(0, div);
    const int every = std::stoi(logType.substr(div + 1));
    if (every > 0) {
      const int digits = (int)std::to_string(maxIter).length();
      logFn = [every, fields, digits](int i, State& s) {
        if (i % every != 0) return;
        const bool logE = fields.find('e') != std::string::npos;
        const bool logG = fields.find('g') != std::string::npos;
        double e = 0;
        vector<double> g;
        s.energyGradient(logE ? &e : nullptr, logG ? &g : nullptr);
        std::ostringstream out;
        out << "I: " << std::setw(digits) << i;
        if (logE) out << "  E: " << e;
        if (logG) out << "  G: " << vec::rms(g);
        print(out.str());
      };
    }
  }
  return minimise(state, logFn);
}

}  // namespace minim
