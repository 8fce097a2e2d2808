// api_potentials.cpp -- LjNd, PhaseField and BarAndHinge of the C++ API.
// Setters and defaults follow the reference (include/potentials/*.h,
// src/potentials/{LjNd,PhaseField,BarAndHinge}.cpp setters); the energy is
// evaluated on the GPU through the device instance made by createDevice().
#include <cmath>
#include <stdexcept>

#include "minim.h"

namespace minim {

void throw_gpu(int rc);

// ---- LjNd -----------------------------------------------------------------------------
void LjNd::init(const vector<double>& coords) {
  if (coords.size() % nDim != 0)
    throw std::invalid_argument("LjNd: Length of coords must be a multiple of the number of dimensions.");
  nParticle = (int)(coords.size() / nDim);
}

// One pair element (src/potentials/LjNd.cpp:29-53), for callers that
// evaluate elements themselves; the State uses the GPU.
void LjNd::elementEnergyGradient(const vector<double>& x, const Element& el, double* e,
                                 vector<double>* g) const {
  double dx[3] = {0, 0, 0}, r2 = 0;
  for (int d = 0; d < nDim; d++) {
    dx[d] = x[el.idof[d]] - x[el.idof[nDim + d]];
    r2 += dx[d] * dx[d];
  }
  if (cutoff > 0 && r2 >= cutoff * cutoff) return;
  const double lj6 = std::pow(sigma, 6) / std::pow(r2, 3);
  const double lj12 = lj6 * lj6;
  if (e) *e += 4 * epsilon * (lj12 - lj6);
  if (g) {
    const double f = -24 * epsilon * (2 * lj12 - lj6) / r2;
    for (int d = 0; d < nDim; d++) {
      (*g)[el.idof[d]] += dx[d] * f;
      (*g)[el.idof[nDim + d]] -= dx[d] * f;
    }
  }
}

minim_gpu_handle LjNd::createDevice(const vector<double>& coords) const {
  minim_gpu_lj_params p{nDim, sigma, epsilon, cutoff};
  minim_gpu_handle h = nullptr;
  throw_gpu(minim_gpu_instance_create(MINIM_GPU_LJ, &p, coords.data(), coords.size(), &h));
  return h;
}

LjNd& LjNd::setSigma(double s) {
  sigma = s;
  return *this;
}
LjNd& LjNd::setEpsilon(double e) {
  epsilon = e;
  return *this;
}
LjNd& LjNd::setCutoff(double rc) {
  if (!(rc >= 0)) throw std::invalid_argument("LjNd: the cutoff must be >= 0.");
  cutoff = rc;
  return *this;
}

// ---- PhaseField -----------------------------------------------------------------------
PhaseField& PhaseField::setNFluid(int n) {
  nFluid = n;
  dofPerNode = n;
  return *this;
}
PhaseField& PhaseField::setGridSize(vector<int> g) {
  gridSize = g;
  nGrid = g[0] * g[1] * g[2];
  return *this;
}
PhaseField& PhaseField::setResolution(double r) {
  resolution = r;
  return *this;
}
PhaseField& PhaseField::setInterfaceSize(double w) {
  interfaceSize = vector<double>(nFluid, w);
  return *this;
}
PhaseField& PhaseField::setInterfaceSize(vector<double> w) {
  interfaceSize = w;
  return *this;
}
PhaseField& PhaseField::setSurfaceTension(double s) {
  surfaceTension = vector<double>(nFluid, s);
  return *this;
}
PhaseField& PhaseField::setSurfaceTension(vector<double> s) {
  surfaceTension = s;
  return *this;
}
PhaseField& PhaseField::setSurfaceTension(std::function<vector<double>(int, int, int)> fn) {
  const int np = (int)fn(0, 0, 0).size();
  surfaceTension.assign((size_t)nGrid * np, 0.0);
  size_t k = 0;
  for (int i = 0; i < gridSize[0]; i++)
    for (int j = 0; j < gridSize[1]; j++)
      for (int l = 0; l < gridSize[2]; l++)
        for (double v : fn(i, j, l)) surfaceTension[k++] = v;
  return *this;
}
PhaseField& PhaseField::setDensityConstraint(std::string m) {
  if (m == "gradient" || m == "hard") densityConstraint = MINIM_PF_DENSITY_HARD;
  else if (m == "energy penalty" || m == "soft") densityConstraint = MINIM_PF_DENSITY_SOFT;
  else if (m == "none") densityConstraint = MINIM_PF_DENSITY_NONE;
  else if (m == "fixed") densityConstraint = MINIM_PF_DENSITY_FIXED;
  else
    throw std::invalid_argument(
        "PhaseField: Invalid density constraint. Allowed methods are: fixed, none, gradient / hard, or energy penalty / soft");
  return *this;
}
PhaseField& PhaseField::setPressure(vector<double> p) {
  pressure = p;
  return *this;
}
PhaseField& PhaseField::setVolume(vector<double> v, double c) {
  volumeFixed = true;
  volConst = c;
  volume = v;
  return *this;
}
PhaseField& PhaseField::setVolumeFixed(bool f, double c) {
  volumeFixed = f;
  volConst = c;
  return *this;
}
PhaseField& PhaseField::setSolid(vector<char> s) {
  solid = s;
  return *this;
}
PhaseField& PhaseField::setSolid(std::function<bool(int, int, int)> fn) {
  solid.assign(nGrid, 0);
  size_t k = 0;
  for (int i = 0; i < gridSize[0]; i++)
    for (int j = 0; j < gridSize[1]; j++)
      for (int l = 0; l < gridSize[2]; l++) solid[k++] = fn(i, j, l);
  return *this;
}
PhaseField& PhaseField::setContactAngle(double a) {
  contactAngle = vector<double>(nGrid, a);
  return *this;
}
PhaseField& PhaseField::setContactAngle(vector<double> a) {
  contactAngle = a;
  return *this;
}
PhaseField& PhaseField::setContactAngle(std::function<double(int, int, int)> fn) {
  contactAngle.assign(nGrid, 0.0);
  size_t k = 0;
  for (int i = 0; i < gridSize[0]; i++)
    for (int j = 0; j < gridSize[1]; j++)
      for (int l = 0; l < gridSize[2]; l++) contactAngle[k++] = fn(i, j, l);
  return *this;
}
PhaseField& PhaseField::setForce(vector<double> f, vector<int> iFluid) {
  if (f.size() != 3) throw std::invalid_argument("PhaseField: Invalid size of force array.");
  if (nFluid == 1 || iFluid.empty()) {
    force = vector<vector<double>>(nFluid, f);
  } else {
    force = vector<vector<double>>(nFluid, {0, 0, 0});
    for (int i : iFluid) force[i] = f;
  }
  return *this;
}
PhaseField& PhaseField::setFixFluid(int i, bool fix) {
  if ((int)fixFluid.size() != nFluid) fixFluid = vector<char>(nFluid, false);
  fixFluid[i] = fix;
  return *this;
}
PhaseField& PhaseField::setConfinement(vector<double> s) {
  confinementStrength = s;
  return *this;
}

void PhaseField::init(const vector<double>& coords) {
  if ((int)coords.size() != nGrid * nFluid)
    throw std::invalid_argument("PhaseField: Size of coordinates array does not match the grid size.");
  double mean = 0;
  for (double s : surfaceTension) mean += s;
  mean /= surfaceTension.empty() ? 1 : surfaceTension.size();
  convergence = 1e-8 * mean * std::pow(resolution, 2);
  if (densityConstraint == MINIM_PF_DENSITY_FIXED) setFixFluid(nFluid - 1, true);
}

minim_gpu_pf_params PhaseField::deviceParams(std::vector<double>& st, std::vector<double>& iw,
                                            std::vector<double>& ca, std::vector<double>& fo,
                                            std::vector<char>& fx, std::vector<double>& cf,
                                            std::vector<double>& pr, std::vector<double>& vol) const {
  minim_gpu_pf_params p;
  minim_gpu_default_pf(&p);
  for (int d = 0; d < 3; d++) p.grid[d] = gridSize.size() > (size_t)d ? gridSize[d] : 1;
  p.nfluid = nFluid;
  p.resolution = resolution;
  iw = interfaceSize;
  p.n_interface_size = (int)iw.size();
  p.interface_size = iw.empty() ? nullptr : iw.data();
  st = surfaceTension;
  p.n_surface_tension = (int)st.size();
  p.surface_tension = st.empty() ? nullptr : st.data();
  p.density_constraint = densityConstraint;
  p.density_const = densityConst;
  p.volume_fixed = volumeFixed;
  p.vol_const = volConst;
  vol = volume;
  p.volume = vol.empty() ? nullptr : vol.data();
  pr = pressure;
  p.pressure = pr.empty() ? nullptr : pr.data();
  p.solid = solid.empty() ? nullptr : solid.data();
  ca = contactAngle;
  p.n_contact_angle = (int)ca.size();
  p.contact_angle = ca.empty() ? nullptr : ca.data();
  fo.clear();
  for (const auto& f : force) fo.insert(fo.end(), f.begin(), f.end());
  p.force = fo.empty() ? nullptr : fo.data();
  fx = fixFluid;
  p.fix_fluid = fx.empty() ? nullptr : fx.data();
  cf = confinementStrength;
  p.confinement = cf.empty() ? nullptr : cf.data();
  return p;
}

minim_gpu_handle PhaseField::createDevice(const vector<double>& coords) const {
  std::vector<double> st, iw, ca, fo, cf, pr, vol;
  std::vector<char> fx;
  minim_gpu_pf_params p = deviceParams(st, iw, ca, fo, fx, cf, pr, vol);
  minim_gpu_handle h = nullptr;
  throw_gpu(minim_gpu_instance_create(MINIM_GPU_PF, &p, coords.data(), coords.size(), &h));
  return h;
}

// PhaseFieldUnstructured (src/potentials/PhaseFieldUnstructured.cpp): the
// same description, created as the element-form kind.
minim_gpu_handle PhaseFieldUnstructured::createDevice(const vector<double>& coords) const {
  std::vector<double> st, iw, ca, fo, cf, pr, vol;
  std::vector<char> fx;
  minim_gpu_pf_params p = deviceParams(st, iw, ca, fo, fx, cf, pr, vol);
  minim_gpu_handle h = nullptr;
  throw_gpu(minim_gpu_instance_create(MINIM_GPU_PFU, &p, coords.data(), coords.size(), &h));
  return h;
}

// diffuseSolid (src/potentials/PhaseField.cpp:998-1035): relax a solid mask
// into a smooth field with a confinement potential, L-BFGS without line
// search for at most 100 iterations (optionally twice).
vector<double> PhaseField::diffuseSolid(vector<char> s, int iFluid, bool twoStep) {
  return diffuseSolid(s, *this, iFluid, twoStep);
}
vector<double> PhaseField::diffuseSolid(vector<char> s, vector<int> g, int nf, int iFluid, bool twoStep) {
  PhaseField pf;
  pf.setNFluid(nf);
  pf.setGridSize(g);
  return diffuseSolid(s, pf, iFluid, twoStep);
}
vector<double> PhaseField::diffuseSolid(vector<char> s, PhaseField pf, int iFluid, bool twoStep) {
  vector<double> conf(pf.nFluid, 0.0);
  conf[iFluid] = 100;
  pf.setConfinement(conf);
  pf.setDensityConstraint("none");
  const int ng = pf.gridSize[0] * pf.gridSize[1] * pf.gridSize[2];
  vector<double> init((size_t)pf.nFluid * ng, 0.0);
  for (int i = 0; i < ng; i++) init[(size_t)i * pf.nFluid + iFluid] = (int)s[i];
  State state(pf, init);
  state.convergence = 1e-8 * pf.surfaceTension[iFluid] * std::pow(pf.resolution, 2);
  Lbfgs min;
  min.setLinesearch("none");
  min.setMaxIter(100);
  vector<double> x = min.minimise(state);
  if (twoStep) {
    state = State(pf, x);
    x = min.minimise(state);
  }
  return x;
}

// ---- BarAndHinge ----------------------------------------------------------------------
void BarAndHinge::init(const vector<double>& coords) {
  if (coords.size() % 3) throw std::invalid_argument("BarAndHinge: coordinates must be 3 per vertex");
}

namespace {
template <typename T>
vector<int> flatten(const vector2d<T>& v, int& stride) {
  stride = 0;
  for (const auto& r : v) stride = std::max<int>(stride, (int)r.size());
  vector<int> out(v.size() * stride, 0);
  for (size_t i = 0; i < v.size(); i++)
    for (size_t j = 0; j < v[i].size(); j++) out[i * stride + j] = v[i][j];
  return out;
}
}  // namespace

minim_gpu_handle BarAndHinge::createDevice(const vector<double>& coords) const {
  minim_gpu_bah_params p;
  minim_gpu_default_bah(&p);
  int ts = 0, bs = 0, hs = 0;
  const vector<int> tri = flatten(_triList, ts);
  const vector<int> bonds = flatten(_bondList, bs);
  const vector<int> hinges = flatten(_hingeList, hs);
  if (!_triList.empty()) {
    if (ts != 3) throw std::invalid_argument("BarAndHinge: triangles must have 3 vertices");
    p.ntri = (int)_triList.size();
    p.tris = tri.data();
  }
  if (!_bondList.empty()) {
    p.nbond = (int)_bondList.size();
    p.bonds = bonds.data();
    p.bond_stride = bs;
  }
  if (!_hingeList.empty()) {
    p.nhinge = (int)_hingeList.size();
    p.hinges = hinges.data();
    p.hinge_stride = hs;
  }
  p.modulus = modulus;
  p.poisson_ratio = poissonRatio;
  p.n_thickness = (int)thickness.size();
  p.thickness = thickness.data();
  p.n_kbond = (int)kBond.size();
  p.kbond = kBond.data();
  p.n_khinge = (int)kHinge.size();
  p.khinge = kHinge.data();
  p.n_length0 = (int)length0.size();
  p.length0 = length0.data();
  p.n_theta0 = (int)theta0.size();
  p.theta0 = theta0.data();
  p.n_force = (int)force.size();
  p.force = force.data();
  p.wall_on = wallOn;
  p.wall_adhesion = wallAdhesion;
  p.wall_epsilon = lj_epsilon;
  p.wall_sigma = lj_sigma;
  minim_gpu_handle h = nullptr;
  throw_gpu(minim_gpu_instance_create(MINIM_GPU_BAH, &p, coords.data(), coords.size(), &h));
  // elements with all dofs fixed are dropped once the fixed dofs are known
  return h;
}

BarAndHinge& BarAndHinge::setTriangulation(const vector2d<int>& t) {
  _triList = t;
  return *this;
}
BarAndHinge& BarAndHinge::setBondList(const vector2d<int>& b) {
  _bondList = b;
  return *this;
}
BarAndHinge& BarAndHinge::setHingeList(const vector2d<int>& h) {
  _hingeList = h;
  return *this;
}
BarAndHinge& BarAndHinge::setModulus(double m) {
  modulus = m;
  return *this;
}
BarAndHinge& BarAndHinge::setThickness(double t) {
  thickness = {t};
  return *this;
}
BarAndHinge& BarAndHinge::setThickness(const vector<double>& t) {
  thickness = t;
  return *this;
}
BarAndHinge& BarAndHinge::setRigidity(double kb, double kh) {
  kBond = {kb};
  kHinge = {kh};
  return *this;
}
BarAndHinge& BarAndHinge::setRigidity(const vector<double>& kb, const vector<double>& kh) {
  if (!kb.empty()) kBond = kb;
  if (!kh.empty()) kHinge = kh;
  return *this;
}
BarAndHinge& BarAndHinge::setLength0(double l) {
  length0 = {l};
  return *this;
}
BarAndHinge& BarAndHinge::setLength0(const vector<double>& l) {
  length0 = l;
  return *this;
}
BarAndHinge& BarAndHinge::setTheta0(double t) {
  theta0 = {t};
  return *this;
}
BarAndHinge& BarAndHinge::setTheta0(const vector<double>& t) {
  theta0 = t;
  return *this;
}
BarAndHinge& BarAndHinge::setWall(bool on) {
  wallOn = on;
  return *this;
}
BarAndHinge& BarAndHinge::setWallAdhesion(bool on) {
  wallAdhesion = on;
  return *this;
}
BarAndHinge& BarAndHinge::setWallParams(double e, double s) {
  lj_epsilon = e;
  lj_sigma = s;
  return *this;
}
BarAndHinge& BarAndHinge::setForce(const vector<double>& f) {
  force = f;
  return *this;
}
BarAndHinge& BarAndHinge::setForce(const vector2d<double>& f) {
  force.clear();
  for (const auto& v : f)
    for (int j = 0; j < 3; j++) force.push_back(v[j]);
  return *this;
}

}  // namespace minim
