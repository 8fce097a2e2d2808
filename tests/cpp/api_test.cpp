// The reference library's unit tests, restated against the source-compatible
// C++ API (include/minim/minim.h): same calls, same expected values.
//   test/unit/State_test.cpp, Fire_test.cpp, Potential_test.cpp,
//   BarAndHinge_test.cpp, PhaseField_test.cpp, PhaseFieldUnstructured_test.cpp,
//   Lbfgs_test.cpp; examples/toy2d (Anneal)
// Usage: api_test host   (host potentials only; no GPU needed)
//        api_test all    (also the GPU-evaluated built-in potentials)
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <string>
#include <vector>

#include "minim.h"

using namespace minim;
typedef std::vector<double> Vector;

static int g_fail = 0, g_pass = 0;
#define CHECK(cond)                                                        \
  do {                                                                     \
    if (cond) g_pass++;                                                    \
    else { g_fail++; std::printf("FAIL %s:%d  %s\n", __FILE__, __LINE__, #cond); } \
  } while (0)

static bool near(const Vector& a, const Vector& b, double d = 1e-6) {
  if (a.size() != b.size()) return false;
  for (size_t i = 0; i < a.size(); i++)
    if (std::fabs(a[i] - b[i]) > d) return false;
  return true;
}
static bool feq(double a, double b) { return std::fabs(a - b) <= 4 * 1.2e-7 * std::max(std::fabs(a), std::fabs(b)) + 1e-12; }

class Toy2d : public NewPotential<Toy2d> {
 public:
  double energy(const std::vector<double>& c) const override { return c[0] * c[0] + c[1] * c[1]; }
  std::vector<double> gradient(const std::vector<double>& c) const override { return 2 * c; }
};

class Quartic2d : public NewPotential<Quartic2d> {  // examples/toy2d
 public:
  double energy(const std::vector<double>& c) const override {
    return c[0] * c[0] + c[1] * c[1] + c[0] * c[0] * c[0] * c[0] + c[1] * c[1] * c[1] * c[1];
  }
  std::vector<double> gradient(const std::vector<double>& c) const override {
    return {2 * c[0] + 4 * c[0] * c[0] * c[0], 2 * c[1] + 4 * c[1] * c[1] * c[1]};
  }
};

static void host_tests() {
  {  // examples/toy2d with Anneal (a fixed seed makes the run repeatable)
    Quartic2d pot;
    Vector out[2];
    int iters[2];
    for (int k = 0; k < 2; k++) {
      State state = pot.newState({1, 4});
      Anneal min = Anneal(1, 0.1).setMaxIter(20000).setSeed(42);
      out[k] = min.minimise(state);
      iters[k] = min.iter;
    }
    CHECK(out[0] == out[1] && iters[0] == 20001);
    CHECK(vec::norm(out[0]) < 0.1);
    State state = pot.newState({1, 4});
    Anneal m2 = Anneal(1, 0.1).setMaxRejections(30).setSeed(3);
    m2.minimise(state);
    CHECK(m2.iter < 100000 && state.energy() < 17);
  }
  {  // Fire_test TestStep
    Vector coords = {1, 4}, g = {2, 8};
    Toy2d pot;
    State state = pot.newState(coords);
    CHECK(feq(state.energy(), 17));
    CHECK(near(state.gradient(), g));
    Fire min = Fire().setMaxIter(0);
    min.minimise(state);
    double dt = 0.1 / std::pow(68, 0.25);
    Vector step = -0.5 * dt * dt * g;
    CHECK(near(state.coords(), coords + step, 1e-15));
  }
  {  // Fire_test TestConvergence
    Toy2d pot;
    State state = pot.newState({1, 4});
    state.convergence = 2e-6 / std::sqrt(2);
    Fire min = Fire();
    min.minimise(state);
    CHECK(vec::norm(state.coords()) < 1e-6);
  }
  {  // Potential_test TestConstraints
    auto efunc = [](const vector<double>& x) { return vec::dotProduct(x, x); };
    auto gfunc = [](const vector<double>& x) { return 2 * x; };
    Potential pot(+efunc, +gfunc);
    vector<double> coords{1, 2};
    auto comm = pot.newComm();
    pot.setConstraints(vector<int>{1});
    auto g = pot.gradient(coords);
    pot.applyConstraints(coords, *comm, g);
    CHECK(g == Vector({2, 0}));
    pot.constraints = {};
    pot.setConstraints(vector2d<int>{{0, 1}}, vector<double>{1, -1});
    g = pot.gradient(coords);
    pot.applyConstraints(coords, *comm, g);
    CHECK(g == Vector({3, 3}));
    pot.constraints = {};
    pot.setConstraints(vector2d<int>{{0, 1}}, [](const vector<int>&, const vector<double>& x) { return x - 1; });
    g = pot.gradient(coords);
    pot.applyConstraints(coords, *comm, g);
    CHECK(g == Vector({2, 0}));
    State s(pot, coords);
    CHECK(s.gradient() == Vector({2, 0}));
    pot.constraints = {};
    pot.setConstraints(vector<int>{1});
    CHECK(pot.isFixed(1) && !pot.isFixed(0));
  }
  {  // Lbfgs_test TestMaxIter
    Lbfgs lbfgs = Lbfgs().setMaxIter(10);
    CHECK(lbfgs.maxIter == 10);
  }
  {  // State::failed() from the adjustState callback ends the loop before
     // that iteration (src/Minimiser.cpp:33, src/State.cpp:326-328)
    Toy2d pot;
    State state = pot.newState({1, 4});
    GradDescent gd = GradDescent().setMaxIter(100);
    gd.minimise(state, [](int i, State& s) {
      if (i == 3) s.failed();
    });
    CHECK(state.isFailed && gd.iter == 3);
    State ref = pot.newState({1, 4});
    GradDescent gd3 = GradDescent().setMaxIter(2);
    gd3.minimise(ref);
    CHECK(state.coords() == ref.coords());
  }
}

static void device_tests() {
  {  // LjNd::setCutoff (no counterpart in the reference): a pair at r = 2
     // counts in full, a pair at r = 3 not at all
    Lj3d pot;
    pot.setCutoff(2.5);
    State near_ = pot.newState({0, 0, 0, 2, 0, 0});
    CHECK(feq(near_.energy(), -63. / 1024));
    State far_ = pot.newState({0, 0, 0, 3, 0, 0});
    CHECK(far_.energy() == 0);
    bool threw = false;
    try {
      Lj3d().setCutoff(-1);
    } catch (const std::invalid_argument&) {
      threw = true;
    }
    CHECK(threw);
  }
  {  // a device minimisation that produces non-finite values reports the
     // reference's failure flag; a clean one does not
    Lj3d pot;
    State bad = pot.newState({0, 0, 0, 1.1, 0, 0, 0, NAN, 0.3});
    Lbfgs().minimise(bad);
    CHECK(bad.isFailed);
    State good = pot.newState({0, 0, 0, 1.1, 0, 0, 0, 1.2, 0.3});
    Lbfgs().minimise(good);
    CHECK(!good.isFailed);
  }
  {  // State_test TestEnergyGradient / TestClone
    Lj3d pot;
    State s = pot.newState({0, 0, 0, 2, 0, 0});
    CHECK(s.device() != nullptr);
    CHECK(s.ndof == 6);
    CHECK(feq(s.energy(), -63. / 1024));
    CHECK(near(s.gradient(), {-93. / 512, 0, 0, 93. / 512, 0, 0}));
    double e2;
    Vector g2;
    s.energyGradient(&e2, &g2);
    CHECK(feq(e2, -63. / 1024));
    CHECK(near(g2, {-93. / 512, 0, 0, 93. / 512, 0, 0}));
    State c = s;
    CHECK(c.device() != nullptr && c.device() != s.device());
    CHECK(feq(c.energy(Vector{0, 0, 0, 2, 0, 0}), -63. / 1024));
  }
  {  // BarAndHinge_test TestMin (theta0 set through the setter)
    double pi = 4 * std::atan(1.0), s2 = std::sqrt(2.0), dz = s2 / 2;
    std::vector<std::pair<double, Vector>> cases = {
        {1e-6, {0, 0, 0.5 + dz, 0, -s2, 0.5 - dz, 0, s2, 0.5 - dz, 0, 0, 0.5 + dz}},
        {pi / 2, {-1, 0, 1, 0, -s2, 0, 0, s2, 0, 1, 0, 1}},
        {pi, {-s2, 0, 0.5, 0, -s2, 0.5, 0, s2, 0.5, s2, 0, 0.5}},
        {3 * pi / 2, {-1, 0, 0, 0, -s2, 1, 0, s2, 1, 1, 0, 0}},
        {2 * pi - 1e-6, {0, 0, 0.5 - dz, 0, -s2, 0.5 + dz, 0, s2, 0.5 + dz, 0, 0, 0.5 - dz}}};
    for (auto& c : cases) {
      BarAndHinge pot;
      pot.setTriangulation({{0, 1, 2}, {1, 3, 2}});
      pot.setRigidity(100, 1);
      pot.setTheta0(c.first);
      State st(pot, {-1, 0, 1, 0, -s2, 0, 0, s2, 0, 1, 0, 1});
      Lbfgs min;
      min.setPrecision("fp64");  // the folded targets need FP64 to follow the reference's path
      Vector x = min.minimise(st);
      CHECK(near(x, c.second, 1e-4));
    }
  }
  {  // PhaseField_test TestBulkEnergy
    PhaseField pot;
    State s1(pot.setGridSize({1, 1, 1}), {1}, {0});
    CHECK(feq(s1.allEnergy(), 0));
    s1.coords({0.1});
    CHECK(feq(s1.allEnergy(), 3.0 / 16 * 1.21 * 0.81));
    CHECK(near(s1.allGradient(), {-3.0 / 4 * 0.099}));
    State s2x = pot.setGridSize({5, 1, 1}).setSolid({1, 0, 0, 0, 1}).newState({0, -1, 0, 1, 0}, {0});
    State s2z = pot.setGridSize({1, 1, 5}).setSolid({1, 0, 0, 0, 1}).newState({0, -1, 0, 1, 0}, {0});
    CHECK(feq(s2x.allEnergy(), 3.0 / 16 + 1.5));
    CHECK(near(s2z.allGradient(), {0, -1.5, 0, 1.5, 0}));
    State s3y = pot.setGridSize({1, 3, 1}).setSolid({0, 1, 0}).newState({-1, 0, 1}, {0});
    CHECK(feq(s3y.allEnergy(), 3.0));
    CHECK(near(s3y.allGradient(), {-3, 0, 3}));
  }
  {  // PhaseField_test TestExternalForce / TestSurfaceEnergy / TestPressureConstraint
    PhaseField pot;
    auto sf = pot.setGridSize({2, 2, 2}).setForce({0, -2, 0}).newState({1, 1, 1, 1, 1, 1, 1, 1});
    CHECK(std::fabs(sf.energy()) < 1e-12);
    CHECK(near(sf.gradient(), {-.5, -.5, .5, .5, -.5, -.5, .5, .5}));
    PhaseField ps;
    ps.setGridSize({2, 1, 1}).setSurfaceTension(0).setContactAngle(Vector{90, 60}).setSolid({1, 0});
    auto ss = ps.newState({0.0, 0.5});
    CHECK(feq(ss.energy(), 0.5 / std::sqrt(2.0) * (-27.0 / 24)));
    PhaseField pp;
    pp.setGridSize({6, 1, 1}).setSolid({1, 0, 0, 0, 0, 1}).setPressure({10});
    auto sp = pp.newState({1, 1, 1, 1, 1, 1});
    CHECK(feq(sp.energy(), -30));
    CHECK(near(sp.gradient(), {0, -2.5, -5, -5, -2.5, 0}));
  }
  {  // PhaseField_test TestFixFluid
    PhaseField pot;
    pot.setNFluid(3).setGridSize({2, 2, 1});
    pot.setDensityConstraint("none");
    pot.setFixFluid(0);
    State s(pot, vector<double>(12, 1));
    auto g = s.gradient();
    for (int i = 0; i < 4; i++) CHECK(g[3 * i] == 0);
  }
  {  // examples/lj3d: four particles to a tetrahedron-like minimum
    Lj3d potential;
    State state(potential, {0, 0, 0, 2, 0, 0, 1, 1, 0, 5, 1, 1});
    state.convergence = 1e-4;
    Lbfgs min;
    auto r = min.minimise(state);
    CHECK(min.iter > 0 && min.iter < 1000);
    CHECK(std::fabs(state.energy() - (-6.0)) < 1e-6);
    // the callback path (host loop, device evaluations) reaches the same minimum
    State s2(potential, {0, 0, 0, 2, 0, 0, 1, 1, 0, 5, 1, 1});
    s2.convergence = 1e-4;
    Lbfgs m2;
    int calls = 0;
    m2.minimise(s2, [&calls](int, State&) { calls++; });
    CHECK(calls > 0 && std::fabs(s2.energy() - (-6.0)) < 1e-6);
  }
  {  // PhaseFieldUnstructured_test TestPressureConstraint / TestVolumeConstraint
    PhaseFieldUnstructured pot;
    pot.setGridSize({6, 1, 1}).setSolid({1, 0, 0, 0, 0, 1}).setPressure({10});
    auto sp = pot.newState({1, 1, 1, 1, 1, 1});
    CHECK(sp.pot->potentialType() == Potential::UNSTRUCTURED);
    CHECK(feq(sp.energy(), -30));
    CHECK(near(sp.gradient(), {0, -2.5, -5, -5, -2.5, 0}));
    PhaseFieldUnstructured pv;
    pv.setGridSize({6, 1, 1});
    pv.setSolid({1, 0, 0, 0, 0, 1});
    pv.setVolumeFixed(true, 1);
    State s1(pv, {1, 1, 1, 1, 1, 1});
    CHECK(std::fabs(s1.energy()) < 1e-12);
    pv.setVolume({1}, 100);
    State s2(pv, {1, 1, 1, 1, 1, 1});
    CHECK(feq(s2.energy(), 100 * 4));
    CHECK(near(s2.gradient(), {0, 0, 0, 0, 0, 0}));
  }
  {  // Anneal on the GPU equals the host loop (same random numbers, device energies)
    Lj3d potential;
    Vector x0 = {0, 0, 0, 2, 0, 0, 1, 1, 0, 5, 1, 1};
    State a(potential, x0), b(potential, x0);
    Anneal ma = Anneal(0.2, 0.05).setMaxIter(2000).setSeed(9);
    Anneal mb = Anneal(0.2, 0.05).setMaxIter(2000).setSeed(9);
    auto xa = ma.minimise(a);
    auto xb = mb.minimise(b, [](int, State&) {});
    CHECK(ma.iter == mb.iter && near(xa, xb, 1e-12));
    CHECK(a.energy() < State(potential, x0).energy());
  }
  {  // diffuseSolid produces a smooth field between 0 and 1
    std::vector<char> solid(16 * 16, 0);
    for (int i = 0; i < 16; i++)
      for (int j = 0; j < 6; j++) solid[i * 16 + j] = 1;
    auto f = PhaseField::diffuseSolid(solid, {16, 16, 1}, 2, 0);
    double mn = 1e9, mx = -1e9;
    for (int i = 0; i < 256; i++) {
      mn = std::min(mn, f[2 * i]);
      mx = std::max(mx, f[2 * i]);
    }
    CHECK(mn > -0.2 && mx < 1.2 && mx - mn > 0.5);
  }
}

int main(int argc, char** argv) {
  const bool all = argc > 1 && std::strcmp(argv[1], "all") == 0;
  host_tests();
  if (all) device_tests();
  std::printf("%d passed, %d failed\n", g_pass, g_fail);
  return g_fail ? 1 : 0;
}
