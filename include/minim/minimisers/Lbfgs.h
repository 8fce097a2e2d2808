#ifndef MINIM_GB300_LBFGS_H
#define MINIM_GB300_LBFGS_H

#include <vector>

#include "../Minimiser.h"

namespace minim {
using std::vector;
class Communicator;

// L-BFGS with the reference's defaults: m = 5, maxStep = 0 (off), initStep = 1.
class Lbfgs : public NewMinimiser<Lbfgs> {
 public:
  Lbfgs& setM(int m);
  Lbfgs& setMaxIter(int maxIter);
  Lbfgs& setMaxStep(double maxStep);
  Lbfgs& setInitStep(double initStep);

  void init(State& state) override;
  void iteration(State& state) override;
  bool checkConvergence(const State& state) override;

 protected:
  bool deviceParams(const State&, minim_gpu_minimiser_params* p) const override;

 private:
  int _m = 5;
  int _i = 0;
  double _maxStep = 0;
  double _initStep = 1;
  vector<double> _g;
  vector<double> _rho;
  vector<vector<double>> _s;
  vector<vector<double>> _y;
  vector<double> getDirection(const Communicator& comm);
};
}  // namespace minim

#endif
