#ifndef MINIM_GB300_FIRE_H
#define MINIM_GB300_FIRE_H

#include <vector>

#include "../Minimiser.h"

namespace minim {
// FIRE as in the reference: Fire() keeps the backtracking line search and
// estimates dtMax = 0.1/sqrt(|g|); Fire(dtMax) uses no line search.
class Fire : public NewMinimiser<Fire> {
 public:
  Fire() = default;
  Fire(double dtMax);

  double dtMax = 0;

  Fire& setMaxIter(int maxIter);
  Fire& setDtMax(double dtMax);

  void init(State& state) override;
  void iteration(State& state) override;
  bool checkConvergence(const State& state) override;

 protected:
  bool deviceParams(const State&, minim_gpu_minimiser_params* p) const override;
  void deviceDone(const minim_gpu_result& r) override { dtMax = r.dt_max; }

 private:
  int _nMin = 5;
  double _fInc = 1.1;
  double _fDec = 0.5;
  double _fA = 0.99;
  double _aStart = 0.1;
  int _nSteps = 0;
  double _a = 0;
  double _dt = 0;
  double _gNorm = 0;
  std::vector<double> _g;
  std::vector<double> _v;
};
}  // namespace minim

#endif
