#ifndef MINIM_GB300_GRADDESCENT_H
#define MINIM_GB300_GRADDESCENT_H

#include <vector>

#include "../Minimiser.h"

namespace minim {
// Gradient descent: step = -alpha * g (alpha = 0.1), optional line search.
class GradDescent : public NewMinimiser<GradDescent> {
 public:
  GradDescent& setAlpha(double alpha);
  GradDescent& setMaxIter(int maxIter);

  void init(State& state) override;
  void iteration(State& state) override;
  bool checkConvergence(const State& state) override;

 protected:
  bool deviceParams(const State&, minim_gpu_minimiser_params* p) const override;

 private:
  double _alpha = 1e-1;
  std::vector<double> _g;
};
}  // namespace minim

#endif
