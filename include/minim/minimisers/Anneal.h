#ifndef MINIM_GB300_ANNEAL_H
#define MINIM_GB300_ANNEAL_H

#include <cstdint>
#include <functional>
#include <vector>

#include "../Minimiser.h"

namespace minim {
// Simulated annealing (the minim library's include/minimisers/Anneal.h):
// every coordinate moves by displacement * U(-1, 1) from the last accepted
// state, accepted by the Metropolis rule at T = tempInit / (1 +
// coolingRate * iter) or T = coolingSchedule(iter); converged after
// maxRejections consecutive rejections (0: never).  The random numbers are a
// counter-based hash of (seed, iter, index), the same on the host loop and on
// the GPU; seed 0 takes the clock, as the library's srand(time(0) + rank).
class Anneal : public NewMinimiser<Anneal> {
 public:
  Anneal(double tempInit, double displacement) : displacement(displacement), tempInit(tempInit) {}

  double displacement;
  double tempInit;
  double coolingRate = 1;
  std::function<double(int)> coolingSchedule = nullptr;
  int maxRejections = 0;
  uint64_t seed = 0;  // GB300 engine extension: a fixed random stream

  Anneal& setDisplacement(double displacement);
  Anneal& setTempInit(double tempInit);
  Anneal& setCoolingRate(double coolingRate);
  Anneal& setCoolingSchedule(std::function<double(int)> coolingSchedule);
  Anneal& setMaxIter(int maxIter);
  Anneal& setMaxRejections(int maxRejections);
  Anneal& setSeed(uint64_t seed);

  void init(State& state) override;
  void iteration(State& state) override;
  bool checkConvergence(const State& state) override;

 protected:
  // the schedule is tabulated for iterations 0..maxIter (at most 2^24
  // entries; later iterations take the last one)
  bool deviceParams(const State&, minim_gpu_minimiser_params* p) const override;

 private:
  int _sinceAccepted = 0;
  double _temp = 0;
  double _currentE = 0;
  uint64_t _seed = 0;
  std::vector<double> _currentState;
  mutable std::vector<double> _table;
  bool acceptMetropolis(double energy);
};
}  // namespace minim

#endif
