// Minimiser: base of the minimisation algorithms (same interface as the minim
// library's Minimiser.h).  minimise() runs the whole minimisation on the GPU
// when the State holds a device potential and no per-iteration callback is
// given; otherwise it runs the iteration loop on the host, with the State's
// energies and gradients still evaluated on the GPU for device potentials.
#ifndef MINIM_GB300_MINIMISER_H
#define MINIM_GB300_MINIMISER_H

#include <functional>
#include <memory>
#include <string>
#include <vector>

#include "minim_gpu.h"

namespace minim {
class State;

class Minimiser {
 public:
  int maxIter = 100000;
  std::string linesearch = "backtracking";
  // GB300 engine extension: coordinate precision of device minimisations
  // ("mixed": FP32 then FP64 polish, "fp64", "fp32")
  std::string precision = "mixed";

  typedef void (*AdjustFunc)(int, State&);
  int iter = 0;
  minim_gpu_result lastResult{};  // device minimisations: status, evaluations, energy

  virtual ~Minimiser() = default;
  virtual std::unique_ptr<Minimiser> clone() const = 0;

  virtual Minimiser& setMaxIter(int maxIter);
  Minimiser& setLinesearch(std::string method);
  Minimiser& setPrecision(std::string p);

  std::vector<double> minimise(State& state, std::function<void(int, State&)> adjustState = nullptr);
  std::vector<double> minimise(State& state, std::string logType);

  virtual void init(State&) {}
  virtual void iteration(State& state) = 0;
  virtual bool checkConvergence(const State&) { return false; }

 protected:
  // Fills the device minimiser parameters; false when the algorithm has no
  // device implementation.
  virtual bool deviceParams(const State&, minim_gpu_minimiser_params*) const { return false; }
  virtual void deviceDone(const minim_gpu_result&) {}
  bool deviceMinimise(State& state);
};

template <typename Derived>
class NewMinimiser : public Minimiser {
 public:
  std::unique_ptr<Minimiser> clone() const override {
    return std::make_unique<Derived>(static_cast<const Derived&>(*this));
  }
};
}  // namespace minim

#endif
