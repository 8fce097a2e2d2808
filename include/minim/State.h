// State: a potential plus its coordinates (same public interface as the minim
// library's State.h).  For a device potential the State also owns the GB300
// engine instance: energies and gradients are evaluated on the GPU, and
// Lbfgs / Fire / GradDescent minimise it device-resident.
#ifndef MINIM_GB300_STATE_H
#define MINIM_GB300_STATE_H

#include <cstddef>
#include <memory>
#include <vector>

#include "Communicator.h"
#include "Potential.h"
#include "minim_gpu.h"

namespace minim {
using std::vector;

class State {
 public:
  size_t ndof;
  double convergence;
  std::unique_ptr<Potential> pot;
  std::unique_ptr<Communicator> comm;
  bool usesThisProc = true;

  State(const Potential& pot, const vector<double>& coords, const vector<int>& ranks = {});
  State(const State& state);
  State& operator=(const State& state);
  ~State();

  double energy() const;
  double energy(const vector<double>& coords) const;
  vector<double> gradient() const;
  vector<double> gradient(const vector<double>& coords) const;
  void energyGradient(double* e, vector<double>* g) const;
  void energyGradient(const vector<double>& coords, double* e, vector<double>* g) const;

  double operator[](int i);
  vector<double> coords() const;
  void coords(const vector<double>& in);

  const vector<double>& blockCoords() const;
  void blockCoords(const vector<double>& in);

  double blockEnergy() const;
  double blockEnergy(const vector<double>& coords) const;
  vector<double> blockGradient() const;
  vector<double> blockGradient(const vector<double>& coords) const;
  void blockEnergyGradient(double* e, vector<double>* g) const;
  void blockEnergyGradient(const vector<double>& coords, double* e, vector<double>* g) const;

  double procEnergy() const;
  double procEnergy(const vector<double>& coords) const;
  vector<double> procGradient() const;
  vector<double> procGradient(const vector<double>& coords) const;
  void procEnergyGradient(double* e, vector<double>* g) const;
  void procEnergyGradient(const vector<double>& coords, double* e, vector<double>* g) const;

  double allEnergy() const;
  vector<double> allGradient() const;
  void allEnergyGradient(double* e, vector<double>* g) const;
  vector<double> allCoords() const;

  double componentEnergy(int component) const;
  void communicate() {}
  void applyConstraints(vector<double>& data) const;

  bool isFailed = false;
  void failed() { isFailed = true; }

  vector<double> _coords;

  // GB300 engine instance of a device potential (nullptr for host potentials)
  minim_gpu_handle device() const { return dev_; }

 private:
  minim_gpu_handle dev_ = nullptr;
  void attachDevice();
};
}  // namespace minim

#endif
