// Potential: base of every energy function (same public interface as the
// minim library's Potential.h).  User potentials (function pointers or
// subclasses) are evaluated on the host; the built-in LjNd, PhaseField and
// BarAndHinge report themselves as device potentials and are evaluated and
// minimised by the GB300 engine through the C ABI in minim_gpu.h.
#ifndef MINIM_GB300_POTENTIAL_H
#define MINIM_GB300_POTENTIAL_H

#include <functional>
#include <memory>
#include <vector>

#include "minim_gpu.h"

namespace minim {
class State;
class Communicator;
using std::vector;
template <typename T> using vector2d = vector<vector<T>>;

class Potential {
  typedef double (*EFunc)(const vector<double>&);
  typedef vector<double> (*GFunc)(const vector<double>&);
  typedef void (*EGFunc)(const vector<double>&, double*, vector<double>*);
  EFunc _energy;
  GFunc _gradient;
  EGFunc _energyGradient;

 public:
  double convergence = 1e-6;

  Potential(EFunc energy, GFunc gradient);
  Potential(EGFunc energyGradient);

  virtual double energy(const vector<double>& coords) const;
  virtual vector<double> gradient(const vector<double>& coords) const;
  virtual void energyGradient(const vector<double>& coords, const Communicator& comm, double* e,
                              vector<double>* g) const;

  State newState(int ndof, const vector<int>& ranks = {});
  State newState(const vector<double>& coords, const vector<int>& ranks = {});

  struct Constraint {
    using NormalFn = std::function<vector<double>(const vector<int>&, const vector<double>&)>;
    using CorrectionFn = std::function<void(const vector<int>&, vector<double>&)>;
    vector<int> idof;
    NormalFn normalFn;
    CorrectionFn correction = nullptr;
    vector<double> normal(const vector<double>& x) const { return normalFn(idof, x); }
  };
  vector<Constraint> constraints;

  Potential& setConstraints(vector<int> iFix);
  Potential& setConstraints(vector2d<int> idofs, vector<double> normal);
  Potential& setConstraints(vector2d<int> idofs, Constraint::NormalFn normal,
                            Constraint::CorrectionFn correction = nullptr);

  void applyConstraints(const vector<double>& coords, const Communicator& comm, vector<double>& step) const;
  void correctConstraints(vector<double>& coords) const;
  virtual void specialisedConstraints(const vector<double>&, const Communicator&, vector<double>&) const {}

  bool isFixed(int index) const;
  vector<char> isFixed(const vector<int>& indices) const;
  vector<int> fixedDofs() const;
  bool hasNormalConstraints() const;

  virtual void init(const vector<double>&) {}
  virtual void initLocal(const vector<double>&, const Communicator&) {}
  bool isSerial() const { return potentialType() == SERIAL; }

  virtual ~Potential() = default;
  virtual std::unique_ptr<Potential> clone() const { return std::make_unique<Potential>(*this); }

  enum { SERIAL = 0, UNSTRUCTURED = 1, GRID = 2 };
  virtual int potentialType() const { return SERIAL; }
  std::unique_ptr<Communicator> newComm() const;

  // UNSTRUCTURED user potentials: energy elements evaluated on the host
  bool distributed = false;
  struct Element {
    int type;
    vector<int> idof;
    vector<double> parameters;
  };
  vector<Element> elements;
  vector<Element> elements_halo;
  Potential& setElements(vector<Element> elements);
  Potential& setElements(vector2d<int> idofs);
  Potential& setElements(vector2d<int> idofs, vector<int> types, vector2d<double> parameters);
  virtual void elementEnergyGradient(const vector<double>&, const Element&, double*, vector<double>*) const {}
  virtual void blockEnergyGradient(const vector<double>&, const Communicator&, double*, vector<double>*) const {}

  // GRID
  int dofPerNode = 1;
  int haloWidth = 1;
  vector<int> gridSize;
  vector<int> commArray;
  Potential& setCommArray(vector<int> commArray);

  // GB300 engine: a device potential creates its device instance here (the
  // State owns the handle).  Host potentials return nullptr.
  virtual minim_gpu_handle createDevice(const vector<double>& coords) const {
    (void)coords;
    return nullptr;
  }

 protected:
  Potential() : _energy(nullptr), _gradient(nullptr), _energyGradient(nullptr) {}
};

template <typename Derived>
class NewPotential : public Potential {
 public:
  std::unique_ptr<Potential> clone() const override {
    return std::make_unique<Derived>(static_cast<const Derived&>(*this));
  }
  Derived& setElements(vector<Element> e) { return static_cast<Derived&>(Potential::setElements(e)); }
  Derived& setElements(vector2d<int> idofs) { return static_cast<Derived&>(Potential::setElements(idofs)); }
  Derived& setElements(vector2d<int> idofs, vector<int> types, vector2d<double> parameters) {
    return static_cast<Derived&>(Potential::setElements(idofs, types, parameters));
  }
  Derived& setConstraints(vector<int> iFix) { return static_cast<Derived&>(Potential::setConstraints(iFix)); }
  Derived& setConstraints(vector2d<int> idofs, vector<double> normal) {
    return static_cast<Derived&>(Potential::setConstraints(idofs, normal));
  }
  Derived& setConstraints(vector2d<int> idofs, Constraint::NormalFn normal,
                          Constraint::CorrectionFn correction = nullptr) {
    return static_cast<Derived&>(Potential::setConstraints(idofs, normal, correction));
  }
};
}  // namespace minim

#endif
