#ifndef MINIM_GB300_LJND_H
#define MINIM_GB300_LJND_H

#include <vector>

#include "../Potential.h"

namespace minim {
using std::vector;

// Lennard-Jones over all particle pairs, evaluated on the GPU.  setCutoff
// (not in the reference) keeps only the pairs closer than the cutoff.
class LjNd : public NewPotential<LjNd> {
 public:
  int potentialType() const override { return Potential::UNSTRUCTURED; }

  int nDim;
  int nParticle = 0;
  double sigma = 1;
  double epsilon = 1;
  double cutoff = 0;  // 0: every pair

  LjNd(int nDim) : nDim(nDim) {}
  LjNd(int nDim, double sigma, double epsilon) : nDim(nDim), sigma(sigma), epsilon(epsilon) {}

  void init(const vector<double>& coords) override;
  void elementEnergyGradient(const vector<double>& coords, const Element& el, double* e,
                             vector<double>* g) const override;
  minim_gpu_handle createDevice(const vector<double>& coords) const override;

  LjNd& setSigma(double sigma);
  LjNd& setEpsilon(double epsilon);
  // Pairs with r >= rc contribute nothing (plain truncation; 0 = every
  // pair).  No counterpart in the reference; found by a device cell list.
  LjNd& setCutoff(double rc);
};

class Lj2d : public LjNd {
 public:
  Lj2d() : LjNd(2) {}
  Lj2d(double sigma, double epsilon) : LjNd(2, sigma, epsilon) {}
  std::unique_ptr<Potential> clone() const override { return std::make_unique<Lj2d>(*this); }
};

class Lj3d : public LjNd {
 public:
  Lj3d() : LjNd(3) {}
  Lj3d(double sigma, double epsilon) : LjNd(3, sigma, epsilon) {}
  std::unique_ptr<Potential> clone() const override { return std::make_unique<Lj3d>(*this); }
};
}  // namespace minim

#endif
