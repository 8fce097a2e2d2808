#ifndef MINIM_GB300_BARANDHINGE_H
#define MINIM_GB300_BARANDHINGE_H

#include <vector>

#include "../Potential.h"

namespace minim {
using std::vector;

// Triangulated elastic sheet: bar stretching, hinge bending, external force
// and substrate wall, evaluated on the GPU (coloured element kernels).
class BarAndHinge : public NewPotential<BarAndHinge> {
 public:
  int potentialType() const override { return Potential::UNSTRUCTURED; }

  void init(const vector<double>& coords) override;
  minim_gpu_handle createDevice(const vector<double>& coords) const override;

  BarAndHinge& setTriangulation(const vector2d<int>& triList);
  BarAndHinge& setBondList(const vector2d<int>& bondList);
  BarAndHinge& setHingeList(const vector2d<int>& hingeList);

  BarAndHinge& setModulus(double modulus);
  BarAndHinge& setThickness(double thickness);
  BarAndHinge& setThickness(const vector<double>& thickness);
  BarAndHinge& setRigidity(double kBond, double kHinge);
  BarAndHinge& setRigidity(const vector<double>& kBond, const vector<double>& kHinge);
  BarAndHinge& setLength0(double length0);
  BarAndHinge& setLength0(const vector<double>& length0);
  BarAndHinge& setTheta0(double theta0);
  BarAndHinge& setTheta0(const vector<double>& theta0);

  BarAndHinge& setWall(bool wallOn = true);
  BarAndHinge& setWallAdhesion(bool wallAdhesion = true);
  BarAndHinge& setWallParams(double epsilon, double sigma);

  BarAndHinge& setForce(const vector<double>& force);
  BarAndHinge& setForce(const vector2d<double>& force);

  double modulus = 1;
  double poissonRatio = 0.3;
  bool wallOn = false;
  bool wallAdhesion = false;
  double lj_epsilon = 1e-12;
  double lj_sigma = 1e-5;

 private:
  vector2d<int> _bondList;
  vector2d<int> _hingeList;
  vector2d<int> _triList;
  vector<double> thickness;
  vector<double> kBond;
  vector<double> kHinge;
  vector<double> length0;
  vector<double> theta0;
  vector<double> force;
};
}  // namespace minim

#endif
