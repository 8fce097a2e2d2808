#ifndef MINIM_GB300_PHASEFIELD_H
#define MINIM_GB300_PHASEFIELD_H

#include <functional>
#include <string>
#include <vector>

#include "../Potential.h"

namespace minim {
using std::vector;

// Diffuse-interface phase field on a regular periodic grid (MODEL_BASIC),
// evaluated on the GPU (7-point stencil kernels).  Setters and defaults as
// in the reference; at most 4 fluids on the device.
class PhaseField : public NewPotential<PhaseField> {
 public:
  int potentialType() const override { return Potential::GRID; }

  int nFluid = 1;
  double resolution = 1;
  PhaseField& setNFluid(int nFluid);
  PhaseField& setGridSize(vector<int> gridSize);
  PhaseField& setResolution(double resolution);

  vector<double> interfaceSize;
  vector<double> surfaceTension = {1};
  PhaseField& setInterfaceSize(double interfaceSize);
  PhaseField& setInterfaceSize(vector<double> interfaceSize);
  PhaseField& setSurfaceTension(double surfaceTension);
  PhaseField& setSurfaceTension(vector<double> surfaceTension);
  PhaseField& setSurfaceTension(std::function<vector<double>(int, int, int)> surfaceTensionFn);

  int densityConstraint = 0;
  double densityConst = 1;
  PhaseField& setDensityConstraint(std::string method);

  bool volumeFixed = false;
  double volConst = 0.01;
  vector<double> pressure;
  vector<double> volume;
  PhaseField& setPressure(vector<double> pressure);
  PhaseField& setVolume(vector<double> volume, double volConst = 0.01);
  PhaseField& setVolumeFixed(bool volumeFixed, double volConst = 0.01);

  vector<char> solid;
  vector<double> contactAngle;
  PhaseField& setSolid(vector<char> solid);
  PhaseField& setSolid(std::function<bool(int, int, int)> solidFn);
  PhaseField& setContactAngle(double contactAngle);
  PhaseField& setContactAngle(vector<double> contactAngle);
  PhaseField& setContactAngle(std::function<double(int, int, int)> contactAngleFn);

  vector<vector<double>> force;
  PhaseField& setForce(vector<double> force, vector<int> iFluid = {});

  vector<char> fixFluid;
  vector<double> confinementStrength;
  PhaseField& setFixFluid(int iFluid, bool fix = true);
  PhaseField& setConfinement(vector<double> strength);

  vector<double> diffuseSolid(vector<char> solid, int iFluid = 0, bool twoStep = false);
  static vector<double> diffuseSolid(vector<char> solid, PhaseField potential, int iFluid = 0,
                                     bool twoStep = false);
  static vector<double> diffuseSolid(vector<char> solid, vector<int> gridSize, int nFluid = 2, int iFluid = 0,
                                     bool twoStep = false);

  void init(const vector<double>& coords) override;
  minim_gpu_handle createDevice(const vector<double>& coords) const override;

  int nGrid = 1;

 protected:
  minim_gpu_pf_params deviceParams(std::vector<double>& st, std::vector<double>& iw,
                                   std::vector<double>& ca, std::vector<double>& fo,
                                   std::vector<char>& fx, std::vector<double>& cf,
                                   std::vector<double>& pr, std::vector<double>& vol) const;
};
}  // namespace minim

#endif
