#ifndef MINIM_GB300_PHASEFIELDUNSTRUCTURED_H
#define MINIM_GB300_PHASEFIELDUNSTRUCTURED_H

#include <memory>
#include <vector>

#include "PhaseField.h"

namespace minim {
// The element form of the phase field (the minim library's
// include/potentials/PhaseFieldUnstructured.h): the same setters as
// PhaseField, with that class's semantics -- a fixed volume is an energy
// penalty (volConst * sigma / res^4 * (V - V0)^2, its force on interface
// nodes only), DENSITY "fixed" evaluates the last fluid as 1 minus the
// others, pressure acts on fixed fluids too, the soft density constraint
// reads the first three fluids.  Evaluated on the GPU by the PhaseField
// sweep with those element semantics.
class PhaseFieldUnstructured : public PhaseField {
 public:
  int potentialType() const override { return Potential::UNSTRUCTURED; }
  std::unique_ptr<Potential> clone() const override { return std::make_unique<PhaseFieldUnstructured>(*this); }
  minim_gpu_handle createDevice(const vector<double>& coords) const override;
};
}  // namespace minim

#endif
