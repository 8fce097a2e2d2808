// setup.h -- host-side set-up of the potentials (what the reference does in
// Potential::init / initLocal), producing the arrays the kernels read.
#pragma once
#include <stdexcept>
#include <string>
#include <vector>

#include "engine.h"
#include "minim_gpu.h"

namespace mg {

struct SetupError : std::runtime_error {
  int code;
  SetupError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// PhaseField: scalar parameters go straight into PotPF; the per-node arrays
// are returned for upload.
struct PfHost {
  PotPF pot{};
  int kernel_kind = K_PF;
  double default_tol = 0;
  std::vector<uint16_t> aux;        // empty when there is no solid
  std::vector<double> wet;          // empty without wetting
  std::vector<double> kappa_node, kappaP_node;
  std::vector<double> ff_init;
  std::vector<double> node_vol;     // per node (diagnostics / tests); empty
  std::vector<double> surface_area; // without solid nodes (all bulk)
  std::vector<double> kappa, kappaP;  // as the reference stores them
};
// unstr: PhaseFieldUnstructured semantics (src/potentials/PhaseFieldUnstructured.cpp)
PfHost setup_pf(const minim_gpu_pf_params& q, const double* x0, size_t ndof, bool unstr = false);

// BarAndHinge topology in the reference's order (computeBondList /
// computeHingeList), built with hash maps in O(T log T) instead of O(T^2).
struct BahTopology {
  std::vector<std::vector<int>> bonds;   // 2 nodes + adjacent triangle vertices
  std::vector<std::vector<int>> hinges;  // 4 nodes (+ bond index)
};
BahTopology bah_topology(const minim_gpu_bah_params& q, int nvert);

struct BahHost {
  // full element lists (before dropping fully fixed elements)
  std::vector<int> bars;       // 2 per bar
  std::vector<double> bpar;    // {k, l0}
  std::vector<int> hinges;     // 4 per hinge
  std::vector<double> hpar;    // {k, theta0}
  std::vector<double> force;
  int nvert = 0;
  int wall_on = 0, wall_adh = 0;
  double wall_eps = 0, wall_sig = 0;
};
BahHost setup_bah(const minim_gpu_bah_params& q, const double* x0, size_t ndof);
// the body force and wall of q into B (B.nvert set)
void bah_scalars(const minim_gpu_bah_params& q, BahHost& B);

// Element arrays after removing fully fixed elements and sorting by colour.
struct BahDevArrays {
  std::vector<int2> bars;
  std::vector<double2> bpar;
  std::vector<int4> hinges;
  std::vector<double2> hpar;
  std::vector<int> bar_off, hinge_off;
  std::vector<unsigned char> node_el;
};
BahDevArrays bah_arrays(const BahHost& b, const std::vector<unsigned char>& fixed);

}  // namespace mg
