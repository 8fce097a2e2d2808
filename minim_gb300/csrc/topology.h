// topology.h -- BarAndHinge set-up on the device (topology.cu).
#pragma once
#include <cuda_runtime.h>

#include "minim_gpu.h"

namespace mg {

// Elements of a triangulation in the reference's order, before fixed-DOF
// filtering and colouring (device arrays, owned by the caller).
struct BahTopoDev {
  int nvert = 0, nbar = 0, nhinge = 0;
  int2* bars = nullptr;       // {a, b}
  double2* bpar = nullptr;    // {k, l0}
  int4* hinges = nullptr;     // 4 nodes
  double2* hpar = nullptr;    // {k, theta0}
};

// Elements without the fully fixed ones, ordered by colour (device arrays,
// owned by the caller); the offsets have ncolors + 1 entries.
struct BahColouredDev {
  int nbar = 0, nhinge = 0, nbar_colors = 0, nhinge_colors = 0;
  int2* bars = nullptr;
  double2* bpar = nullptr;
  int4* hinges = nullptr;
  double2* hpar = nullptr;
  int* bar_off = nullptr;
  int* hinge_off = nullptr;
  unsigned char* node_el = nullptr;
};

enum TopoResult { MG_TOPO_OK = 0, MG_TOPO_HOST = 1, MG_TOPO_INVALID = 2, MG_TOPO_CUDA = 3 };

}  // namespace mg

extern "C" {
// Bonds, hinges and their parameters of the triangulation in q (which must
// have no explicit bond / hinge lists) with host coordinates x0.  Returns a
// TopoResult: MG_TOPO_HOST when the triangulation needs the host builder,
// MG_TOPO_INVALID with the message in err for invalid parameters.
int mg_bah_topology_device(const minim_gpu_bah_params* q, const double* x0, int nvert, mg::BahTopoDev* out,
                           void* stream, char* err, int errlen);
// Drops the elements whose coordinates are all fixed (fixed: 3 per vertex on
// the host, or NULL), colours the rest and orders them by colour.
int mg_bah_colour_device(const mg::BahTopoDev* t, const unsigned char* fixed, mg::BahColouredDev* out,
                         void* stream);
void mg_bah_free_device(void* p, void* stream);
}
