// Process-level communicator stand-in.  The GB300 engine runs one process
// per GPU and needs no message passing, so `mpi` reports size 1 / rank 0 and
// every reduction is local (same interface as the minim library's utils/mpi.h).
#ifndef MINIM_GB300_MPI_H
#define MINIM_GB300_MPI_H

#include <vector>

namespace minim {
class Mpi {
 public:
  int size = 1;
  int rank = 0;
  void init() {}
  void init(int*, char***) {}
  double sum(double a) const { return a; }
  double sum(const std::vector<double>& a) const {
    double s = 0;
    for (double v : a) s += v;
    return s;
  }
  double dotProduct(const std::vector<double>& a, const std::vector<double>& b) const {
    double s = 0;
    for (size_t i = 0; i < a.size(); i++) s += a[i] * b[i];
    return s;
  }
  void bcast(int&, int = 0) const {}
  void bcast(double&, int = 0) const {}
  void bcast(std::vector<double>&, int = 0, int = 0) const {}
  void barrier() const {}
};
extern Mpi mpi;
inline void mpiInit() {}
inline void mpiInit(int*, char***) {}
}  // namespace minim

#endif
