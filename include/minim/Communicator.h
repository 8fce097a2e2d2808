// Communicator: the single-GPU device communicator.  With one process per
// GPU there is no halo exchange (periodic neighbours are read inside the
// kernels) and every reduction is local; on the device, reductions are
// deterministic FP64 block reductions inside the kernels.  Same interface as
// the minim library's Communicator for the calls user code makes.
#ifndef MINIM_GB300_COMMUNICATOR_H
#define MINIM_GB300_COMMUNICATOR_H

#include <cmath>
#include <memory>
#include <vector>

namespace minim {
using std::vector;
class Potential;

class Communicator {
 public:
  size_t ndof = 0;    // total degrees of freedom
  size_t nproc = 0;   // degrees of freedom held by this process (all of them)
  size_t nblock = 0;
  bool usesThisProc = true;
  vector<int> ranks = {0};

  int rank() const { return 0; }
  int size() const { return 1; }

  double get(const vector<double>& v, int loc) const { return v[loc]; }
  void communicate(vector<double>&) const {}
  void communicateAccumulate(vector<double>&) const {}
  vector<double> gather(const vector<double>& block, int = -1) const { return block; }
  vector<double> scatter(const vector<double>& data, int = -1) const { return data; }
  vector<double> assignBlock(const vector<double>& in) const { return in; }
  vector<double> assignProc(const vector<double>& in) const { return in; }
  void bcast(int&, int = 0) const {}
  void bcast(double&, int = 0) const {}
  void bcast(vector<double>&, int = 0) const {}

  double sum(double a) const { return a; }
  double sum(const vector<double>& a) const {
    double s = 0;
    for (double v : a) s += v;
    return s;
  }
  double dotProduct(const vector<double>& a, const vector<double>& b) const {
    double s = 0;
    for (size_t i = 0; i < a.size(); i++) s += a[i] * b[i];
    return s;
  }
  double norm(const vector<double>& a) const { return std::sqrt(dotProduct(a, a)); }

  void setup(const Potential&, size_t n, const vector<int>& = {}) { ndof = nproc = nblock = n; }
  std::unique_ptr<Communicator> clone() const { return std::make_unique<Communicator>(*this); }
};
}  // namespace minim

#endif
