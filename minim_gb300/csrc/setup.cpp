// setup.cpp -- host-side potential set-up (not on the iteration path).
//
//   PhaseField   PhaseField::init / assignFluidCoefficients / initLocal /
//                getType           src/potentials/PhaseField.cpp:78-235, 903-995
//   PhaseFieldUnstructured::init / checkArraySizes
//                                  src/potentials/PhaseFieldUnstructured.cpp:71-256, 929-954
//   BarAndHinge  BarAndHinge::init / computeBondList / computeHingeList /
//                computeRigidities / computeLength0 / computeTheta0
//                                  src/potentials/BarAndHinge.cpp:16-248
#include "setup.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <unordered_map>

#include <vector_functions.h>

namespace mg {

static const double kPi = 3.14159265358979323846;

// ---------------------------------------------------------------------------
// PhaseField
// ---------------------------------------------------------------------------
namespace {
const int kNei26[26][3] = {
    {-1, 0, 0}, {0, -1, 0}, {0, 0, -1}, {0, 0, 1}, {0, 1, 0}, {1, 0, 0},
    {-1, -1, 0}, {-1, 0, -1}, {-1, 0, 1}, {-1, 1, 0}, {0, -1, -1}, {0, -1, 1},
    {0, 1, -1}, {0, 1, 1}, {1, -1, 0}, {1, 0, -1}, {1, 0, 1}, {1, 1, 0},
    {-1, -1, -1}, {-1, -1, 1}, {-1, 1, -1}, {-1, 1, 1}, {1, -1, -1}, {1, -1, 1},
    {1, 1, -1}, {1, 1, 1}};

inline int wrap(int a, int n) { return ((a % n) + n) % n; }

// getType: surface classification from the 26-neighbourhood (-2: undefined)
int node_type(const std::vector<char>& solid, const int* n, int x, int y, int z) {
  auto idx = [&](int a, int b, int c) { return (wrap(a, n[0]) * n[1] + wrap(b, n[1])) * n[2] + wrap(c, n[2]); };
  if (solid[idx(x, y, z)]) return -1;
  int s[26];
  for (int d = 0; d < 26; d++) s[d] = solid[idx(x + kNei26[d][0], y + kNei26[d][1], z + kNei26[d][2])] != 0;
  int nF = s[0] + s[1] + s[2] + s[3] + s[4] + s[5], nE = 0, nC = 0;
  for (int d = 6; d < 18; d++) nE += s[d];
  for (int d = 18; d < 26; d++) nC += s[d];
  if (nF + nE + nC == 0) return 0;
  if (nF == 0) {
    if (nE == 0 && nC == 1) return 1;
    if (nE == 1 && nC <= 2) return 2;
    if (nE == 2 && nC <= 3) return 3;
  } else if (nF == 1) {
    bool one = ((s[0] || s[5]) && !(s[10] || s[11] || s[12] || s[13])) ||
               ((s[1] || s[4]) && !(s[7] || s[8] || s[15] || s[16])) ||
               ((s[2] || s[3]) && !(s[6] || s[9] || s[14] || s[17]));
    return one ? 4 : 5;
  } else if (nF == 2) {
    return 6;
  } else if (nF == 3) {
    return 7;
  }
  return -2;
}
}  // namespace

PfHost setup_pf(const minim_gpu_pf_params& q, const double* x0, size_t ndof, bool unstr) {
  PfHost H;
  PotPF& P = H.pot;
  for (int d = 0; d < 3; d++) {
    if (q.grid[d] < 1) throw SetupError(MINIM_GPU_ERR_INVALID, "PhaseField: invalid grid size");
    P.n[d] = q.grid[d];
  }
  const int nf = q.nfluid;
  if (nf < 1) throw SetupError(MINIM_GPU_ERR_INVALID, "PhaseField: invalid nFluid");
  if (nf > MINIM_MAXF)
    throw SetupError(MINIM_GPU_ERR_INVALID, "PhaseField: the device engine supports at most 4 fluids");
  const long long ngl = (long long)q.grid[0] * q.grid[1] * q.grid[2];
  if (ngl * nf > 0x7fffffffLL) throw SetupError(MINIM_GPU_ERR_INVALID, "PhaseField: grid too large");
  const int ng = (int)ngl;
  if ((size_t)ng * nf != ndof)
    throw SetupError(MINIM_GPU_ERR_INVALID, "PhaseField: Size of coordinates array does not match the grid size.");
  P.nfluid = nf;
  P.ngrid = ng;
  P.res = q.resolution;
  P.res2 = std::pow(q.resolution, 2);
  const int nparams = nf;

  // surface tensions and interface widths (assignFluidCoefficients)
  std::vector<double> st_in = (q.n_surface_tension > 0)
                                  ? std::vector<double>(q.surface_tension, q.surface_tension + q.n_surface_tension)
                                  : std::vector<double>{1.0};
  // PhaseFieldUnstructured has no per-node surface tensions and wants one
  // interface width per fluid (checkArraySizes)
  const int nkgrid = (!unstr && (int)st_in.size() == ng * nparams) ? ng : 1;
  if (unstr && q.n_interface_size != 0 && q.n_interface_size != nf)
    throw SetupError(MINIM_GPU_ERR_INVALID, "PhaseFieldUnstructured: Invalid size interfaceSize array.");
  const int nst = nkgrid * nparams;
  std::vector<double> st(nst);
  if (st_in.size() == 1) std::fill(st.begin(), st.end(), st_in[0]);
  else if ((int)st_in.size() != nst)
    throw SetupError(MINIM_GPU_ERR_INVALID, "PhaseField: Invalid size of surfaceTension array.");
  else st = st_in;
  double sum = 0;
  for (double v : st) sum += v;
  const double st_mean = sum / nst;
  std::vector<double> iw(nst);
  if (q.n_interface_size == 0) {
    for (int i = 0; i < nparams; i++) iw[i] = q.resolution;
  } else if (q.n_interface_size == 1 || q.n_interface_size == nparams) {
    for (int i = 0; i < nparams; i++) iw[i] = q.interface_size[q.n_interface_size == 1 ? 0 : i];
  } else {
    throw SetupError(MINIM_GPU_ERR_INVALID, "PhaseField: Invalid size interfaceSize array.");
  }
  for (int k = 1; k < nkgrid; k++)
    for (int j = 0; j < nparams; j++) iw[k * nparams + j] = iw[j];
  std::vector<double> kap(nst), kapP(nst);
  if (nf <= 2) {
    for (int i = 0; i < nst; i++) {
      kap[i] = 3 * st[i] / iw[i];
      kapP[i] = 3 * st[i] * iw[i];
    }
  } else {
    for (int kg = 0; kg < nkgrid; kg++) {
      const int i0 = kg * nparams;
      std::vector<double> ks(nparams), kps(nparams);
      for (int j = 0; j < nparams; j++) {
        ks[j] = 6 * st[i0 + j] / iw[i0 + j];
        kps[j] = 6 * st[i0 + j] * iw[i0 + j];
      }
      kap[i0 + 0] = 0.5 * (ks[0] + ks[1] - ks[nf - 1]);
      kap[i0 + 1] = 0.5 * (ks[0] - ks[1] + ks[nf - 1]);
      kap[i0 + 2] = 0.5 * (-ks[0] + ks[1] + ks[nf - 1]);
      kapP[i0 + 0] = 0.5 * (kps[0] + kps[1] - kps[nf - 1]);
      kapP[i0 + 1] = 0.5 * (kps[0] - kps[1] + kps[nf - 1]);
      kapP[i0 + 2] = 0.5 * (-kps[0] + kps[1] + kps[nf - 1]);
      for (int f = 3; f < nf; f++) {
        kap[i0 + f] = ks[f - 1] - kap[i0 + 0];
        kapP[i0 + f] = kps[f - 1] - kapP[i0 + 0];
      }
    }
  }
  H.kappa = kap;
  H.kappaP = kapP;
  unsigned flags = 0;
  if (nkgrid > 1) {
    flags |= PF_NODE_KAPPA;
    H.kappa_node = kap;
    H.kappaP_node = kapP;
  } else {
    for (int f = 0; f < nf; f++) {
      P.kappa[f] = kap[f];
      P.kappaP[f] = kapP[f];
    }
  }
  H.default_tol = 1e-8 * st_mean * std::pow(q.resolution, 2);

  // fluids: fixed, pressure, density constraint, confinement, force
  unsigned fix = 0;
  if (q.fix_fluid)
    for (int f = 0; f < nf; f++)
      if (q.fix_fluid[f]) fix |= 1u << f;
  if (q.density_constraint < 0 || q.density_constraint > 3)
    throw SetupError(MINIM_GPU_ERR_INVALID, "PhaseField: Invalid density constraint.");
  if (q.density_constraint == MINIM_PF_DENSITY_FIXED) fix |= 1u << (nf - 1);
  P.fix_mask = fix;
  if (fix) flags |= PF_FIXFLUID;
  P.nvar = 0;
  for (int f = 0; f < nf; f++)
    if (!((fix >> f) & 1u)) P.nvar++;
  if (nf > 1 && q.density_constraint == MINIM_PF_DENSITY_HARD) flags |= PF_HARD;
  if (nf > 1 && q.density_constraint == MINIM_PF_DENSITY_SOFT) flags |= PF_SOFT;
  P.soft_coef = q.density_const * st_mean * P.res2;
  if (q.pressure) {
    for (int f = 0; f < nf; f++) {
      P.pressure[f] = q.pressure[f];
      if (q.pressure[f] != 0) flags |= PF_PRESSURE;
    }
  }
  bool any_conf = false;
  if (q.confinement) {
    for (int f = 0; f < nf; f++) {
      P.confine_coef[f] = q.confinement[f] * st_mean * P.res2;
      if (q.confinement[f] != 0) any_conf = true;
    }
  }
  if (any_conf) {
    flags |= PF_CONFINE;
    H.ff_init.assign(x0, x0 + ndof);
  }
  if (q.force) {
    bool any = false;
    for (int f = 0; f < nf; f++) {
      const double* F = q.force + 3 * f;
      P.fmag[f] = std::sqrt(F[0] * F[0] + F[1] * F[1] + F[2] * F[2]);
      for (int d = 0; d < 3; d++) P.fnorm[f][d] = P.fmag[f] != 0 ? F[d] / P.fmag[f] : 0.0;
      if (P.fmag[f] != 0) any = true;
    }
    if (any) flags |= PF_FORCE;
  }

  // node types (initLocal / getType) and per-node arrays
  const double r3 = std::pow(q.resolution, 3), r2 = P.res2;
  P.vol_of_type[0] = 0.0;
  P.vol_of_type[1] = 1.0 * r3;
  for (int t = 1; t <= 7; t++) P.vol_of_type[t + 1] = (t / 8.0) * r3;
  // without solid nodes every node is bulk (nodeVol = res^3, surfaceArea =
  // 0) and the per-node arrays stay empty: nothing per node is built on the
  // host for such grids (a 192^3 grid would fill 113 MB here per instance)
  bool any_solid = false;
  std::vector<char> solid;
  if (q.solid) {
    solid.assign(ng, 0);
    for (int i = 0; i < ng; i++) {
      solid[i] = q.solid[i] != 0;
      any_solid |= solid[i] != 0;
    }
  }
  auto node_vol = [&](int i) { return H.node_vol.empty() ? r3 : H.node_vol[i]; };
  if (any_solid) {
    H.node_vol.assign(ng, r3);
    H.surface_area.assign(ng, 0.0);
    flags |= PF_SOLID;
    H.aux.resize(ng);
    const int* n = P.n;
    for (int x = 0; x < n[0]; x++)
      for (int y = 0; y < n[1]; y++)
        for (int z = 0; z < n[2]; z++) {
          const int i = (x * n[1] + y) * n[2] + z;
          const int t = node_type(solid, n, x, y, z);
          if (t == -2) throw SetupError(MINIM_GPU_ERR_RUNTIME, "PhaseField: Undefined surface type");
          unsigned mask = 0;
          const int nb[6] = {(wrap(x - 1, n[0]) * n[1] + y) * n[2] + z, (wrap(x + 1, n[0]) * n[1] + y) * n[2] + z,
                             (x * n[1] + wrap(y - 1, n[1])) * n[2] + z, (x * n[1] + wrap(y + 1, n[1])) * n[2] + z,
                             (x * n[1] + y) * n[2] + wrap(z - 1, n[2]), (x * n[1] + y) * n[2] + wrap(z + 1, n[2])};
          for (int k = 0; k < 6; k++)
            if (solid[nb[k]]) mask |= 1u << k;
          H.aux[i] = (uint16_t)((t + 1) | (mask << 4));
          double vol = 0, area = 0;
          if (t == 0) vol = 1;
          else if (t > 0) {
            vol = t / 8.0;
            if (t == 2 || t == 4 || t == 6) area = 1;
            if (t == 1 || t == 7) area = 0.75;
            if (t == 3 || t == 5) area = 1.25;
          }
          H.node_vol[i] = vol * r3;
          H.surface_area[i] = area * r2;
        }
  }
  if (q.n_contact_angle > 0) {
    if (q.n_contact_angle != ng * nf)
      throw SetupError(MINIM_GPU_ERR_INVALID, "PhaseField: Invalid size of contactAngle array.");
    if (nf == 1 && !H.surface_area.empty()) {
      H.wet.assign(ng, 0.0);
      bool any = false;
      for (int i = 0; i < ng; i++) {
        const double ca = q.contact_angle[i];
        if (H.surface_area[i] == 0 || ca == 90) continue;
        H.wet[i] = 1 / std::sqrt(2.0) * std::cos(ca * 3.1415926536 / 180) * H.surface_area[i];
        any = true;
      }
      if (any) flags |= PF_CONTACT;
      else H.wet.clear();
    }
  }
  if (unstr) {
    // element form: the fixed volume is an energy penalty on the volumes
    // sum c * nodeVol (targets default to the initial ones), and
    // DENSITY_FIXED evaluates the last fluid as 1 minus the others
    flags |= PF_UNSTR;
    if (nf == 2 && q.density_constraint == MINIM_PF_DENSITY_SOFT)
      throw SetupError(MINIM_GPU_ERR_INVALID,
                       "PhaseFieldUnstructured: the soft density constraint needs at least three fluids");
    if (q.density_constraint == MINIM_PF_DENSITY_FIXED) flags |= PF_NALL;
    if (q.volume_fixed) {
      flags |= PF_UVOL;
      for (int f = 0; f < nf; f++) {
        double v = 0;
        if (q.volume) {
          v = q.volume[f];
        } else {
          for (int i = 0; i < ng; i++) v += x0[f + (size_t)nf * i] * node_vol(i);
        }
        P.vol_target[f] = v;
      }
      P.vol_coef = q.vol_const * st_mean / std::pow(q.resolution, 4);
    }
  } else if (q.volume_fixed) {
    flags |= PF_VOLUME;
    double tv = 0;
    for (int i = 0; i < ng; i++) tv += node_vol(i) * node_vol(i);
    P.total_volume2 = tv;
  }
  P.flags = flags;
  // PF_UNSTR alone changes nothing for one fluid without the optional terms
  const unsigned general = PF_SOLID | PF_CONTACT | PF_SOFT | PF_HARD | PF_VOLUME | PF_FORCE |
                           PF_CONFINE | PF_NODE_KAPPA | PF_FIXFLUID | PF_UVOL | PF_NALL;
  H.kernel_kind = (nf == 1 && !(flags & general)) ? K_PF1 : K_PF;
  (void)kPi;
  return H;
}

// ---------------------------------------------------------------------------
// BarAndHinge
// ---------------------------------------------------------------------------
namespace {
inline uint64_t key2(int a, int b) { return ((uint64_t)(uint32_t)a << 32) | (uint32_t)b; }
}  // namespace

BahTopology bah_topology(const minim_gpu_bah_params& q, int nvert) {
  BahTopology T;
  const int ntri = q.ntri;
  auto check_node = [&](int v) {
    if (v < 0 || v >= nvert)
      throw SetupError(MINIM_GPU_ERR_INVALID, "BarAndHinge: The triangulation expects more coordinates than are given.");
  };
  // bonds
  if (q.nbond > 0) {
    if (q.bond_stride < 2) throw SetupError(MINIM_GPU_ERR_INVALID, "BarAndHinge: bond stride must be >= 2");
    T.bonds.resize(q.nbond);
    for (int i = 0; i < q.nbond; i++) {
      T.bonds[i].assign(q.bonds + (size_t)i * q.bond_stride, q.bonds + (size_t)(i + 1) * q.bond_stride);
      check_node(T.bonds[i][0]);
      check_node(T.bonds[i][1]);
    }
  } else {
    if (ntri <= 0) throw SetupError(MINIM_GPU_ERR_INVALID, "BarAndHinge: The triangulation has not been set.");
    std::vector<std::pair<int, int>> pairs;
    pairs.reserve((size_t)ntri * 3);
    for (int t = 0; t < ntri; t++) {
      int s[3] = {q.tris[3 * t], q.tris[3 * t + 1], q.tris[3 * t + 2]};
      for (int k = 0; k < 3; k++) check_node(s[k]);
      std::sort(s, s + 3);
      pairs.push_back({s[0], s[1]});
      pairs.push_back({s[0], s[2]});
      pairs.push_back({s[1], s[2]});
    }
    std::sort(pairs.begin(), pairs.end());
    pairs.erase(std::unique(pairs.begin(), pairs.end()), pairs.end());
    std::unordered_map<uint64_t, int> bidx;
    bidx.reserve(pairs.size() * 2);
    T.bonds.resize(pairs.size());
    for (size_t i = 0; i < pairs.size(); i++) {
      T.bonds[i] = {pairs[i].first, pairs[i].second};
      bidx[key2(pairs[i].first, pairs[i].second)] = (int)i;
    }
    // third vertices of the triangles on each bond, in triangle order
    for (int t = 0; t < ntri; t++) {
      const int* tr = q.tris + 3 * t;
      for (int k = 0; k < 3; k++) {
        int a = tr[k], b = tr[(k + 1) % 3], c = tr[(k + 2) % 3];
        if (a > b) std::swap(a, b);
        auto it = bidx.find(key2(a, b));
        if (it == bidx.end()) continue;
        auto& bond = T.bonds[it->second];
        if (std::find(bond.begin(), bond.end(), c) == bond.end()) bond.push_back(c);
      }
    }
  }
  // hinges
  if (q.nhinge > 0) {
    if (q.hinge_stride < 4) throw SetupError(MINIM_GPU_ERR_INVALID, "BarAndHinge: hinge stride must be >= 4");
    T.hinges.resize(q.nhinge);
    for (int i = 0; i < q.nhinge; i++) {
      T.hinges[i].assign(q.hinges + (size_t)i * q.hinge_stride, q.hinges + (size_t)(i + 1) * q.hinge_stride);
      for (int k = 0; k < 4; k++) check_node(T.hinges[i][k]);
    }
  } else {
    if (ntri <= 0) throw SetupError(MINIM_GPU_ERR_INVALID, "BarAndHinge: The triangulation has not been set.");
    // triangles on each edge; every pair of triangles sharing exactly two
    // vertices shares an edge, so candidates come from the edge lists
    std::unordered_map<uint64_t, std::vector<int>> on_edge;
    on_edge.reserve((size_t)ntri * 3);
    for (int t = 0; t < ntri; t++) {
      const int* tr = q.tris + 3 * t;
      for (int k = 0; k < 3; k++) {
        int a = tr[k], b = tr[(k + 1) % 3];
        if (a > b) std::swap(a, b);
        if (a == b) continue;
        auto& v = on_edge[key2(a, b)];
        if (v.empty() || v.back() != t) v.push_back(t);
      }
    }
    std::vector<std::pair<int, int>> cand;
    for (auto& kv : on_edge) {
      auto& v = kv.second;
      for (size_t i = 0; i < v.size(); i++)
        for (size_t j = i + 1; j < v.size(); j++) cand.push_back({v[i], v[j]});
    }
    std::sort(cand.begin(), cand.end());
    cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
    for (auto& pr : cand) {
      const int* A = q.tris + 3 * pr.first;
      const int* B = q.tris + 3 * pr.second;
      bool sh[6] = {false, false, false, false, false, false};
      int ns = 0;
      for (int i1 = 0; i1 < 3; i1++)
        for (int i2 = 0; i2 < 3; i2++) {
          if (A[i1] != B[i2]) continue;
          ns++;
          sh[i1] = true;
          sh[3 + i2] = true;
        }
      if (ns != 2) continue;
      std::vector<int> nodes(4);
      for (int i1 = 0; i1 < 3; i1++)
        if (!sh[i1]) {
          nodes[0] = A[i1];
          nodes[1] = A[(i1 + 1) % 3];
          nodes[2] = A[(i1 + 2) % 3];
        }
      for (int i2 = 0; i2 < 3; i2++)
        if (!sh[3 + i2]) nodes[3] = B[i2];
      T.hinges.push_back(nodes);
    }
    // bond index of each hinge (first bond containing nodes 1 and 2)
    std::unordered_map<uint64_t, int> first;
    first.reserve(T.bonds.size() * 2);
    for (size_t i = 0; i < T.bonds.size(); i++) {
      const int a = T.bonds[i][0], b = T.bonds[i][1];
      first.emplace(key2(a, b), (int)i);
      first.emplace(key2(b, a), (int)i);
    }
    for (auto& h : T.hinges) {
      auto it = first.find(key2(h[1], h[2]));
      if (it != first.end()) h.push_back(it->second);
    }
  }
  return T;
}

BahHost setup_bah(const minim_gpu_bah_params& q, const double* x, size_t ndof) {
  if (ndof % 3) throw SetupError(MINIM_GPU_ERR_INVALID, "BarAndHinge: coordinates must be 3 per vertex");
  BahHost B;
  B.nvert = (int)(ndof / 3);
  BahTopology T = bah_topology(q, B.nvert);
  const int nb = (int)T.bonds.size(), nh = (int)T.hinges.size();
  std::vector<double> kb(nb), kh(nh);
  const bool have_kb = q.n_kbond > 0, have_kh = q.n_khinge > 0;
  if (q.n_kbond == 1) std::fill(kb.begin(), kb.end(), q.kbond[0]);
  else if (q.n_kbond > 1) {
    if (q.n_kbond != nb) throw SetupError(MINIM_GPU_ERR_INVALID, "BarAndHinge: kBond has the wrong size");
    kb.assign(q.kbond, q.kbond + nb);
  }
  if (q.n_khinge == 1) std::fill(kh.begin(), kh.end(), q.khinge[0]);
  else if (q.n_khinge > 1) {
    if (q.n_khinge != nh) throw SetupError(MINIM_GPU_ERR_INVALID, "BarAndHinge: kHinge has the wrong size");
    kh.assign(q.khinge, q.khinge + nh);
  }
  if (!have_kb || !have_kh) {
    if (q.n_thickness <= 0)
      throw SetupError(MINIM_GPU_ERR_INVALID, "BarAndHinge requires either the rigidities or the thickness to be set");
    std::vector<double> th(B.nvert);
    for (int i = 0; i < B.nvert; i++) th[i] = q.n_thickness == 1 ? q.thickness[0] : q.thickness[i];
    std::vector<double> lsq(nb), asum(nb);
    for (int i = 0; i < nb; i++) {
      const auto& bd = T.bonds[i];
      if (bd.size() == 2)
        throw SetupError(MINIM_GPU_ERR_INVALID, "The bondList should contain the indicies of the adjacent triangles.");
      const double* x1 = x + 3 * bd[0];
      const double* x2 = x + 3 * bd[1];
      const double d21[3] = {x2[0] - x1[0], x2[1] - x1[1], x2[2] - x1[2]};
      lsq[i] = std::pow(d21[0], 2) + std::pow(d21[1], 2) + std::pow(d21[2], 2);
      for (size_t j = 2; j < bd.size(); j++) {
        const double* x3 = x + 3 * bd[j];
        const double d31[3] = {x3[0] - x1[0], x3[1] - x1[1], x3[2] - x1[2]};
        const double c[3] = {d21[1] * d31[2] - d21[2] * d31[1], d21[2] * d31[0] - d21[0] * d31[2],
                             d21[0] * d31[1] - d21[1] * d31[0]};
        asum[i] += std::fabs(std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2])) / 2;
      }
    }
    if (!have_kb)
      for (int i = 0; i < nb; i++) {
        const double t = (th[T.bonds[i][0]] + th[T.bonds[i][1]]) / 2;
        kb[i] = q.modulus * t * (asum[i] / lsq[i]);
      }
    if (!have_kh)
      for (int h = 0; h < nh; h++) {
        const auto& hg = T.hinges[h];
        if (hg.size() == 4)
          throw SetupError(MINIM_GPU_ERR_INVALID, "The hingeList should contain the index of the bond.");
        const double t = (th[hg[0]] + th[hg[1]] + th[hg[2]] + th[hg[3]]) / 4;
        const double rig = q.modulus * std::pow(t, 3) / (12 * (1 - std::pow(q.poisson_ratio, 2)));
        kh[h] = rig * (lsq[hg[4]] / asum[hg[4]]);
      }
  }
  B.bars.resize(2 * nb);
  B.bpar.resize(2 * nb);
  for (int i = 0; i < nb; i++) {
    const int a = T.bonds[i][0], b = T.bonds[i][1];
    B.bars[2 * i] = a;
    B.bars[2 * i + 1] = b;
    B.bpar[2 * i] = kb[i];
    double l0;
    if (q.n_length0 == 1) l0 = q.length0[0];
    else if (q.n_length0 > 1) {
      if (q.n_length0 != nb) throw SetupError(MINIM_GPU_ERR_INVALID, "BarAndHinge: length0 has the wrong size");
      l0 = q.length0[i];
    } else {
      const double d[3] = {x[3 * a] - x[3 * b], x[3 * a + 1] - x[3 * b + 1], x[3 * a + 2] - x[3 * b + 2]};
      l0 = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    }
    B.bpar[2 * i + 1] = l0;
  }
  B.hinges.resize(4 * nh);
  B.hpar.resize(2 * nh);
  for (int h = 0; h < nh; h++) {
    const auto& hg = T.hinges[h];
    for (int k = 0; k < 4; k++) B.hinges[4 * h + k] = hg[k];
    B.hpar[2 * h] = kh[h];
    double t0;
    if (q.n_theta0 == 1) t0 = q.theta0[0];
    else if (q.n_theta0 > 1) {
      if (q.n_theta0 != nh) throw SetupError(MINIM_GPU_ERR_INVALID, "BarAndHinge: theta0 has the wrong size");
      t0 = q.theta0[h];
    } else {
      const double *x1 = x + 3 * hg[0], *x2 = x + 3 * hg[1], *x3 = x + 3 * hg[2], *x4 = x + 3 * hg[3];
      double a[3], b[3], c[3];
      for (int d = 0; d < 3; d++) { a[d] = x2[d] - x1[d]; b[d] = x3[d] - x2[d]; c[d] = x4[d] - x3[d]; }
      const double n1[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
      const double n2[3] = {b[1] * c[2] - b[2] * c[1], b[2] * c[0] - b[0] * c[2], b[0] * c[1] - b[1] * c[0]};
      const double cs = (n1[0] * n2[0] + n1[1] * n2[1] + n1[2] * n2[2]) /
                        (std::sqrt(n1[0] * n1[0] + n1[1] * n1[1] + n1[2] * n1[2]) *
                         std::sqrt(n2[0] * n2[0] + n2[1] * n2[1] + n2[2] * n2[2]));
      const double n1b3 = n1[0] * c[0] + n1[1] * c[1] + n1[2] * c[2];
      t0 = (n1b3 >= 0) ? std::acos(cs) : 2 * kPi - std::acos(cs);
    }
    B.hpar[2 * h + 1] = t0;
  }
  bah_scalars(q, B);
  return B;
}

void bah_scalars(const minim_gpu_bah_params& q, BahHost& B) {
  if (q.n_force > 0) {
    if (q.n_force != 3 && q.n_force != 3 * B.nvert)
      throw SetupError(MINIM_GPU_ERR_INVALID, "BarAndHinge: force must have 3 or 3*nvert entries");
    B.force.assign(q.force, q.force + q.n_force);
  }
  B.wall_on = q.wall_on;
  B.wall_adh = q.wall_adhesion;
  B.wall_eps = q.wall_epsilon;
  B.wall_sig = q.wall_sigma;
}

namespace {
// Greedy colouring: each element takes the smallest colour not yet used by
// an element sharing one of its vertices.  Returns the colour per element.
std::vector<int> greedy_colour(const std::vector<int>& elem_nodes, int per, int nvert, int& ncol) {
  const int ne = (int)(elem_nodes.size() / per);
  std::vector<std::vector<uint64_t>> used(nvert);
  std::vector<int> col(ne);
  ncol = 0;
  for (int e = 0; e < ne; e++) {
    int c = 0;
    for (;; c++) {
      const int w = c >> 6;
      const uint64_t bit = 1ull << (c & 63);
      bool free = true;
      for (int k = 0; k < per && free; k++) {
        const auto& u = used[elem_nodes[per * e + k]];
        if (w < (int)u.size() && (u[w] & bit)) free = false;
      }
      if (free) break;
    }
    col[e] = c;
    ncol = std::max(ncol, c + 1);
    const int w = c >> 6;
    for (int k = 0; k < per; k++) {
      auto& u = used[elem_nodes[per * e + k]];
      if ((int)u.size() <= w) u.resize(w + 1, 0);
      u[w] |= 1ull << (c & 63);
    }
  }
  return col;
}
}  // namespace

BahDevArrays bah_arrays(const BahHost& b, const std::vector<unsigned char>& fixed) {
  BahDevArrays D;
  auto all_fixed = [&](const int* nodes, int k) {
    if (fixed.empty()) return false;
    for (int i = 0; i < k; i++)
      for (int d = 0; d < 3; d++)
        if (!fixed[3 * nodes[i] + d]) return false;
    return true;
  };
  std::vector<int> bn, hn;
  std::vector<double> bp, hp;
  const int nb = (int)(b.bars.size() / 2), nh = (int)(b.hinges.size() / 4);
  for (int i = 0; i < nb; i++) {
    if (all_fixed(&b.bars[2 * i], 2)) continue;
    bn.insert(bn.end(), {b.bars[2 * i], b.bars[2 * i + 1]});
    bp.insert(bp.end(), {b.bpar[2 * i], b.bpar[2 * i + 1]});
  }
  for (int h = 0; h < nh; h++) {
    if (all_fixed(&b.hinges[4 * h], 4)) continue;
    hn.insert(hn.end(), &b.hinges[4 * h], &b.hinges[4 * h + 4]);
    hp.insert(hp.end(), {b.hpar[2 * h], b.hpar[2 * h + 1]});
  }
  int nbc = 0, nhc = 0;
  auto bc = greedy_colour(bn, 2, b.nvert, nbc);
  auto hc = greedy_colour(hn, 4, b.nvert, nhc);
  // stable counting sort by colour
  D.bar_off.assign(nbc + 1, 0);
  for (int c : bc) D.bar_off[c + 1]++;
  for (int c = 0; c < nbc; c++) D.bar_off[c + 1] += D.bar_off[c];
  D.bars.resize(bc.size());
  D.bpar.resize(bc.size());
  {
    std::vector<int> pos(D.bar_off.begin(), D.bar_off.end() - 1);
    for (size_t e = 0; e < bc.size(); e++) {
      const int p = pos[bc[e]]++;
      D.bars[p] = make_int2(bn[2 * e], bn[2 * e + 1]);
      D.bpar[p] = make_double2(bp[2 * e], bp[2 * e + 1]);
    }
  }
  D.hinge_off.assign(nhc + 1, 0);
  for (int c : hc) D.hinge_off[c + 1]++;
  for (int c = 0; c < nhc; c++) D.hinge_off[c + 1] += D.hinge_off[c];
  D.hinges.resize(hc.size());
  D.hpar.resize(hc.size());
  {
    std::vector<int> pos(D.hinge_off.begin(), D.hinge_off.end() - 1);
    for (size_t e = 0; e < hc.size(); e++) {
      const int p = pos[hc[e]]++;
      D.hinges[p] = make_int4(hn[4 * e], hn[4 * e + 1], hn[4 * e + 2], hn[4 * e + 3]);
      D.hpar[p] = make_double2(hp[2 * e], hp[2 * e + 1]);
    }
  }
  D.node_el.assign(b.nvert, 1);
  if (!fixed.empty())
    for (int v = 0; v < b.nvert; v++)
      D.node_el[v] = !(fixed[3 * v] && fixed[3 * v + 1] && fixed[3 * v + 2]);
  return D;
}

}  // namespace mg
