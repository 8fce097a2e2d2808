/*
 * minim_oracle.c -- FP64 CPU restatement of the reference minim hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Tests, the smoke check and bench.py's CPU
 * baseline leg use this file as the checker; the GPU engine never calls it.
 * Every function names the reference source lines (paths relative to the
 * minim source tree) whose behaviour it restates, quirks included.
 * Arithmetic follows the reference's expressions and summation order so that
 * results agree with the reference library to rounding (the tests pin this).
 */
#define _POSIX_C_SOURCE 200809L
#include "minim_oracle.h"

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static char g_err[512];
/* Threaded loops for the all-core CPU timing; with one thread every loop
 * runs serially in the reference's order (the parity tests use that). */
#define OMP_FOR _Pragma("omp parallel for if(o->nthreads > 1) num_threads(o->nthreads) schedule(static)")

static int set_err(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
  return code;
}
const char* oracle_last_error(void) { return g_err; }

static const double PI_REF = 3.14159265358979323846; /* 4*atan(1), src/potentials/BarAndHinge.cpp:13 */

/* ------------------------------------------------------------------------ */
/* Instance                                                                  */
/* ------------------------------------------------------------------------ */
typedef struct {
  /* PhaseField state after init/initLocal (src/potentials/PhaseField.cpp:137-235) */
  int n[3], nfluid, ngrid;
  double res;
  int density;       /* DENSITY_* */
  double density_const;
  int volume_fixed;
  double total_volume2;
  double* kappa;     /* nk */
  double* kappaP;
  int nk;
  double st_mean;    /* surfaceTensionMean */
  double* node_vol;  /* ngrid */
  double* surf_area; /* ngrid */
  char* solid;       /* ngrid */
  double* contact;   /* ngrid*? or NULL */
  int ncontact;
  double* pressure;  /* nfluid */
  char* fix_fluid;   /* nfluid */
  double* confine;   /* nfluid */
  double* ff_init;   /* ndof or NULL */
  double* fmag;      /* nfluid */
  double* fnorm;     /* nfluid*3 */
  int any_force;
  /* PhaseFieldUnstructured (element form, src/potentials/PhaseFieldUnstructured.cpp) */
  int unstr;
  double vol_const;
  double* volume;    /* nfluid target volumes (PFU with a fixed volume) */
} pf_t;

typedef struct {
  int nbar, nhinge, nvert;
  int* bars;      /* 2 per bar */
  double* bpar;   /* {k, l0} */
  int* hinges;    /* 4 per hinge */
  double* hpar;   /* {k, theta0} */
  char* node_el;  /* per vertex: force element present (not all dofs fixed) */
  double* force;  /* 0, 3 or 3*nvert entries */
  int nforce;
  int wall_on, wall_adh;
  double wall_eps, wall_sig;
} bah_t;

struct oracle_inst {
  int kind;
  size_t ndof;
  double* x;
  char* fixed;  /* ndof flags (generic fixed-dof constraints) or NULL */
  double tol_default;
  /* LJ */
  int ndim;
  double sigma, eps;
  double rc2;  /* cutoff squared (0: every pair) */
  pf_t pf;
  bah_t bah;
  long evals;
  int nthreads;  /* > 1: parallel loops (timing runs only); 1: serial reference order */
};

size_t oracle_ndof(const oracle_inst* o) { return o->ndof; }
void oracle_set_threads(oracle_inst* o, int nthreads) { o->nthreads = nthreads > 1 ? nthreads : 1; }
double oracle_default_tol(const oracle_inst* o) { return o->tol_default; }

/* ------------------------------------------------------------------------ */
/* LjNd: src/potentials/LjNd.cpp:12-53                                       */
/* ------------------------------------------------------------------------ */
/* One element per pair i<j in (i, j) order (LjNd::init, lines 17-25).  With
   a cutoff (an extension: the reference has none) a pair with r2 >= rc2 is
   left out, r2 summed over the dimensions in order, one rounding each. */
static void lj_eg(const oracle_inst* o, const double* x, double* e, double* g) {
  int nd = o->ndim;
  int np = (int)(o->ndof / nd);
  double s6 = pow(o->sigma, 6);
  for (int i = 0; i < np; i++) {
    for (int j = i + 1; j < np; j++) {
      double dx[3] = {0, 0, 0};
      double r2 = 0;
      for (int d = 0; d < nd; d++) dx[d] = x[nd * i + d] - x[nd * j + d];
      for (int d = 0; d < nd; d++) r2 += dx[d] * dx[d];
      if (o->rc2 > 0 && r2 >= o->rc2) continue;
      double lj6 = s6 / pow(r2, 3);
      double lj12 = lj6 * lj6;
      if (e) *e += 4 * o->eps * (lj12 - lj6);
      if (g) {
        double factor = -24 * o->eps * (2 * lj12 - lj6) / r2;
        for (int d = 0; d < nd; d++) {
          g[nd * i + d] += dx[d] * factor;
          g[nd * j + d] -= dx[d] * factor;
        }
      }
    }
  }
}

/* ------------------------------------------------------------------------ */
/* PhaseField (MODEL_BASIC)                                                  */
/* ------------------------------------------------------------------------ */
enum { D_HARD = 0, D_SOFT = 1, D_NONE = 2, D_FIXED = 3 };

static int pf_idx(const pf_t* p, int x, int y, int z) {
  /* getIdx with periodic wrap, src/potentials/PhaseField.cpp:44-49 */
  x = (x + p->n[0]) % p->n[0];
  y = (y + p->n[1]) % p->n[1];
  z = (z + p->n[2]) % p->n[2];
  return (x * p->n[1] + y) * p->n[2] + z;
}

/* 26-neighbour offsets in the reference's order (PhaseField.cpp:65-75). */
static const int NEI26[26][3] = {
    {-1, 0, 0}, {0, -1, 0}, {0, 0, -1}, {0, 0, 1}, {0, 1, 0}, {1, 0, 0},
    {-1, -1, 0}, {-1, 0, -1}, {-1, 0, 1}, {-1, 1, 0}, {0, -1, -1}, {0, -1, 1},
    {0, 1, -1}, {0, 1, 1}, {1, -1, 0}, {1, 0, -1}, {1, 0, 1}, {1, 1, 0},
    {-1, -1, -1}, {-1, -1, 1}, {-1, 1, -1}, {-1, 1, 1}, {1, -1, -1}, {1, -1, 1},
    {1, 1, -1}, {1, 1, 1}};

/* PhaseField::getType, src/potentials/PhaseField.cpp:903-958.
 * Returns -2 for the reference's "Undefined surface type" exception. */
static int pf_type(const pf_t* p, int i) {
  if (p->solid[i]) return -1;
  int z = i % p->n[2], y = (i / p->n[2]) % p->n[1], x = i / (p->n[1] * p->n[2]);
  int s[26];
  for (int d = 0; d < 26; d++) s[d] = p->solid[pf_idx(p, x + NEI26[d][0], y + NEI26[d][1], z + NEI26[d][2])] != 0;
  int nF = s[0] + s[1] + s[2] + s[3] + s[4] + s[5];
  int nE = 0, nC = 0;
  for (int d = 6; d < 18; d++) nE += s[d];
  for (int d = 18; d < 26; d++) nC += s[d];
  if (nF + nE + nC == 0) return 0;
  if (nF == 0) {
    if (nE == 0 && nC == 1) return 1;
    if (nE == 1 && nC <= 2) return 2;
    if (nE == 2 && nC <= 3) return 3;
  } else if (nF == 1) {
    int one = ((s[0] || s[5]) && !(s[10] || s[11] || s[12] || s[13])) ||
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

static void* xcalloc(size_t n, size_t sz) {
  void* p = calloc(n ? n : 1, sz);
  return p;
}

/* PhaseField::init + assignFluidCoefficients + initLocal
 * (src/potentials/PhaseField.cpp:78-235; 1 rank so procSizes == gridSize and
 * no halo). */
static int pf_setup(oracle_inst* o, const minim_gpu_pf_params* q, const double* x0, int unstr) {
  pf_t* p = &o->pf;
  memset(p, 0, sizeof *p);
  p->unstr = unstr;
  for (int d = 0; d < 3; d++) p->n[d] = q->grid[d];
  p->nfluid = q->nfluid;
  p->ngrid = q->grid[0] * q->grid[1] * q->grid[2];
  p->res = q->resolution;
  if (p->nfluid < 1 || p->ngrid < 1) return set_err(MINIM_GPU_ERR_INVALID, "PhaseField: invalid grid or nFluid");
  if ((size_t)p->ngrid * p->nfluid != o->ndof)
    return set_err(MINIM_GPU_ERR_INVALID, "PhaseField: Size of coordinates array does not match the grid size.");
  int nf = p->nfluid, ng = p->ngrid;
  int nparams = nf;
  /* surface tensions: assignFluidCoefficients lines 78-88 */
  int nst = q->n_surface_tension > 0 ? q->n_surface_tension : 1;
  const double one = 1.0;
  const double* st_in = q->n_surface_tension > 0 ? q->surface_tension : &one;
  /* PhaseFieldUnstructured has no per-node surface tensions
   * (PhaseFieldUnstructured.cpp:71-86), and checkArraySizes (lines 929-933) wants
   * one interface width per fluid */
  int nkgrid = (!unstr && nst == ng * nparams) ? ng : 1;
  int nstt = nkgrid * nparams;
  if (unstr && q->n_interface_size != 0 && q->n_interface_size != nf)
    return set_err(MINIM_GPU_ERR_INVALID, "PhaseFieldUnstructured: Invalid size interfaceSize array.");
  double* st = xcalloc(nstt, sizeof(double));
  if (nst == 1) {
    for (int i = 0; i < nstt; i++) st[i] = st_in[0];
  } else if (nst != nstt) {
    free(st);
    return set_err(MINIM_GPU_ERR_INVALID, "PhaseField: Invalid size of surfaceTension array.");
  } else {
    memcpy(st, st_in, nstt * sizeof(double));
  }
  double sum = 0;
  for (int i = 0; i < nstt; i++) sum += st[i];
  p->st_mean = sum / nstt;
  /* interface widths (setDefaults line 962: default = resolution) */
  double* iw = xcalloc(nstt, sizeof(double));
  if (q->n_interface_size == 0) {
    for (int i = 0; i < nparams; i++) iw[i] = p->res;
  } else if (q->n_interface_size == 1) {
    for (int i = 0; i < nparams; i++) iw[i] = q->interface_size[0];
  } else if (q->n_interface_size == nparams) {
    for (int i = 0; i < nparams; i++) iw[i] = q->interface_size[i];
  } else {
    free(st); free(iw);
    return set_err(MINIM_GPU_ERR_INVALID, "PhaseField: Invalid size interfaceSize array.");
  }
  for (int k = 1; k < nkgrid; k++)
    for (int j = 0; j < nparams; j++) iw[k * nparams + j] = iw[j];
  p->nk = nstt;
  p->kappa = xcalloc(nstt, sizeof(double));
  p->kappaP = xcalloc(nstt, sizeof(double));
  if (nf <= 2) {
    for (int i = 0; i < nstt; i++) {
      p->kappa[i] = 3 * st[i] / iw[i];
      p->kappaP[i] = 3 * st[i] * iw[i];
    }
  } else {
    /* ternary combination, lines 113-133 */
    for (int kg = 0; kg < nkgrid; kg++) {
      int i0 = kg * nparams;
      double ks[64], kps[64];
      for (int j = 0; j < nparams && j < 64; j++) {
        ks[j] = 6 * st[i0 + j] / iw[i0 + j];
        kps[j] = 6 * st[i0 + j] * iw[i0 + j];
      }
      p->kappa[i0 + 0] = 0.5 * (ks[0] + ks[1] - ks[nf - 1]);
      p->kappa[i0 + 1] = 0.5 * (ks[0] - ks[1] + ks[nf - 1]);
      p->kappa[i0 + 2] = 0.5 * (-ks[0] + ks[1] + ks[nf - 1]);
      p->kappaP[i0 + 0] = 0.5 * (kps[0] + kps[1] - kps[nf - 1]);
      p->kappaP[i0 + 1] = 0.5 * (kps[0] - kps[1] + kps[nf - 1]);
      p->kappaP[i0 + 2] = 0.5 * (-kps[0] + kps[1] + kps[nf - 1]);
      for (int f = 3; f < nf; f++) {
        p->kappa[i0 + f] = ks[f - 1] - p->kappa[i0 + 0];
        p->kappaP[i0 + f] = kps[f - 1] - p->kappaP[i0 + 0];
      }
    }
  }
  free(st);
  free(iw);
  o->tol_default = 1e-8 * p->st_mean * pow(p->res, 2); /* line 146 */
  p->density = q->density_constraint;
  p->density_const = q->density_const;
  p->volume_fixed = q->volume_fixed;
  p->pressure = xcalloc(nf, sizeof(double));
  if (q->pressure) memcpy(p->pressure, q->pressure, nf * sizeof(double));
  p->fix_fluid = xcalloc(nf, 1);
  if (q->fix_fluid) memcpy(p->fix_fluid, q->fix_fluid, nf);
  if (p->density == D_FIXED) p->fix_fluid[nf - 1] = 1; /* line 147 */
  p->confine = xcalloc(nf, sizeof(double));
  if (q->confinement) memcpy(p->confine, q->confinement, nf * sizeof(double));
  p->solid = xcalloc(ng, 1);
  if (q->solid) memcpy(p->solid, q->solid, ng);
  if (q->n_contact_angle > 0) {
    if (q->n_contact_angle != ng * nf) {
      /* checkArraySizes (line 977) only accepts ngrid*nfluid entries */
      return set_err(MINIM_GPU_ERR_INVALID, "PhaseField: Invalid size of contactAngle array.");
    }
    p->ncontact = q->n_contact_angle;
    p->contact = xcalloc(p->ncontact, sizeof(double));
    memcpy(p->contact, q->contact_angle, p->ncontact * sizeof(double));
  }
  /* forces: lines 150-157 */
  p->fmag = xcalloc(nf, sizeof(double));
  p->fnorm = xcalloc(3 * nf, sizeof(double));
  if (q->force) {
    for (int f = 0; f < nf; f++) {
      const double* F = q->force + 3 * f;
      p->fmag[f] = sqrt(F[0] * F[0] + F[1] * F[1] + F[2] * F[2]);
      for (int d = 0; d < 3; d++) p->fnorm[3 * f + d] = F[d] / p->fmag[f];
      if (p->fmag[f] != 0) p->any_force = 1;
    }
  }
  /* nodeVol / surfaceArea: lines 194-208 */
  p->node_vol = xcalloc(ng, sizeof(double));
  p->surf_area = xcalloc(ng, sizeof(double));
  for (int i = 0; i < ng; i++) {
    int t = pf_type(p, i);
    if (t == -2) return set_err(MINIM_GPU_ERR_RUNTIME, "PhaseField: Undefined surface type");
    if (t == 0) {
      p->node_vol[i] = 1;
    } else if (t > 0) {
      p->node_vol[i] = t / 8.0;
      if (t == 2 || t == 4 || t == 6) p->surf_area[i] = 1;
      if (t == 1 || t == 7) p->surf_area[i] = 0.75;
      if (t == 3 || t == 5) p->surf_area[i] = 1.25;
    }
    p->node_vol[i] = p->node_vol[i] * pow(p->res, 3);
    p->surf_area[i] = p->surf_area[i] * pow(p->res, 2);
  }
  /* totalVolume2 (lines 226-230).  The reference computes it only when no
   * target volume is given; it is always computed here. */
  if (p->volume_fixed) {
    double tv = 0;
    for (int i = 0; i < ng; i++) tv += p->node_vol[i] * p->node_vol[i];
    p->total_volume2 = tv;
  }
  int anyc = 0;
  for (int f = 0; f < nf; f++) anyc |= (p->confine[f] != 0);
  if (anyc) {
    p->ff_init = xcalloc(o->ndof, sizeof(double));
    memcpy(p->ff_init, x0, o->ndof * sizeof(double));
  }
  if (unstr) {
    /* the soft density element reads the node's first three fluids
     * (PhaseFieldUnstructured.cpp:631-642); with two it would read past them */
    if (nf == 2 && p->density == D_SOFT)
      return set_err(MINIM_GPU_ERR_INVALID,
                     "PhaseFieldUnstructured: the soft density constraint needs at least three fluids");
    p->vol_const = q->vol_const;
    if (p->volume_fixed) {
      p->volume = xcalloc(nf, sizeof(double));
      if (q->volume) {
        memcpy(p->volume, q->volume, nf * sizeof(double));
      } else {
        /* initial volumes, lines 148-156: sum of c * nodeVol (also for one
         * fluid, whose penalty then measures 0.5 (c + 1) * nodeVol) */
        for (int i = 0; i < ng; i++)
          for (int f = 0; f < nf; f++) p->volume[f] += x0[f + nf * i] * p->node_vol[i];
      }
    }
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* PhaseFieldUnstructured: src/potentials/PhaseFieldUnstructured.cpp         */
/* ------------------------------------------------------------------------ */
/* phaseGradient for one fluid, lines 311-396: idof[0] is the node, idof[1..6]
 * its x-, y-, z-, z+, y+, x+ neighbours; a neighbour whose index equals the
 * node's (a solid neighbour, or a dimension of size 1) drops that side. */
static void pfu_phase_gradient(const double* c, const int* idof, double factor, double* e, double* g) {
  static const int side[3][2] = {{1, 6}, {2, 5}, {3, 4}};
  double c1 = c[idof[0]];
  double grad2 = 0;
  for (int d = 0; d < 3; d++) {
    int im = idof[side[d][0]], ip = idof[side[d][1]];
    if (im != idof[0] && ip != idof[0]) {
      double gm = c1 - c[im], gp = c1 - c[ip];
      if (e) grad2 += 0.5 * (pow(gm, 2) + pow(gp, 2));
      if (g) {
        g[idof[0]] += factor * (gm + gp);
        g[im] -= factor * gm;
        g[ip] -= factor * gp;
      }
    } else if (ip != idof[0]) {
      double gp = c1 - c[ip];
      if (e) grad2 += pow(gp, 2);
      if (g) {
        g[idof[0]] += factor * 2 * gp;
        g[ip] -= factor * 2 * gp;
      }
    } else if (im != idof[0]) {
      double gm = c1 - c[im];
      if (e) grad2 += pow(gm, 2);
      if (g) {
        g[idof[0]] += factor * 2 * gm;
        g[im] -= factor * 2 * gm;
      }
    }
  }
  if (e) *e += factor * grad2;
}

/* fluidEnergy, lines 518-538 */
static void pfu_fluid(const pf_t* p, const double* c, const int* idof, double V, int f, double* e, double* g) {
  int nf = p->nfluid;
  double cc = c[idof[0]];
  if (nf == 1) {
    double fac = p->kappa[0] / 16 * V;
    if (e) *e += fac * pow(cc + 1, 2) * pow(cc - 1, 2);
    if (g) g[idof[0]] += fac * 4 * cc * (cc * cc - 1);
  } else {
    double fac = 0.5 * p->kappa[f] * V;
    if (e) *e += fac * pow(cc, 2) * pow(cc - 1, 2);
    if (g) g[idof[0]] += fac * 2 * cc * (cc - 1) * (2 * cc - 1);
  }
  double fac = (nf == 1) ? 0.25 * p->kappaP[0] * V : 0.5 * p->kappaP[f] * V;
  fac = fac / pow(p->res, 2);
  pfu_phase_gradient(c, idof, fac, e, g);
}

/* fluidEnergyAll (DENSITY_FIXED), lines 541-586: the last fluid's
 * concentration is 1 minus the others'.  Its gradient term runs over the
 * local indices 0..6, which are all distinct, so a solid neighbour (whose
 * index is the node's own) enters as a zero difference on the two-sided
 * form, and its factor is not divided by res^2 -- both as in the reference. */
static void pfu_fluid_all(const pf_t* p, const double* c, const int* idof, double V, double* e, double* g) {
  static const int iota7[7] = {0, 1, 2, 3, 4, 5, 6};
  int nf = p->nfluid;
  double cN[7], gN[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int i = 0; i < 7; i++) cN[i] = 1;
  for (int f = 0; f < nf - 1; f++)
    for (int i = 0; i < 7; i++) cN[i] -= c[idof[i] + f];
  double bN = 0.5 * p->kappa[nf - 1] * V;
  double gfN = 0.5 * p->kappaP[nf - 1] * V;
  if (e) *e += bN * pow(cN[0], 2) * pow(cN[0] - 1, 2);
  if (g) {
    gN[0] += bN * 2 * cN[0] * (cN[0] - 1) * (2 * cN[0] - 1);
    pfu_phase_gradient(cN, iota7, gfN, e, gN);
  } else {
    pfu_phase_gradient(cN, iota7, gfN, e, NULL);
  }
  for (int f = 0; f < nf - 1; f++) {
    int id[7];
    for (int i = 0; i < 7; i++) id[i] = idof[i] + f;
    double cc = c[id[0]];
    double bf = 0.5 * p->kappa[f] * V;
    if (e) *e += bf * pow(cc, 2) * pow(cc - 1, 2);
    if (g) g[id[0]] += bf * 2 * cc * (cc - 1) * (2 * cc - 1);
    double gf = 0.5 * p->kappaP[f] * V;
    gf = gf / pow(p->res, 2);
    pfu_phase_gradient(c, id, gf, e, g);
    if (g)
      for (int i = 0; i < 7; i++) g[id[i]] -= gN[i];
  }
}

/* The energy elements of PhaseFieldUnstructured::init (lines 158-236) in
 * their order, evaluated as State's elementEG does (src/State.cpp:58-79),
 * then blockEnergyGradient (lines 280-308). */
static void pfu_eg(const oracle_inst* o, const double* c, double* e, double* g) {
  const pf_t* p = &o->pf;
  int nf = p->nfluid, ng = p->ngrid;
  double res2 = pow(p->res, 2);
  for (int iG = 0; iG < ng; iG++) {
    if (p->solid[iG]) continue;
    int z = iG % p->n[2], y = (iG / p->n[2]) % p->n[1], x = iG / (p->n[1] * p->n[2]);
    int nodes[7] = {iG, pf_idx(p, x - 1, y, z), pf_idx(p, x, y - 1, z), pf_idx(p, x, y, z - 1),
                    pf_idx(p, x, y, z + 1), pf_idx(p, x, y + 1, z), pf_idx(p, x + 1, y, z)};
    for (int k = 1; k < 7; k++)
      if (p->solid[nodes[k]]) nodes[k] = iG;
    double V = p->node_vol[iG];
    if (p->density == D_FIXED) {
      int idof[7];
      for (int k = 0; k < 7; k++) idof[k] = nodes[k] * nf;
      pfu_fluid_all(p, c, idof, V, e, g);
    } else {
      for (int f = 0; f < nf; f++) {
        int idof[7];
        for (int k = 0; k < 7; k++) idof[k] = nodes[k] * nf + f;
        pfu_fluid(p, c, idof, V, f, e, g);
      }
    }
    /* pressureEnergy, lines 613-628 (every fluid with a pressure) */
    for (int f = 0; f < nf; f++) {
      if (p->pressure[f] == 0) continue;
      int iD = iG * nf + f;
      if (nf == 1) {
        double vol = 0.5 * (c[iD] + 1) * V;
        if (e) *e -= p->pressure[f] * vol;
        if (g) g[iD] -= 0.5 * p->pressure[f] * V;
      } else {
        double vol = c[iD] * V;
        if (e) *e -= p->pressure[f] * vol;
        if (g) g[iD] -= p->pressure[f] * V;
      }
    }
    /* densityConstraintEnergy, lines 631-642: the first three fluids */
    if (nf > 1 && p->density == D_SOFT) {
      double coef = p->density_const * p->st_mean * res2;
      int i0 = iG * nf;
      double rd = c[i0] + c[i0 + 1] + c[i0 + 2] - 1;
      if (e) *e += coef * pow(rd, 2);
      if (g) {
        g[i0] += 2 * coef * rd;
        g[i0 + 1] += 2 * coef * rd;
        g[i0 + 2] += 2 * coef * rd;
      }
    }
    /* surfaceEnergy, lines 645-654 (binary fluids only) */
    if (p->surf_area[iG] > 0 && p->ncontact > 0 && p->contact[iG] != 90 && nf == 1) {
      double w = 1 / sqrt(2.0) * cos(p->contact[iG] * 3.1415926536 / 180);
      double phi = c[iG];
      if (e) *e += w * (pow(phi, 3) / 3 - phi - 2.0 / 3) * p->surf_area[iG];
      if (g) g[iG] += w * (pow(phi, 2) - 1) * p->surf_area[iG];
    }
    /* forceEnergy, lines 657-676 */
    if (p->any_force) {
      double co[3] = {x - (p->n[0] - 1) / 2.0, y - (p->n[1] - 1) / 2.0, z - (p->n[2] - 1) / 2.0};
      for (int f = 0; f < nf; f++) {
        if (!(p->fmag[f] > 0)) continue;
        const double* fn = p->fnorm + 3 * f;
        double h = -(co[0] * fn[0] + co[1] * fn[1] + co[2] * fn[2]) * p->res;
        int iD = iG * nf + f;
        double cc = (nf == 1) ? 0.5 * (1 + c[iD]) : c[iD];
        if (cc < 0.01) continue;
        if (e) *e += cc * V * p->fmag[f] * h;
        if (g) g[iD] += (nf == 1) ? 0.5 * V * p->fmag[f] * h : V * p->fmag[f] * h;
      }
    }
    /* ffConfinementEnergy, lines 679-692 */
    for (int f = 0; f < nf; f++) {
      if (p->confine[f] == 0) continue;
      int iD = iG * nf + f;
      double coef = p->confine[f] * p->st_mean * res2;
      double cc = c[iD], c0 = p->ff_init[iD];
      if ((c0 - 0.5) * (cc - 0.5) < 0) {
        if (e) *e += coef * pow(cc - 0.5, 2);
        if (g) g[iD] += coef * 2 * (cc - 0.5);
      }
    }
  }
  /* blockEnergyGradient: the fixed volume as an energy penalty whose
   * gradient acts on interface nodes only */
  if (p->volume_fixed) {
    double vf[64] = {0};
    for (int i = 0; i < ng * nf; i++) {
      double V = p->node_vol[i / nf];
      if (nf == 1) vf[0] += 0.5 * (c[i] + 1) * V;
      else vf[i % nf] += c[i] * V;
    }
    double coef = p->vol_const * p->st_mean / pow(p->res, 4);
    for (int f = 0; f < nf; f++) {
      double dv = vf[f] - p->volume[f];
      if (e) *e += coef * pow(dv, 2);
      if (!g) continue;
      for (int iG = 0; iG < ng; iG++) {
        int iD = iG * nf + f;
        double w = 4 * c[iD] * (1 - c[iD]);
        if (w < 0) w = 0;
        g[iD] += coef * dv * p->node_vol[iG] * w;
      }
    }
  }
}

/* The constraints PhaseFieldUnstructured::init sets (lines 239-256): the hard
 * density normal (1,..,1) over the variable fluids of every node, through
 * Potential::applyConstraints (src/Potential.cpp:102-115), then the fixed
 * fluids. */
static void pfu_constraints(const oracle_inst* o, double* v) {
  const pf_t* p = &o->pf;
  int nf = p->nfluid, ng = p->ngrid;
  int var[64], nvar = 0;
  for (int f = 0; f < nf; f++)
    if (!p->fix_fluid[f] && nvar < 64) var[nvar++] = f;
  if (nf > 1 && p->density == D_HARD) {
    for (int i = 0; i < ng; i++) {
      double nsq = 0, gn = 0;
      for (int k = 0; k < nvar; k++) nsq += 1.0;
      for (int k = 0; k < nvar; k++) gn += v[i * nf + var[k]];
      for (int k = 0; k < nvar; k++) v[i * nf + var[k]] -= gn * 1.0 / nsq;
    }
  }
  for (int f = 0; f < nf; f++)
    if (p->fix_fluid[f])
      for (int i = 0; i < ng; i++) v[i * nf + f] = 0;
}

/* phaseGradient, src/potentials/PhaseField.cpp:238-288 */
static void pf_phase_gradient(const pf_t* p, const double* c, int iGrid, int f, const int* nb,
                              double factor, double* e, double* g) {
  int nf = p->nfluid;
  int i0 = iGrid * nf + f;
  double c1 = c[i0];
  double grad2 = 0;
  for (int d = 0; d < 3; d++) {
    if (p->n[d] == 1) continue;
    int imG = nb[2 * d], ipG = nb[2 * d + 1];
    int im = imG * nf + f, ip = ipG * nf + f;
    if (!p->solid[imG] && !p->solid[ipG]) {
      double gm = c1 - c[im], gp = c1 - c[ip];
      if (e) grad2 += 0.5 * (pow(gm, 2) + pow(gp, 2));
      if (g) {
        g[i0] += factor * (gm + gp);
        g[im] -= factor * gm;
        g[ip] -= factor * gp;
      }
    } else if (!p->solid[ipG]) {
      double gp = c1 - c[ip];
      if (e) grad2 += pow(gp, 2);
      if (g) {
        g[i0] += factor * 2 * gp;
        g[ip] -= factor * 2 * gp;
      }
    } else if (!p->solid[imG]) {
      double gm = c1 - c[im];
      if (e) grad2 += pow(gm, 2);
      if (g) {
        g[i0] += factor * 2 * gm;
        g[im] -= factor * 2 * gm;
      }
    }
  }
  if (e) *e += factor * grad2;
}

/* PhaseField::energyGradient loop body, lines 662-703, with fluidEnergy
 * (365-393), surfaceEnergy (476-487), pressureEnergy (432-454),
 * densityConstraintEnergy (457-473), forceEnergy (490-518) and
 * ffConfinementEnergy (521-537).  Serial order. */
static void pf_node(const oracle_inst* o, const double* c, int x, int y, int z, double* e, double* g);

static void pf_eg(const oracle_inst* o, const double* c, double* e, double* g) {
  const pf_t* p = &o->pf;
  if (o->nthreads > 1 && p->n[0] >= 6) {
    /* x planes in three colours: a plane writes gradient terms only to its
     * own plane and the two next to it, so planes of one colour never touch
     * the same entries; the last nx % 3 planes run serially */
    const int nx3 = p->n[0] - p->n[0] % 3;
    double et = 0;
    for (int col = 0; col < 3; col++) {
#pragma omp parallel for num_threads(o->nthreads) schedule(static) reduction(+ : et)
      for (int x = col; x < nx3; x += 3) {
        double el = 0;
        for (int y = 0; y < p->n[1]; y++)
          for (int z = 0; z < p->n[2]; z++) pf_node(o, c, x, y, z, e ? &el : NULL, g);
        et += el;
      }
    }
    for (int x = nx3; x < p->n[0]; x++)
      for (int y = 0; y < p->n[1]; y++)
        for (int z = 0; z < p->n[2]; z++) pf_node(o, c, x, y, z, e ? &et : NULL, g);
    if (e) *e += et;
    return;
  }
  for (int x = 0; x < p->n[0]; x++)
    for (int y = 0; y < p->n[1]; y++)
      for (int z = 0; z < p->n[2]; z++) pf_node(o, c, x, y, z, e, g);
}

static void pf_node(const oracle_inst* o, const double* c, int x, int y, int z, double* e, double* g) {
  const pf_t* p = &o->pf;
  int nf = p->nfluid;
  double res2 = pow(p->res, 2);
  int iG = (x * p->n[1] + y) * p->n[2] + z;
  int nb[6] = {pf_idx(p, x - 1, y, z), pf_idx(p, x + 1, y, z), pf_idx(p, x, y - 1, z),
               pf_idx(p, x, y + 1, z), pf_idx(p, x, y, z - 1), pf_idx(p, x, y, z + 1)};
  double V = p->node_vol[iG];
  /* fluidEnergy */
  for (int f = 0; f < nf; f++) {
    int iD = iG * nf + f;
    double cc = c[iD];
    int iK = (p->nk == nf) ? f : iG * nf + f;
    if (nf == 1) {
      double fac = p->kappa[iK] / 16 * V;
      if (e) *e += fac * pow(cc + 1, 2) * pow(cc - 1, 2);
      if (g) g[iD] += fac * 4 * cc * (cc * cc - 1);
    } else {
      double fac = 0.5 * p->kappa[iK] * V;
      if (e) *e += fac * pow(cc, 2) * pow(cc - 1, 2);
      if (g) g[iD] += fac * 2 * cc * (cc - 1) * (2 * cc - 1);
    }
    double fac = (nf == 1) ? 0.25 * p->kappaP[iK] * V : 0.5 * p->kappaP[iK] * V;
    fac = fac / res2;
    pf_phase_gradient(p, c, iG, f, nb, fac, e, g);
  }
  /* surfaceEnergy */
  if (!(p->surf_area[iG] == 0 || p->ncontact == 0 || p->contact[iG] == 90) && nf == 1) {
    double w = 1 / sqrt(2.0) * cos(p->contact[iG] * 3.1415926536 / 180);
    double phi = c[iG];
    if (e) *e += w * (pow(phi, 3) / 3 - phi - 2.0 / 3) * p->surf_area[iG];
    if (g) g[iG] += w * (pow(phi, 2) - 1) * p->surf_area[iG];
  }
  /* pressureEnergy */
  for (int f = 0; f < nf; f++) {
    if (p->pressure[f] == 0 || p->fix_fluid[f]) continue;
    if (nf == 1) {
      double vol = 0.5 * (c[iG] + 1) * V;
      if (e) *e -= p->pressure[f] * vol;
      if (g) g[iG] -= 0.5 * p->pressure[f] * V;
    } else {
      int iD = iG * nf + f;
      double vol = c[iD] * V;
      if (e) *e -= p->pressure[f] * vol;
      if (g) g[iD] -= p->pressure[f] * V;
    }
  }
  /* densityConstraintEnergy */
  if (nf > 1 && p->density == D_SOFT) {
    double coef = p->density_const * p->st_mean * res2;
    double rd = -1;
    for (int f = 0; f < nf; f++) rd += c[iG * nf + f];
    if (e) *e += coef * pow(rd, 2);
    if (g)
      for (int f = 0; f < nf; f++) g[iG * nf + f] += 2 * coef * rd;
  }
  /* forceEnergy (note the reference's early return when no gradient
   * is requested: only the first qualifying fluid's energy counts) */
  if (!p->solid[iG] && p->any_force) {
    double co[3] = {x - (p->n[0] - 1) / 2.0, y - (p->n[1] - 1) / 2.0, z - (p->n[2] - 1) / 2.0};
    for (int f = 0; f < nf; f++) {
      if (p->fmag[f] == 0) continue;
      int iD = iG * nf + f;
      double cc = (nf == 1) ? 0.5 * (1 + c[iD]) : c[iD];
      if (cc < 0.01) continue;
      const double* fn = p->fnorm + 3 * f;
      double h = -(co[0] * fn[0] + co[1] * fn[1] + co[2] * fn[2]) * p->res;
      double epc = V * p->fmag[f] * h;
      if (e) *e += cc * epc;
      if (!g) break;
      g[iD] += (nf == 1) ? 0.5 * epc : epc;
    }
  }
  /* ffConfinementEnergy */
  for (int f = 0; f < nf; f++) {
    if (p->confine[f] == 0) continue;
    int iD = iG * nf + f;
    double coef = p->confine[f] * p->st_mean * res2;
    double cc = c[iD], c0 = p->ff_init[iD];
    if ((c0 - 0.5) * (cc - 0.5) < 0) {
      if (e) *e += coef * pow(cc - 0.5, 2);
      if (g) g[iD] += coef * 2 * (cc - 0.5);
    }
  }
}

/* specialisedConstraints, src/potentials/PhaseField.cpp:580-659 */
static void pf_constraints(const oracle_inst* o, double* v) {
  const pf_t* p = &o->pf;
  int nf = p->nfluid, ng = p->ngrid;
  int var[64], nvar = 0;
  for (int f = 0; f < nf; f++) {
    if (p->fix_fluid[f]) {
      for (int i = 0; i < ng; i++) v[i * nf + f] = 0;
    } else if (nvar < 64) {
      var[nvar++] = f;
    }
  }
  if (nf > 1 && p->density == D_HARD) {
    double nfac = 1.0 / nvar;
    for (int i = 0; i < ng; i++) {
      double comp = 0;
      for (int k = 0; k < nvar; k++) comp += v[i * nf + var[k]];
      comp *= nfac;
      for (int k = 0; k < nvar; k++) v[i * nf + var[k]] -= comp;
    }
  }
  if (p->volume_fixed) {
    double comp[64] = {0};
    for (int i = 0; i < ng; i++) {
      double V = p->node_vol[i];
      for (int k = 0; k < nvar; k++) {
        int f = var[k];
        comp[f] += v[i * nf + f] * V;
        if (p->density == D_HARD)
          for (int k2 = 0; k2 < nvar; k2++) comp[f] -= v[i * nf + var[k2]] * V / nvar;
      }
    }
    for (int k = 0; k < nvar; k++) comp[var[k]] = comp[var[k]] / p->total_volume2;
    for (int i = 0; i < ng; i++) {
      double V = p->node_vol[i];
      for (int k = 0; k < nvar; k++) {
        int f = var[k];
        v[i * nf + f] -= comp[f] * V;
        if (p->density == D_HARD)
          for (int k2 = 0; k2 < nvar; k2++) v[i * nf + var[k2]] += comp[f] * V / nvar;
      }
    }
  }
}

/* ------------------------------------------------------------------------ */
/* BarAndHinge: src/potentials/BarAndHinge.cpp                               */
/* ------------------------------------------------------------------------ */
static int cmp_pair(const void* a, const void* b) {
  const int* x = a;
  const int* y = b;
  if (x[0] != y[0]) return x[0] < y[0] ? -1 : 1;
  if (x[1] != y[1]) return x[1] < y[1] ? -1 : 1;
  return 0;
}

static void sort3(int* t) {
  int a;
  if (t[0] > t[1]) { a = t[0]; t[0] = t[1]; t[1] = a; }
  if (t[1] > t[2]) { a = t[1]; t[1] = t[2]; t[2] = a; }
  if (t[0] > t[1]) { a = t[0]; t[0] = t[1]; t[1] = a; }
}

static int in3(const int* t, int v) { return t[0] == v || t[1] == v || t[2] == v; }

static void cross3(const double* a, const double* b, double* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}
static double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

/* Topology + parameters + element list: BarAndHinge::init (16-67),
 * computeBondList (70-93), computeHingeList (96-147), computeRigidities
 * (150-210), computeLength0 (213-226), computeTheta0 (229-248). */
static int bah_setup(oracle_inst* o, const minim_gpu_bah_params* q, const double* x) {
  bah_t* b = &o->bah;
  memset(b, 0, sizeof *b);
  if (o->ndof % 3) return set_err(MINIM_GPU_ERR_INVALID, "BarAndHinge: coords must be 3 per vertex");
  b->nvert = (int)(o->ndof / 3);
  int nb = 0, bstride = 0;
  int* bl = NULL; /* bonds with adjacent vertices: up to 4 ints each + count */
  int* bcnt = NULL;
  if (q->nbond > 0) {
    nb = q->nbond;
    bstride = q->bond_stride;
    bl = xcalloc((size_t)nb * 4, sizeof(int));
    bcnt = xcalloc(nb, sizeof(int));
    for (int i = 0; i < nb; i++) {
      int k = bstride < 4 ? bstride : 4;
      for (int j = 0; j < k; j++) bl[4 * i + j] = q->bonds[i * bstride + j];
      bcnt[i] = k;
    }
  } else {
    if (q->ntri <= 0) return set_err(MINIM_GPU_ERR_INVALID, "BarAndHinge: The triangulation has not been set.");
    int* pairs = xcalloc((size_t)q->ntri * 6, sizeof(int));
    for (int t = 0; t < q->ntri; t++) {
      int s[3] = {q->tris[3 * t], q->tris[3 * t + 1], q->tris[3 * t + 2]};
      sort3(s);
      int* P = pairs + 6 * t;
      P[0] = s[0]; P[1] = s[1]; P[2] = s[0]; P[3] = s[2]; P[4] = s[1]; P[5] = s[2];
    }
    qsort(pairs, (size_t)q->ntri * 3, 2 * sizeof(int), cmp_pair);
    bl = xcalloc((size_t)q->ntri * 3 * 4, sizeof(int));
    bcnt = xcalloc((size_t)q->ntri * 3, sizeof(int));
    for (int i = 0; i < q->ntri * 3; i++) {
      if (nb > 0 && bl[4 * (nb - 1)] == pairs[2 * i] && bl[4 * (nb - 1) + 1] == pairs[2 * i + 1]) continue;
      bl[4 * nb] = pairs[2 * i];
      bl[4 * nb + 1] = pairs[2 * i + 1];
      bcnt[nb] = 2;
      nb++;
    }
    free(pairs);
    /* additional indices: third vertices of the triangles on each bond */
    for (int i = 0; i < nb; i++) {
      for (int t = 0; t < q->ntri; t++) {
        const int* T = q->tris + 3 * t;
        if (!in3(T, bl[4 * i]) || !in3(T, bl[4 * i + 1])) continue;
        for (int k = 0; k < 3; k++) {
          int v = T[k];
          int have = 0;
          for (int j = 0; j < bcnt[i]; j++) have |= (bl[4 * i + j] == v);
          if (!have && bcnt[i] < 4) bl[4 * i + bcnt[i]++] = v;
        }
      }
    }
  }
  /* hinges */
  int nh = 0;
  int* hl = NULL; /* 5 ints each: 4 nodes + bond index */
  int* hcnt = NULL;
  if (q->nhinge > 0) {
    nh = q->nhinge;
    hl = xcalloc((size_t)nh * 5, sizeof(int));
    hcnt = xcalloc(nh, sizeof(int));
    for (int i = 0; i < nh; i++) {
      int k = q->hinge_stride < 5 ? q->hinge_stride : 5;
      for (int j = 0; j < k; j++) hl[5 * i + j] = q->hinges[i * q->hinge_stride + j];
      hcnt[i] = k;
    }
  } else {
    if (q->ntri <= 0) { free(bl); free(bcnt); return set_err(MINIM_GPU_ERR_INVALID, "BarAndHinge: The triangulation has not been set."); }
    int cap = 3 * q->ntri + 1;
    hl = xcalloc((size_t)cap * 5, sizeof(int));
    hcnt = xcalloc(cap, sizeof(int));
    for (int t1 = 0; t1 < q->ntri; t1++) {
      const int* A = q->tris + 3 * t1;
      for (int t2 = t1 + 1; t2 < q->ntri; t2++) {
        const int* B = q->tris + 3 * t2;
        int sh[6] = {0, 0, 0, 0, 0, 0}, ns = 0;
        for (int i1 = 0; i1 < 3; i1++)
          for (int i2 = 0; i2 < 3; i2++) {
            if (A[i1] != B[i2]) continue;
            ns++;
            sh[i1] = 1;
            sh[3 + i2] = 1;
          }
        if (ns != 2) continue;
        if (nh >= cap) break;
        int* H = hl + 5 * nh;
        for (int i1 = 0; i1 < 3; i1++)
          if (!sh[i1]) {
            H[0] = A[i1];
            H[1] = A[(i1 + 1) % 3];
            H[2] = A[(i1 + 2) % 3];
          }
        for (int i2 = 0; i2 < 3; i2++)
          if (!sh[3 + i2]) H[3] = B[i2];
        hcnt[nh] = 4;
        nh++;
      }
    }
    for (int h = 0; h < nh; h++) {
      int* H = hl + 5 * h;
      for (int i = 0; i < nb; i++) {
        int b0 = bl[4 * i], b1 = bl[4 * i + 1];
        if ((b0 == H[1] || b1 == H[1]) && (b0 == H[2] || b1 == H[2])) {
          H[4] = i;
          hcnt[h] = 5;
          break;
        }
      }
    }
  }
  /* rigidities */
  double* kb = xcalloc(nb, sizeof(double));
  double* kh = xcalloc(nh, sizeof(double));
  int have_kb = q->n_kbond > 0, have_kh = q->n_khinge > 0;
  if (q->n_kbond == 1) for (int i = 0; i < nb; i++) kb[i] = q->kbond[0];
  else if (q->n_kbond > 1) for (int i = 0; i < nb && i < q->n_kbond; i++) kb[i] = q->kbond[i];
  if (q->n_khinge == 1) for (int i = 0; i < nh; i++) kh[i] = q->khinge[0];
  else if (q->n_khinge > 1) for (int i = 0; i < nh && i < q->n_khinge; i++) kh[i] = q->khinge[i];
  if (!have_kb || !have_kh) {
    if (q->n_thickness <= 0) {
      free(bl); free(bcnt); free(hl); free(hcnt); free(kb); free(kh);
      return set_err(MINIM_GPU_ERR_INVALID, "BarAndHinge requires either the rigidities or the thickness to be set");
    }
    double* th = xcalloc(b->nvert, sizeof(double));
    for (int i = 0; i < b->nvert; i++) th[i] = q->n_thickness == 1 ? q->thickness[0] : q->thickness[i];
    double* lsq = xcalloc(nb, sizeof(double));
    double* asum = xcalloc(nb, sizeof(double));
    for (int i = 0; i < nb; i++) {
      if (bcnt[i] == 2) {
        free(th); free(lsq); free(asum);
        free(bl); free(bcnt); free(hl); free(hcnt); free(kb); free(kh);
        return set_err(MINIM_GPU_ERR_INVALID, "The bondList should contain the indicies of the adjacent triangles.");
      }
      const double* x1 = x + 3 * bl[4 * i];
      const double* x2 = x + 3 * bl[4 * i + 1];
      double d21[3] = {x2[0] - x1[0], x2[1] - x1[1], x2[2] - x1[2]};
      lsq[i] = pow(d21[0], 2) + pow(d21[1], 2) + pow(d21[2], 2);
      for (int j = 2; j < bcnt[i]; j++) {
        const double* x3 = x + 3 * bl[4 * i + j];
        double d31[3] = {x3[0] - x1[0], x3[1] - x1[1], x3[2] - x1[2]}, cr[3];
        cross3(d21, d31, cr);
        asum[i] += fabs(sqrt(dot3(cr, cr))) / 2;
      }
    }
    if (!have_kb)
      for (int i = 0; i < nb; i++) {
        double t = (th[bl[4 * i]] + th[bl[4 * i + 1]]) / 2;
        kb[i] = q->modulus * t * (asum[i] / lsq[i]);
      }
    if (!have_kh)
      for (int h = 0; h < nh; h++) {
        if (hcnt[h] == 4) {
          free(th); free(lsq); free(asum);
          free(bl); free(bcnt); free(hl); free(hcnt); free(kb); free(kh);
          return set_err(MINIM_GPU_ERR_INVALID, "The hingeList should contain the index of the bond.");
        }
        const int* H = hl + 5 * h;
        double t = (th[H[0]] + th[H[1]] + th[H[2]] + th[H[3]]) / 4;
        double rig = q->modulus * pow(t, 3) / (12 * (1 - pow(q->poisson_ratio, 2)));
        kh[h] = rig * (lsq[H[4]] / asum[H[4]]);
      }
    free(th); free(lsq); free(asum);
  }
  /* rest lengths and angles */
  double* l0 = xcalloc(nb, sizeof(double));
  for (int i = 0; i < nb; i++) {
    if (q->n_length0 == 1) l0[i] = q->length0[0];
    else if (q->n_length0 > 1) l0[i] = q->length0[i];
    else {
      const double* x1 = x + 3 * bl[4 * i];
      const double* x2 = x + 3 * bl[4 * i + 1];
      double d[3] = {x1[0] - x2[0], x1[1] - x2[1], x1[2] - x2[2]};
      l0[i] = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    }
  }
  double* t0 = xcalloc(nh, sizeof(double));
  for (int h = 0; h < nh; h++) {
    if (q->n_theta0 == 1) t0[h] = q->theta0[0];
    else if (q->n_theta0 > 1) t0[h] = q->theta0[h];
    else {
      const int* H = hl + 5 * h;
      const double *x1 = x + 3 * H[0], *x2 = x + 3 * H[1], *x3 = x + 3 * H[2], *x4 = x + 3 * H[3];
      double a[3], bb[3], c[3], n1[3], n2[3];
      for (int d = 0; d < 3; d++) { a[d] = x2[d] - x1[d]; bb[d] = x3[d] - x2[d]; c[d] = x4[d] - x3[d]; }
      cross3(a, bb, n1);
      cross3(bb, c, n2);
      double cs = dot3(n1, n2) / (sqrt(dot3(n1, n1)) * sqrt(dot3(n2, n2)));
      double n1b3 = dot3(n1, c);
      t0[h] = (n1b3 >= 0) ? acos(cs) : 2 * PI_REF - acos(cs);
    }
  }
  /* elements (skip those whose dofs are all fixed) */
  b->bars = xcalloc((size_t)nb * 2, sizeof(int));
  b->bpar = xcalloc((size_t)nb * 2, sizeof(double));
  b->hinges = xcalloc((size_t)nh * 4, sizeof(int));
  b->hpar = xcalloc((size_t)nh * 2, sizeof(double));
  for (int i = 0; i < nb; i++) {
    int allfix = o->fixed != NULL;
    for (int k = 0; k < 2 && allfix; k++)
      for (int d = 0; d < 3; d++) allfix &= o->fixed[3 * bl[4 * i + k] + d] != 0;
    if (allfix) continue;
    b->bars[2 * b->nbar] = bl[4 * i];
    b->bars[2 * b->nbar + 1] = bl[4 * i + 1];
    b->bpar[2 * b->nbar] = kb[i];
    b->bpar[2 * b->nbar + 1] = l0[i];
    b->nbar++;
  }
  for (int h = 0; h < nh; h++) {
    int allfix = o->fixed != NULL;
    for (int k = 0; k < 4 && allfix; k++)
      for (int d = 0; d < 3; d++) allfix &= o->fixed[3 * hl[5 * h + k] + d] != 0;
    if (allfix) continue;
    for (int k = 0; k < 4; k++) b->hinges[4 * b->nhinge + k] = hl[5 * h + k];
    b->hpar[2 * b->nhinge] = kh[h];
    b->hpar[2 * b->nhinge + 1] = t0[h];
    b->nhinge++;
  }
  b->node_el = xcalloc(b->nvert, 1);
  for (int v = 0; v < b->nvert; v++) {
    int allfix = o->fixed != NULL;
    for (int d = 0; d < 3 && allfix; d++) allfix &= o->fixed[3 * v + d] != 0;
    b->node_el[v] = !allfix;
  }
  b->nforce = q->n_force;
  if (q->n_force > 0) {
    b->force = xcalloc(q->n_force, sizeof(double));
    memcpy(b->force, q->force, q->n_force * sizeof(double));
  }
  b->wall_on = q->wall_on;
  b->wall_adh = q->wall_adhesion;
  b->wall_eps = q->wall_epsilon;
  b->wall_sig = q->wall_sigma;
  free(bl); free(bcnt); free(hl); free(hcnt); free(kb); free(kh); free(l0); free(t0);
  return 0;
}

/* stretching (269-290), bending (293-356), forceEnergy (359-369),
 * substrate (372-387), evaluated in element order. */
static void bah_eg(const oracle_inst* o, const double* x, double* e, double* g) {
  const bah_t* b = &o->bah;
  for (int i = 0; i < b->nbar; i++) {
    int n1 = b->bars[2 * i], n2 = b->bars[2 * i + 1];
    double dx[3] = {x[3 * n1] - x[3 * n2], x[3 * n1 + 1] - x[3 * n2 + 1], x[3 * n1 + 2] - x[3 * n2 + 2]};
    double l = sqrt(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
    double dl = l - b->bpar[2 * i + 1];
    double k = b->bpar[2 * i];
    if (e) *e += 0.5 * k * pow(dl, 2);
    if (g) {
      double gf = 2 * k * dl / l; /* the reference's factor of 2 */
      for (int d = 0; d < 3; d++) {
        g[3 * n1 + d] += gf * dx[d];
        g[3 * n2 + d] -= gf * dx[d];
      }
    }
  }
  for (int h = 0; h < b->nhinge; h++) {
    const int* H = b->hinges + 4 * h;
    const double *x1 = x + 3 * H[0], *x2 = x + 3 * H[1], *x3 = x + 3 * H[2], *x4 = x + 3 * H[3];
    double b1[3], b2[3], b3[3], n1[3], n2[3];
    for (int d = 0; d < 3; d++) { b1[d] = x2[d] - x1[d]; b2[d] = x3[d] - x2[d]; b3[d] = x4[d] - x3[d]; }
    double b2m = sqrt(dot3(b2, b2));
    cross3(b1, b2, n1);
    cross3(b2, b3, n2);
    double n1sq = dot3(n1, n1), n2sq = dot3(n2, n2);
    double n12m = sqrt(n1sq * n2sq);
    double c = dot3(n1, n2) / n12m;
    if (c < -1.0) c = -1.0;
    if (c > 1.0) c = 1.0;
    double n1b3 = dot3(n1, b3);
    double th = (n1b3 >= 0) ? acos(c) : 2 * PI_REF - acos(c);
    double dth = th - b->hpar[2 * h + 1];
    dth = fmod(dth + PI_REF, 2 * PI_REF) - PI_REF;
    double k = b->hpar[2 * h];
    if (e) *e += 0.5 * k * pow(dth, 2);
    if (g) {
      double gf = k * dth;
      double n1h[3], n2h[3];
      for (int d = 0; d < 3; d++) { n1h[d] = b2m / n1sq * n1[d]; n2h[d] = b2m / n2sq * n2[d]; }
      double sk1 = -dot3(b1, b2) / (b2m * b2m);
      double sk2 = -dot3(b3, b2) / (b2m * b2m);
      for (int d = 0; d < 3; d++) {
        g[3 * H[0] + d] += -gf * n1h[d];
        g[3 * H[1] + d] += gf * ((1 - sk1) * n1h[d] - sk2 * n2h[d]);
        g[3 * H[2] + d] += -gf * ((1 - sk2) * n2h[d] - sk1 * n1h[d]);
        g[3 * H[3] + d] += gf * n2h[d];
      }
    }
  }
  for (int v = 0; v < b->nvert; v++) {
    if (!b->node_el[v]) continue;
    double fz = 0;
    if (b->nforce == 3) fz = b->force[2];
    else if (b->nforce > 0) fz = b->force[3 * v + 2];
    if (e) *e -= fz * x[3 * v + 2];
    if (g) g[3 * v + 2] -= fz;
    if (b->wall_on) {
      double hgt = x[3 * v + 2];
      if (!b->wall_adh && hgt > 0) continue;
      double r0 = 0.858374218932559 * b->wall_sig;
      hgt = fmax(hgt + r0, r0 / 2);
      double lj9 = 2.0 / 15 * pow(b->wall_sig / hgt, 9);
      double lj3 = pow(b->wall_sig / hgt, 3);
      double s3 = pow(b->wall_sig, 3);
      double s9 = pow(s3, 3);
      double lj9_0 = 0.5270462766947298 * s9;
      double lj3_0 = 1.5811388300841895 * s3;
      if (e) *e += b->wall_eps * ((lj9 - lj9_0) - (lj3 - lj3_0));
      if (g) g[3 * v + 2] -= b->wall_eps * (9 * lj9 - 3 * lj3) / hgt;
    }
  }
}

/* ------------------------------------------------------------------------ */
/* State-level evaluation: elementEG / basicEG (src/State.cpp:48-79) and      */
/* Potential::applyConstraints (src/Potential.cpp:102-115)                   */
/* ------------------------------------------------------------------------ */
static void apply_constraints(const oracle_inst* o, double* v) {
  if (o->kind == MINIM_GPU_PFU) {
    /* init replaces the constraint list (PhaseFieldUnstructured.cpp:240), so
     * fixed degrees of freedom set on the state come after its own */
    pfu_constraints(o, v);
    if (o->fixed)
      for (size_t i = 0; i < o->ndof; i++)
        if (o->fixed[i]) v[i] = 0;
    return;
  }
  if (o->fixed)
    for (size_t i = 0; i < o->ndof; i++)
      if (o->fixed[i]) v[i] = 0;
  if (o->kind == MINIM_GPU_PF) pf_constraints(o, v);
}

static void raw_eg(const oracle_inst* o, const double* x, double* e, double* g) {
  if (o->kind == MINIM_GPU_LJ) lj_eg(o, x, e, g);
  else if (o->kind == MINIM_GPU_PF) pf_eg(o, x, e, g);
  else if (o->kind == MINIM_GPU_PFU) pfu_eg(o, x, e, g);
  else bah_eg(o, x, e, g);
}

/* State::energy(coords): energy-only evaluation. */
static double st_energy(oracle_inst* o, const double* x) {
  double e = 0;
  raw_eg(o, x, &e, NULL);
  o->evals++;
  return e;
}

/* State::gradient(coords): zeroed, evaluated, constrained. */
static void st_gradient(oracle_inst* o, const double* x, double* g) {
  memset(g, 0, o->ndof * sizeof(double));
  raw_eg(o, x, NULL, g);
  apply_constraints(o, g);
  o->evals++;
}

int oracle_energy_gradient(oracle_inst* o, const double* x, double* e, double* g) {
  const double* xx = x ? x : o->x;
  if (e) *e = st_energy(o, xx);
  if (g) st_gradient(o, xx, g);
  return 0;
}

int oracle_apply_constraints(oracle_inst* o, double* v) {
  apply_constraints(o, v);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Vector algebra (Communicator::dotProduct, 1 rank: src/Communicator.cpp:170-173) */
/* ------------------------------------------------------------------------ */
static double vdot(const oracle_inst* o, const double* a, const double* b, size_t n) {
  double s = 0;
#pragma omp parallel for if(o->nthreads > 1) num_threads(o->nthreads) schedule(static) reduction(+ : s)
  for (size_t i = 0; i < n; i++) s += a[i] * b[i];
  return s;
}

/* backtrackingLinesearch, src/minimisers/linesearch.cpp:8-30.
 * Moves o->x; step is scaled in place. */
static double linesearch(oracle_inst* o, double* step, double de0, double* tmp) {
  const double c = 0.5, tau = 0.5;
  size_t n = o->ndof;
  double t = -c * de0;
  double e0 = st_energy(o, o->x);
  double mult = 1;
  OMP_FOR
  for (size_t i = 0; i < n; i++) tmp[i] = o->x[i] + step[i];
  for (int k = 0; k < 10; k++) {
    double e = st_energy(o, tmp);
    if (e0 - e >= t) break;
    OMP_FOR
    for (size_t i = 0; i < n; i++) {
      step[i] = step[i] * tau;
      tmp[i] = o->x[i] + step[i];
    }
    mult = mult * tau;
    t = t * tau;
  }
  memcpy(o->x, tmp, n * sizeof(double));
  return mult;
}

/* Minimiser::minimise loop (src/Minimiser.cpp:27-38) with Lbfgs
 * (src/minimisers/Lbfgs.cpp:34-133), Fire (src/minimisers/Fire.cpp:27-90)
 * and GradDescent (src/minimisers/GradDescent.cpp:22-46). */
/* ------------------------------------------------------------------------ */
/* Anneal: src/minimisers/Anneal.cpp:45-95                                   */
/* ------------------------------------------------------------------------ */
/* The device engine's random numbers: SplitMix64's output mix (Steele, Lea
 * and Flood 2014) applied twice to a counter made of the iteration and the
 * coordinate index, keyed by the seed; 53 bits give u in [0, 1). */
static uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}
static double anneal_unit(uint64_t seed, int iter, uint32_t idx) {
  uint64_t h = mix64(seed ^ mix64(((uint64_t)(uint32_t)iter << 32) | idx));
  return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

/* one random number: counter mode (the device engine's) or the C library's
 * rand() in the reference's call order (to pin this restatement to the
 * reference library itself) */
typedef struct {
  int libc;
  uint64_t seed;
} anneal_rng;
static double anneal_draw(const anneal_rng* r, int iter, uint32_t idx) {
  if (r->libc) return (double)rand() / RAND_MAX;
  return anneal_unit(r->seed, iter, idx);
}

static int anneal_run(oracle_inst* o, const minim_gpu_minimiser_params* mp, const anneal_rng* rng,
                      minim_gpu_result* res) {
  size_t n = o->ndof;
  int maxIter = mp->max_iter;
  double* cur = xcalloc(n, sizeof(double));
  o->evals = 0;
  /* init: _sinceAccepted = 0, _currentState, _currentE */
  memcpy(cur, o->x, n * sizeof(double));
  double curE = st_energy(o, o->x);
  int since = 0, iter;
  for (iter = 0; iter <= maxIter; iter++) {
    double T;
    if (mp->n_temp_schedule > 0) {
      int k = iter < mp->n_temp_schedule ? iter : mp->n_temp_schedule - 1;
      T = mp->temp_schedule[k];
    } else {
      T = mp->temp_init / (1 + mp->cooling_rate * iter);
    }
    for (size_t j = 0; j < n; j++) {
      double random = 2 * anneal_draw(rng, iter, (uint32_t)j) - 1;
      o->x[j] = cur[j] + random * mp->displacement;
    }
    double e = st_energy(o, o->x);
    /* acceptMetropolis: the random number is drawn before the comparison */
    double u = anneal_draw(rng, iter, (uint32_t)n);
    int accept = (e < curE) ? 1 : (u < exp((curE - e) / T));
    if (accept) {
      memcpy(cur, o->x, n * sizeof(double));
      curE = e;
      since = 0;
    } else {
      since++;
    }
    int conv = (mp->max_rejections > 0) && (since >= mp->max_rejections);
    if (conv || iter == maxIter) memcpy(o->x, cur, n * sizeof(double));
    if (conv) break;
  }
  free(cur);
  if (res) {
    memset(res, 0, sizeof *res);
    res->iter = iter;
    res->status = iter <= maxIter ? MINIM_RES_CONVERGED : MINIM_RES_MAXITER;
    res->fp64_iters = iter <= maxIter ? iter + 1 : maxIter + 1;
    res->evals = (int)o->evals;
    res->energy = curE;
    res->rms = 0; /* no gradient */
  }
  return 0;
}

int oracle_anneal_libc(oracle_inst* o, const minim_gpu_minimiser_params* mp, unsigned seed,
                       minim_gpu_result* res) {
  anneal_rng r = {1, 0};
  srand(seed);
  return anneal_run(o, mp, &r, res);
}

int oracle_minimise(oracle_inst* o, const minim_gpu_minimiser_params* mp, minim_gpu_result* res) {
  if (mp->method == MINIM_ANNEAL) {
    anneal_rng r = {0, mp->seed};
    return anneal_run(o, mp, &r, res);
  }
  size_t n = o->ndof;
  double tol = mp->tol >= 0 ? mp->tol : o->tol_default;
  int ls = mp->linesearch == MINIM_LS_BACKTRACKING;
  int maxIter = mp->max_iter;
  double* g = xcalloc(n, sizeof(double));
  double* gn = xcalloc(n, sizeof(double));
  double* step = xcalloc(n, sizeof(double));
  double* tmp = xcalloc(n, sizeof(double));
  int iter = 0;
  double dtmax = mp->dt_max;
  o->evals = 0;
  if (mp->method == MINIM_LBFGS) {
    int m = mp->m;
    double* S = xcalloc((size_t)m * n, sizeof(double));
    double* Y = xcalloc((size_t)m * n, sizeof(double));
    double* rho = xcalloc(m, sizeof(double));
    double* alpha = xcalloc(m, sizeof(double));
    int ii = 0;
    for (iter = 0; iter <= maxIter; iter++) {
      /* iteration */
      if (iter == 0) { st_gradient(o, o->x, g); ii = 0; }
      else ii++;
      /* getDirection */
      int mt = ii < m ? ii : m;
      int ic = ii % m;
      OMP_FOR
      for (size_t j = 0; j < n; j++) step[j] = -g[j];
      if (ii == 0) {
        double gnorm = sqrt(vdot(o, g, g, n));
        if (gnorm > 0)
          OMP_FOR
          for (size_t j = 0; j < n; j++) step[j] *= mp->init_step / gnorm;
      } else {
        for (int i1 = 0; i1 < mt; i1++) {
          int k = ((ic - 1 - i1) + m) % m;
          alpha[k] = rho[k] * vdot(o, step, S + (size_t)k * n, n);
          OMP_FOR
          for (size_t j = 0; j < n; j++) step[j] -= alpha[k] * Y[(size_t)k * n + j];
        }
        int k = (ic - 1 + m) % m;
        double gamma = 1 / (rho[k] * vdot(o, Y + (size_t)k * n, Y + (size_t)k * n, n));
        OMP_FOR
        for (size_t j = 0; j < n; j++) step[j] *= gamma;
        for (int i1 = 0; i1 < mt; i1++) {
          int kk = ((ic - mt + i1) + m) % m;
          double beta = rho[kk] * vdot(o, step, Y + (size_t)kk * n, n);
          OMP_FOR
          for (size_t j = 0; j < n; j++) step[j] += (alpha[kk] - beta) * S[(size_t)kk * n + j];
        }
        if (mp->max_step != 0) {
          double ss = sqrt(vdot(o, step, step, n));
          if (ss > mp->max_step)
            OMP_FOR
            for (size_t j = 0; j < n; j++) step[j] *= mp->max_step / ss;
        }
      }
      apply_constraints(o, step);
      double gs = vdot(o, g, step, n);
      if (gs > 0) {
        gs = -gs;
        OMP_FOR
        for (size_t j = 0; j < n; j++) step[j] = -step[j];
      }
      if (ls) linesearch(o, step, gs, tmp);
      else for (size_t j = 0; j < n; j++) o->x[j] += step[j];
      st_gradient(o, o->x, gn);
      OMP_FOR
      for (size_t j = 0; j < n; j++) tmp[j] = gn[j] - g[j];
      double sy = vdot(o, step, tmp, n);
      if (sy != 0) {
        int c = ii % m;
        memcpy(S + (size_t)c * n, step, n * sizeof(double));
        memcpy(Y + (size_t)c * n, tmp, n * sizeof(double));
        rho[c] = 1 / sy;
      } else {
        ii--;
      }
      memcpy(g, gn, n * sizeof(double));
      /* checkConvergence */
      if (sqrt(vdot(o, g, g, n) / n) < tol) break;
    }
    free(S); free(Y); free(rho); free(alpha);
  } else if (mp->method == MINIM_FIRE) {
    const int nMin = 5;
    const double fInc = 1.1, fDec = 0.5, fA = 0.99, aStart = 0.1;
    double* v = xcalloc(n, sizeof(double));
    double gNorm = 0, dt = 0, a = 0;
    int nSteps = 0;
    if (dtmax == 0) { /* Fire::init */
      st_gradient(o, o->x, g);
      gNorm = sqrt(vdot(o, g, g, n));
      dtmax = (gNorm != 0) ? 0.1 / sqrt(gNorm) : 1;
    }
    for (iter = 0; iter <= maxIter; iter++) {
      if (iter == 0) {
        dt = dtmax;
        st_gradient(o, o->x, g);
        gNorm = sqrt(vdot(o, g, g, n));
      }
      double p = -vdot(o, v, g, n);
      if (p > 0) {
        double vNorm = sqrt(vdot(o, v, v, n));
        OMP_FOR
        for (size_t j = 0; j < n; j++) v[j] = (1 - a) * v[j] - (a * vNorm / gNorm + dt) * g[j];
        nSteps++;
      } else {
        OMP_FOR
        for (size_t j = 0; j < n; j++) v[j] = -dt * g[j];
        nSteps = 0;
      }
      if (p > 0 && nSteps > nMin) {
        a = a * fA;
        dt = dt * fInc;
        if (dt > dtmax) dt = dtmax;
      } else if (p <= 0) {
        a = aStart;
        dt = dt * fDec;
      }
      OMP_FOR
      for (size_t j = 0; j < n; j++) step[j] = dt * v[j];
      apply_constraints(o, step);
      if (ls) {
        double gs = vdot(o, g, step, n);
        linesearch(o, step, gs, tmp);
      } else {
        OMP_FOR
        for (size_t j = 0; j < n; j++) o->x[j] += step[j];
      }
      st_gradient(o, o->x, g);
      gNorm = sqrt(vdot(o, g, g, n));
      if (gNorm / sqrt((double)n) < tol) break;
    }
    free(v);
  } else if (mp->method == MINIM_GD) {
    for (iter = 0; iter <= maxIter; iter++) {
      st_gradient(o, o->x, g);
      OMP_FOR
      for (size_t j = 0; j < n; j++) step[j] = -mp->alpha * g[j];
      if (ls) {
        double gs = vdot(o, g, step, n);
        linesearch(o, step, gs, tmp);
      } else {
        OMP_FOR
        for (size_t j = 0; j < n; j++) o->x[j] += step[j];
      }
      if (sqrt(vdot(o, g, g, n) / n) < tol) break;
    }
  } else {
    free(g); free(gn); free(step); free(tmp);
    return set_err(MINIM_GPU_ERR_INVALID, "unknown minimiser");
  }
  if (res) {
    memset(res, 0, sizeof *res);
    res->iter = iter;
    res->status = iter <= maxIter ? MINIM_RES_CONVERGED : MINIM_RES_MAXITER;
    res->fp64_iters = iter <= maxIter ? iter + 1 : maxIter + 1;
    long ev = o->evals;
    res->energy = st_energy(o, o->x);
    st_gradient(o, o->x, g);
    res->rms = sqrt(vdot(o, g, g, n) / n);
    res->evals = (int)ev;
    res->dt_max = dtmax;
    if (!(res->energy == res->energy)) res->status = MINIM_RES_NAN;
  }
  free(g); free(gn); free(step); free(tmp);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Construction                                                              */
/* ------------------------------------------------------------------------ */
void oracle_destroy(oracle_inst* o) {
  if (!o) return;
  free(o->x);
  free(o->fixed);
  pf_t* p = &o->pf;
  free(p->kappa); free(p->kappaP); free(p->node_vol); free(p->surf_area); free(p->solid);
  free(p->contact); free(p->pressure); free(p->fix_fluid); free(p->confine); free(p->ff_init);
  free(p->fmag); free(p->fnorm); free(p->volume);
  bah_t* b = &o->bah;
  free(b->bars); free(b->bpar); free(b->hinges); free(b->hpar); free(b->node_el); free(b->force);
  free(o);
}

int oracle_create(int kind, const void* params, const double* x0, size_t ndof,
                  const int* fixed, int nfixed, oracle_inst** out) {
  *out = NULL;
  oracle_inst* o = xcalloc(1, sizeof *o);
  o->nthreads = 1;
  o->kind = kind;
  o->ndof = ndof;
  o->x = xcalloc(ndof, sizeof(double));
  memcpy(o->x, x0, ndof * sizeof(double));
  o->tol_default = 1e-6; /* Potential::convergence default, include/Potential.h:22 */
  if (nfixed > 0) {
    o->fixed = xcalloc(ndof, 1);
    for (int i = 0; i < nfixed; i++)
      if (fixed[i] >= 0 && (size_t)fixed[i] < ndof) o->fixed[fixed[i]] = 1;
  }
  int rc = 0;
  if (kind == MINIM_GPU_LJ) {
    const minim_gpu_lj_params* q = params;
    o->ndim = q->ndim;
    o->sigma = q->sigma;
    o->eps = q->epsilon;
    o->rc2 = q->cutoff > 0 ? q->cutoff * q->cutoff : 0.0;
    if (q->ndim < 1 || q->ndim > 3 || ndof % q->ndim)
      rc = set_err(MINIM_GPU_ERR_INVALID, "LjNd: Length of coords must be a multiple of the number of dimensions.");
  } else if (kind == MINIM_GPU_PF || kind == MINIM_GPU_PFU) {
    rc = pf_setup(o, params, x0, kind == MINIM_GPU_PFU);
  } else if (kind == MINIM_GPU_BAH) {
    rc = bah_setup(o, params, x0);
  } else {
    rc = set_err(MINIM_GPU_ERR_INVALID, "unknown potential kind");
  }
  if (rc) {
    oracle_destroy(o);
    return rc;
  }
  *out = o;
  return 0;
}

int oracle_set_coords(oracle_inst* o, const double* x) {
  memcpy(o->x, x, o->ndof * sizeof(double));
  return 0;
}

int oracle_get_coords(const oracle_inst* o, double* x) {
  memcpy(x, o->x, o->ndof * sizeof(double));
  return 0;
}

int oracle_bah_elements(const oracle_inst* o, int* nbar, const int** bars, const double** bar_par,
                        int* nhinge, const int** hinges, const double** hinge_par) {
  if (o->kind != MINIM_GPU_BAH) return set_err(MINIM_GPU_ERR_INVALID, "not a BarAndHinge instance");
  *nbar = o->bah.nbar;
  *bars = o->bah.bars;
  *bar_par = o->bah.bpar;
  *nhinge = o->bah.nhinge;
  *hinges = o->bah.hinges;
  *hinge_par = o->bah.hpar;
  return 0;
}

int oracle_pf_internals(const oracle_inst* o, const double** kappa, const double** kappaP,
                        const double** node_vol, const double** surface_area, int* nk) {
  if (o->kind != MINIM_GPU_PF && o->kind != MINIM_GPU_PFU)
    return set_err(MINIM_GPU_ERR_INVALID, "not a PhaseField instance");
  *kappa = o->pf.kappa;
  *kappaP = o->pf.kappaP;
  *node_vol = o->pf.node_vol;
  *surface_area = o->pf.surf_area;
  *nk = o->pf.nk;
  return 0;
}
