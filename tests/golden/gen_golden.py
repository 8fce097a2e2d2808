"""Generates the golden fixtures in this folder from the reference minim
library itself (oracle/_ref/libminim_ref.so, built from the reference's own
sources by oracle/Makefile; run `make -C oracle ref` first).

Each case stores the potential description (keyword arguments of
minim_gb300.abi.*), the inputs and the reference's outputs:
  lj_eg / pf_eg / bah_eg : energy and constrained gradient at x (State::energy,
                           State::gradient), plus applyConstraints of a vector
  *_min                  : Minimiser::minimise results (final x, energy, iter)
  pf_setup               : kappa, kappaP, nodeVol, surfaceArea
  bah_setup              : element lists (bars, hinges) with their parameters
  pfu_eg / pfu_min       : the same for PhaseFieldUnstructured
  anneal_min             : Anneal runs with rand() seeded by srand(seed) after
                           Anneal::init (the reference seeds it from the clock)
Usage: python tests/golden/gen_golden.py [lj] [pf] [bah] [pfu] [anneal]   (default: all)
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from minim_gb300 import abi  # noqa: E402
from oracle.oracle import Reference  # noqa: E402
from tests.workloads import Rng, lj_cluster, pf_noise, pf_simplex, sheet  # noqa: E402


def params_from(kind, kw):
    kw = dict(kw)
    if kind == "lj":
        return abi.lj(**kw)
    if kind in ("pf", "pfu"):
        for k in ("solid", "fix_fluid"):
            if k in kw and kw[k] is not None:
                kw[k] = np.asarray(kw[k], np.uint8)
        return abi.phase_field(**kw) if kind == "pf" else abi.phase_field_unstructured(**kw)
    if kind == "bah":
        return abi.bar_and_hinge(**kw)
    raise ValueError(kind)


def mp_from(kw):
    return abi.minimiser(**kw)


def tolist(v):
    if isinstance(v, np.ndarray):
        return v.tolist()
    if isinstance(v, (list, tuple)):
        return [tolist(a) for a in v]
    return v


def eg_case(name, kind, kw, x0, x=None, fixed=None, seed=0):
    p = params_from(kind, kw)
    ref = Reference(p, x0, fixed=fixed)
    xe = x0 if x is None else x
    e, g = ref.energy_gradient(xe)
    v = Rng(seed + 99).normal(len(x0))
    vc = ref.apply_constraints(v)
    return {"name": name, "kind": kind, "params": json.dumps({k: tolist(v_) for k, v_ in kw.items()}),
            "x0": np.asarray(x0, float), "x": np.asarray(xe, float), "energy": e, "gradient": g,
            "fixed": np.asarray(fixed if fixed is not None else [], np.int32), "v": v, "v_constrained": vc,
            "default_tol": ref.default_tol}


def min_case(name, kind, kw, x0, mkw, fixed=None, coords=None):
    p = params_from(kind, kw)
    ref = Reference(p, x0, fixed=fixed)
    if coords is not None:
        ref.coords = coords
    r = ref.minimise(mp_from(mkw))
    return {"name": name, "kind": kind, "params": json.dumps({k: tolist(v_) for k, v_ in kw.items()}),
            "minimiser": json.dumps(mkw), "x0": np.asarray(x0, float),
            "start": np.asarray(coords if coords is not None else x0, float),
            "fixed": np.asarray(fixed if fixed is not None else [], np.int32),
            "x_final": ref.coords, "energy": r.energy, "rms": r.rms, "iter": r.iter, "status": r.status,
            "dt_max": r.dt_max}


def save(fname, cases):
    out = {}
    for i, c in enumerate(cases):
        for k, v in c.items():
            out[f"{i}:{k}"] = v
    out["ncases"] = len(cases)
    np.savez_compressed(os.path.join(HERE, fname), **out)


def main(parts):
    parts = set(parts) or {"lj", "pf", "bah", "pfu", "anneal"}
    if "lj" in parts:
        gen_lj()
    if "pf" in parts:
        gen_pf()
    if "bah" in parts:
        gen_bah()
    if "pfu" in parts:
        gen_pfu()
    if "anneal" in parts:
        gen_anneal()
    print("wrote fixtures to", HERE)


def gen_lj():
    lj = [eg_case("pair_kat", "lj", {}, [0, 0, 0, 2, 0, 0])]
    for n, nd, sig, eps in [(13, 3, 1.0, 1.0), (40, 3, 1.1, 0.7), (25, 2, 1.0, 1.0)]:
        x = lj_cluster(n, seed=n, ndim=nd)
        lj.append(eg_case(f"lj{n}_{nd}d", "lj", {"ndim": nd, "sigma": sig, "epsilon": eps}, x, seed=n))
    lj.append(eg_case("lj20_fixed", "lj", {}, lj_cluster(20, seed=1), fixed=[0, 1, 2, 17, 40]))
    save("lj_eg.npz", lj)
    ljm = []
    for meth, mkw in [("lbfgs", {"method": "lbfgs", "tol": 1e-6}),
                      ("lbfgs_m3_maxstep", {"method": "lbfgs", "m": 3, "max_step": 0.3, "tol": 1e-6}),
                      ("fire_ls", {"method": "fire", "linesearch": "backtracking", "tol": 1e-6}),
                      ("fire_dt", {"method": "fire", "dt_max": 0.1, "tol": 1e-6, "max_iter": 5000}),
                      ("gd", {"method": "gd", "tol": 1e-4, "max_iter": 20000}),
                      ("gd_nols", {"method": "gd", "linesearch": "none", "alpha": 0.01, "tol": 1e-4,
                                   "max_iter": 20000})]:
        ljm.append(min_case(f"lj13_{meth}", "lj", {}, lj_cluster(13, seed=5), mkw))
    ljm.append(min_case("config0_small_lbfgs", "lj", {}, lj_cluster(38, seed=0),
                        {"method": "lbfgs", "m": 5, "tol": 1e-6}))
    save("lj_min.npz", ljm)


def gen_pf():
    pf = []
    pf.append(eg_case("binary_3d", "pf", {"grid": [6, 5, 4]}, pf_noise((6, 5, 4), seed=2, amp=0.5)))
    pf.append(eg_case("binary_res2_pressure", "pf", {"grid": [5, 6, 7], "resolution": 2.0, "pressure": [1.5]},
                      pf_noise((5, 6, 7), seed=3, amp=0.9)))
    solid = np.zeros((9, 8, 5), np.uint8)
    solid[3:5, 2:4, 1:3] = 1
    solid[:, 0, :] = 1
    ca = Rng(4).uniform(solid.size) * 120 + 30
    pf.append(eg_case("binary_solid_contact_force", "pf",
                      {"grid": [9, 8, 5], "solid": solid.ravel(), "contact_angle": ca,
                       "force": [0.1, -0.3, 0.2], "pressure": [0.4]}, pf_noise((9, 8, 5), seed=4, amp=0.9)))
    walls = np.zeros((12, 10, 1), np.uint8)
    walls[:, 0, :] = 1
    for dens in ["hard", "soft", "none", "fixed"]:
        pf.append(eg_case(f"ternary_{dens}", "pf",
                          {"grid": [12, 10, 1], "nfluid": 3, "solid": walls.ravel(), "volume_fixed": True,
                           "density_constraint": dens, "surface_tension": [1.0, 0.8, 1.2],
                           "pressure": [0, 0.3, 0], "force": [[0, -1, 0], [0.2, 0, 0], [0, 0, 0]],
                           "confinement": [0, 1.0, 0]}, pf_simplex((12, 10, 1), 3, seed=5), seed=5))
    pf.append(eg_case("binary_fixfluid_nodetension", "pf",
                      {"grid": [6, 5, 3], "nfluid": 2, "surface_tension": 0.5 + Rng(7).uniform(180),
                       "fix_fluid": [1, 0], "density_constraint": "none"}, pf_simplex((6, 5, 3), 2, seed=7)))
    save("pf_eg.npz", pf)
    pfm = [min_case("binary_8cubed", "pf", {"grid": [8, 8, 8]}, pf_noise((8, 8, 8), seed=21),
                    {"method": "lbfgs", "m": 10, "tol": 1e-7}),
           min_case("ternary_volume_16", "pf", {"grid": [16, 16, 1], "nfluid": 3, "volume_fixed": True},
                    pf_simplex((16, 16, 1), 3, seed=22), {"method": "lbfgs", "tol": 1e-7, "max_iter": 20000})]
    save("pf_min.npz", pfm)
    ps = []
    for name, kw, shape in [("walls", {"grid": [12, 10, 1], "nfluid": 3, "solid": walls.ravel()}, (12, 10, 1)),
                            ("block", {"grid": [9, 8, 5], "solid": solid.ravel()}, (9, 8, 5))]:
        nf = kw.get("nfluid", 1)
        x = pf_simplex(shape, nf, seed=1) if nf > 1 else pf_noise(shape, seed=1)
        ref = Reference(params_from("pf", kw), x)
        k, kp, nv, sa = ref.pf_internals()
        ps.append({"name": name, "params": json.dumps({a: tolist(b) for a, b in kw.items()}), "x0": x,
                   "kappa": k, "kappaP": kp, "node_vol": nv, "surface_area": sa})
    save("pf_setup.npz", ps)


def gen_bah():
    s2 = np.sqrt(2.0)
    x2 = np.array([-1, 0, 1, 0, -s2, 0, 0, s2, 0, 1, 0, 1.0])
    tri2 = [[0, 1, 2], [1, 3, 2]]
    bah = [eg_case("two_triangles", "bah", {"triangulation": tri2, "rigidity": [100, 1]}, x2,
                   x2 + Rng(8).normal(12) * 0.2)]
    flat, tris, pert = sheet(6, seed=6)
    bah.append(eg_case("sheet6", "bah", {"triangulation": tris, "rigidity": [1, 0.01]}, flat, pert))
    flat8, tris8, pert8 = sheet(8, seed=9)
    bah.append(eg_case("sheet8_thickness_force_wall_fixed", "bah",
                       {"triangulation": tris8, "thickness": 0.1, "modulus": 2.0, "force": [0, 0, -0.01],
                        "wall": True, "wall_adhesion": True, "wall_params": [1e-3, 0.5]},
                       flat8, pert8 - 0.05, fixed=list(range(9))))
    save("bah_eg.npz", bah)
    bs = []
    for name, kw, x in [("sheet6", {"triangulation": tris, "rigidity": [1, 0.01]}, flat),
                        ("sheet8_thick", {"triangulation": tris8, "thickness": 0.1}, flat8)]:
        ref = Reference(params_from("bah", kw), x)
        b, bp, h, hp = ref.bah_elements()
        bs.append({"name": name, "params": json.dumps({a: tolist(v) for a, v in kw.items()}), "x0": x,
                   "bars": b, "bar_par": bp, "hinges": h, "hinge_par": hp})
    save("bah_setup.npz", bs)
    bm = []
    for t0 in [1e-6, np.pi / 2, np.pi, 3 * np.pi / 2, 2 * np.pi - 1e-6]:
        bm.append(min_case(f"hinge_theta0_{t0:.6f}", "bah",
                           {"triangulation": tri2, "rigidity": [100, 1], "theta0": [t0]}, x2,
                           {"method": "lbfgs"}))
    bm.append(min_case("sheet6_relax", "bah", {"triangulation": tris, "rigidity": [1, 0.01]}, flat,
                       {"method": "lbfgs", "tol": 1e-7}, coords=pert))
    save("bah_min.npz", bm)


def gen_pfu():
    """PhaseFieldUnstructured: every element type, both fixed-volume forms,
    all four density constraints (soft with three and four fluids), at
    points away from the initial state (so the volume penalty acts)."""
    solid = np.zeros((9, 8, 5), np.uint8)
    solid[3:5, 2:4, 1:3] = 1
    solid[:, 0, :] = 1
    walls = np.zeros((12, 10, 1), np.uint8)
    walls[:, 0, :] = 1
    ca = Rng(14).uniform(solid.size) * 120 + 30

    def case(name, kw, x0, seed, fixed=None):
        x = np.asarray(x0, float) + 0.05 * Rng(seed + 50).normal(len(x0))
        return eg_case(name, "pfu", kw, x0, x=x, fixed=fixed, seed=seed)

    pfu = [case("binary_3d", {"grid": [6, 5, 4]}, pf_noise((6, 5, 4), seed=12, amp=0.5), 12),
           case("binary_solid_contact_force_volume",
                {"grid": [9, 8, 5], "solid": solid.ravel(), "contact_angle": ca, "force": [0.1, -0.3, 0.2],
                 "pressure": [0.4], "volume_fixed": True, "vol_const": 0.5},
                pf_noise((9, 8, 5), seed=14, amp=0.9), 14, fixed=[3, 50, 51]),
           case("binary_2d_target_volume_res2",
                {"grid": [10, 8, 1], "resolution": 2.0, "volume_fixed": True, "volume": [120.0],
                 "vol_const": 0.2, "confinement": [1.5]}, pf_noise((10, 8, 1), seed=15, amp=0.9), 15)]
    for dens in ["hard", "soft", "none", "fixed"]:
        pfu.append(case(f"ternary_{dens}",
                        {"grid": [12, 10, 1], "nfluid": 3, "solid": walls.ravel(), "volume_fixed": True,
                         "density_constraint": dens, "surface_tension": [1.0, 0.8, 1.2],
                         "pressure": [0, 0.3, 0], "force": [[0, -1, 0], [0.2, 0, 0], [0, 0, 0]],
                         "confinement": [0, 1.0, 0]}, pf_simplex((12, 10, 1), 3, seed=16), 16))
    for dens in ["soft", "fixed"]:
        pfu.append(case(f"four_fluids_{dens}",
                        {"grid": [5, 4, 3], "nfluid": 4, "density_constraint": dens,
                         "solid": solid[:5, :4, :3].ravel(), "pressure": [0.1, 0, 0.2, 0.3]},
                        pf_simplex((5, 4, 3), 4, seed=17), 17))
    pfu.append(case("binary_fluids_fixfluid_pressure",
                    {"grid": [6, 5, 3], "nfluid": 2, "fix_fluid": [1, 0], "pressure": [0.5, 0.25]},
                    pf_simplex((6, 5, 3), 2, seed=18), 18, fixed=[4, 9]))
    save("pfu_eg.npz", pfu)
    pfum = [min_case("binary_8cubed", "pfu", {"grid": [8, 8, 8]}, pf_noise((8, 8, 8), seed=31),
                     {"method": "lbfgs", "m": 10, "tol": 1e-7}),
            min_case("binary_drop_volume_16", "pfu", {"grid": [16, 16, 1], "volume_fixed": True, "vol_const": 0.1},
                     pfu_drop(16), {"method": "lbfgs", "tol": 1e-7, "max_iter": 20000}),
            min_case("ternary_fixed_walls", "pfu",
                     {"grid": [12, 10, 1], "nfluid": 3, "solid": walls.ravel(), "density_constraint": "fixed"},
                     pf_simplex((12, 10, 1), 3, seed=33), {"method": "lbfgs", "tol": 1e-7, "max_iter": 20000})]
    save("pfu_min.npz", pfum)


def gen_anneal():
    """Anneal (src/minimisers/Anneal.cpp) on each potential kind: cooling by
    rate and by a tabulated schedule, stopping on max_iter and on
    max_rejections."""
    flat, tris, pert = sheet(4, seed=71)
    cases = [
        ("lj13_maxiter", "lj", {}, lj_cluster(13, seed=5),
         {"temp_init": 0.5, "displacement": 0.02, "max_iter": 3000, "seed": 11}),
        ("lj13_max_rejections", "lj", {}, lj_cluster(13, seed=5),
         {"temp_init": 0.1, "displacement": 0.05, "max_rejections": 50, "seed": 12}),
        ("lj38_cooling_rate", "lj", {}, lj_cluster(38, seed=2),
         {"temp_init": 2.0, "displacement": 0.01, "cooling_rate": 0.01, "max_iter": 2000, "seed": 13}),
        ("lj13_schedule", "lj", {}, lj_cluster(13, seed=5),
         {"temp_init": 1.0, "displacement": 0.02, "max_iter": 500, "seed": 14,
          "temp_schedule": np.linspace(1, 0.001, 300).tolist()}),
        ("pf_binary_6cubed", "pf", {"grid": [6, 6, 6]}, pf_noise((6, 6, 6), seed=3),
         {"temp_init": 0.01, "displacement": 0.01, "max_iter": 500, "seed": 15}),
        ("pfu_ternary", "pfu", {"grid": [6, 5, 1], "nfluid": 3}, pf_simplex((6, 5, 1), 3, seed=4),
         {"temp_init": 0.05, "displacement": 0.01, "max_iter": 400, "seed": 16}),
        ("bah_sheet4", "bah", {"triangulation": tris, "rigidity": [1, 0.01]}, pert,
         {"temp_init": 1e-3, "displacement": 1e-3, "max_iter": 800, "seed": 17}),
    ]
    out = []
    for name, kind, kw, x0, akw in cases:
        mkw = dict(akw, method="anneal")
        out.append(min_case(name, kind, kw, x0, mkw))
    save("anneal_min.npz", out)


def pfu_drop(n):
    """A binary disc of radius 5 on an n x n grid (tanh profile)."""
    X, Y = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    d = np.sqrt((X - (n - 1) / 2) ** 2 + (Y - (n - 1) / 2) ** 2)
    return np.tanh((5 - d) / np.sqrt(2)).ravel()


if __name__ == "__main__":
    main(sys.argv[1:])
