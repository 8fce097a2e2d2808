"""BarAndHinge set-up on the device (minim_gb300/csrc/topology.cu) against
the host builder, which follows the reference's BarAndHinge::init
(src/potentials/BarAndHinge.cpp:16-248): the same bonds and hinges with the
same parameters, the same vertex-disjoint colouring, the same energies, and
the host builder taking over for triangulations the device one leaves."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from minim_gb300 import abi, runtime
from oracle.oracle import Oracle
from tests.workloads import Rng, sheet

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _sorted_rows(el, par):
    order = np.lexsort(el.T[::-1])
    return el[order], par[order]


def _check_colours(a, nvert):
    for key, off in (("bars", a["bar_off"]), ("hinges", a["hinge_off"])):
        el = a[key]
        assert off[0] == 0 and off[-1] == len(el)
        for c in range(len(off) - 1):
            # no vertex in two elements of one colour
            v = np.concatenate([np.unique(r) for r in el[off[c]:off[c + 1]]] + [np.zeros(0, np.int32)])
            assert len(np.unique(v)) == len(v), (key, c)
            assert v.max(initial=-1) < nvert


def _compare_with_host(p, x0, on_device=True):
    inst = runtime.Instance(p, x0)
    a = inst.bah_arrays()
    assert a["on_device"] == on_device
    h_bars, h_bpar, h_hinges, h_hpar = runtime.bah_elements(p, x0)
    nvert = len(x0) // 3
    _check_colours(a, nvert)
    hb, hbp = _sorted_rows(h_bars, h_bpar)
    db, dbp = _sorted_rows(a["bars"], a["bar_par"])
    assert np.array_equal(hb, db)
    assert np.allclose(hbp, dbp, rtol=1e-13, atol=0)
    hh, hhp = _sorted_rows(h_hinges, h_hpar)
    dh, dhp = _sorted_rows(a["hinges"], a["hinge_par"])
    assert np.array_equal(hh, dh)
    assert np.allclose(hhp[:, 0], dhp[:, 0], rtol=1e-13, atol=0)
    assert np.allclose(hhp[:, 1], dhp[:, 1], rtol=0, atol=1e-12)
    return inst, a


@pytest.mark.parametrize("k", [3, 6, 20, 60])
def test_sheet_matches_host(k):
    flat, tris, pert = sheet(k, seed=40 + k)
    p = abi.bar_and_hinge(triangulation=tris, rigidity=(1, 0.01))
    inst, a = _compare_with_host(p, flat)
    nbc, nhc, _ = runtime.bah_colouring(p, flat)
    # the same greedy pass in element order: the host's colour counts
    assert len(a["bar_off"]) - 1 == nbc
    assert len(a["hinge_off"]) - 1 == nhc
    e, g = inst.energy_gradient(pert)
    eo, go = Oracle(p, flat).energy_gradient(pert)
    assert abs(e - eo) <= 1e-12 * abs(eo)
    assert np.max(np.abs(g - go)) <= 1e-12 * np.max(np.abs(go))


def test_thickness_rigidities_and_given_lengths():
    flat, tris, pert = sheet(12, seed=51)
    nb = len(runtime.bah_elements(abi.bar_and_hinge(triangulation=tris, rigidity=(1, 1)), flat)[0])
    th = 0.05 + 0.1 * Rng(52).uniform(len(flat) // 3)
    l0 = 1.0 + 0.01 * Rng(53).uniform(nb)
    p = abi.bar_and_hinge(triangulation=tris, thickness=th, modulus=3.0, poisson_ratio=0.25, length0=l0)
    _compare_with_host(p, flat)


def _octahedron():
    x = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]], float)
    t = [[0, 2, 4], [2, 1, 4], [1, 3, 4], [3, 0, 4], [2, 0, 5], [1, 2, 5], [3, 1, 5], [0, 3, 5]]
    return x.ravel(), np.array(t, np.int32)


def test_closed_surface_and_shared_edges():
    x, t = _octahedron()
    _compare_with_host(abi.bar_and_hinge(triangulation=t, rigidity=(2, 0.3)), x)
    # three triangles on one edge (0-1): every pair of them is a hinge
    x3 = np.array([[0, 0, 0], [1, 0, 0], [0.5, 1, 0], [0.5, -1, 0], [0.5, 0, 1]], float).ravel()
    t3 = np.array([[0, 1, 2], [1, 0, 3], [0, 1, 4]], np.int32)
    _compare_with_host(abi.bar_and_hinge(triangulation=t3, rigidity=(1, 0.1)), x3)


def test_degenerate_triangle_uses_host_builder():
    flat, tris, _ = sheet(5, seed=54)
    tris = np.concatenate([tris, [[3, 3, 7]]]).astype(np.int32)
    _compare_with_host(abi.bar_and_hinge(triangulation=tris, rigidity=(1, 0.01)), flat, on_device=False)


def test_fixed_vertices_recoloured():
    flat, tris, pert = sheet(10, seed=55)
    p = abi.bar_and_hinge(triangulation=tris, rigidity=(1, 0.01))
    fixed = list(range(3 * 10))  # the first row of vertices
    inst = runtime.Instance(p, flat, fixed=fixed)
    a = inst.bah_arrays()
    assert a["on_device"]
    _check_colours(a, len(flat) // 3)
    full = runtime.Instance(p, flat).bah_arrays()
    # the 9 bars inside the fixed row go; every hinge spans two rows and stays
    assert len(a["bars"]) == len(full["bars"]) - 9 and len(a["hinges"]) == len(full["hinges"])
    e, g = inst.energy_gradient(pert)
    eo, go = Oracle(p, flat, fixed=fixed).energy_gradient(pert)
    assert abs(e - eo) <= 1e-12 * abs(eo)
    assert np.max(np.abs(g - go)) <= 1e-12 * np.max(np.abs(go))


def test_set_up_time_large_sheet():
    """A 100k-vertex sheet: instance creation with the device set-up against
    the host one (separate process), reported; both give the same energy."""
    code = (
        "import json, sys, time; sys.path.insert(0, '.');"
        "from minim_gb300 import abi, runtime; from tests.workloads import sheet;"
        "flat, tris, pert = sheet(316, seed=56); p = abi.bar_and_hinge(triangulation=tris, rigidity=(1, 0.01));"
        "f4, t4, _ = sheet(4); w = runtime.Instance(abi.bar_and_hinge(triangulation=t4, rigidity=(1, 1)), f4);"
        "t = time.perf_counter(); i = runtime.Instance(p, flat); dt = time.perf_counter() - t;"
        "print(json.dumps({'ms': dt * 1e3, 'e': i.energy(pert), 'dev': i.bah_arrays()['on_device']}))"
    )
    out = {}
    for env in ("1", "0"):
        r = subprocess.run([sys.executable, "-c", code], cwd=REPO, capture_output=True, text=True, timeout=600,
                           env=dict(os.environ, MINIM_GPU_BAH_DEVICE_SETUP=env))
        assert r.returncode == 0, r.stderr
        out[env] = json.loads(r.stdout.strip().splitlines()[-1])
    print("100k-vertex sheet set-up ms: device %.1f host %.1f" % (out["1"]["ms"], out["0"]["ms"]))
    assert out["1"]["dev"] and not out["0"]["dev"]
    assert abs(out["1"]["e"] - out["0"]["e"]) <= 1e-12 * abs(out["0"]["e"])
