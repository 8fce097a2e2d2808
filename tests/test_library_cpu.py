"""The engine library on a machine without a GPU: it loads, exports every
symbol include/minim_gpu.h declares, its host-side set-up matches the
reference fixtures, and compute calls fail loudly (no CPU fallback)."""
import os
import re

import numpy as np
import pytest

from minim_gb300 import abi, runtime
from tests import golden_io as G

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(REPO, "include", "minim_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(minim_gpu_\w+)\s*\(", txt)))


def test_exports_every_declared_symbol(engine):
    decl = declared_symbols()
    assert len(decl) >= 30
    for name in decl:
        assert hasattr(engine, name), name
    assert sorted(runtime.EXPORTS) == decl


def test_abi_version(engine):
    assert engine.minim_gpu_abi_version() == 2


def test_struct_layout_matches_header(tmp_path):
    """The ctypes mirror has the C compiler's layout: sizes and every offset."""
    import ctypes as C
    import subprocess
    structs = {"minim_gpu_lj_params": abi.LjParams, "minim_gpu_pf_params": abi.PfParams,
               "minim_gpu_bah_params": abi.BahParams, "minim_gpu_minimiser_params": abi.MinimiserParams,
               "minim_gpu_result": abi.Result, "minim_gpu_run_stats": abi.RunStats,
               "minim_gpu_server_config": abi.ServerConfig}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "minim_gpu.h"', "int main(void){"]
    for cname, cls in structs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l}
    for cname, cls in structs.items():
        assert got[(cname, "size")] == C.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert got[(cname, f)] == getattr(cls, f).offset, (cname, f)


def test_bah_setup_matches_reference():
    for c in G.load("bah_setup.npz"):
        p = G.params_from("bah", c["params_kw"])
        b, bp, h, hp = runtime.bah_elements(p, c["x0"])
        assert np.array_equal(b, c["bars"]) and np.array_equal(h, c["hinges"])
        assert np.allclose(bp, c["bar_par"], rtol=1e-14) and np.allclose(hp, c["hinge_par"], rtol=1e-14)
        nbc, nhc, ok = runtime.bah_colouring(p, c["x0"])
        assert ok and nbc >= 1 and nhc >= 1


def test_bah_topology_large_sheet_is_fast():
    from tests.workloads import sheet
    import time
    flat, tris, _ = sheet(200, seed=1)  # 40k vertices: the reference's O(T^2) search takes minutes
    t = time.time()
    b, _, h, _ = runtime.bah_elements(abi.bar_and_hinge(triangulation=tris, rigidity=(1, 0.01)), flat)
    assert time.time() - t < 20
    assert len(b) == 3 * 199 * 199 + 2 * 199 and len(h) == len(b) - 4 * 199
    nbc, nhc, ok = runtime.bah_colouring(abi.bar_and_hinge(triangulation=tris, rigidity=(1, 0.01)), flat)
    assert ok and nbc <= 16 and nhc <= 32


def test_pf_setup_matches_reference():
    for c in G.load("pf_setup.npz"):
        p = G.params_from("pf", c["params_kw"])
        s = runtime.pf_setup(p, c["x0"])
        assert np.array_equal(s["kappa"], c["kappa"]) and np.array_equal(s["kappaP"], c["kappaP"])
        assert np.array_equal(s["node_vol"], c["node_vol"]) and np.array_equal(s["surface_area"],
                                                                               c["surface_area"])


def test_pf_kernel_variant():
    x = np.zeros(8 ** 3)
    assert runtime.pf_setup(abi.phase_field([8, 8, 8]), x)["kernel_variant"] == 3
    assert runtime.pf_setup(abi.phase_field([8, 8, 8], pressure=[1.0]), x)["kernel_variant"] == 3
    solid = np.zeros(8 ** 3, np.uint8)
    solid[:64] = 1
    assert runtime.pf_setup(abi.phase_field([8, 8, 8], solid=solid), x)["kernel_variant"] == 1


def test_setup_errors():
    with pytest.raises(runtime.MinimGpuError) as e:
        runtime.pf_setup(abi.phase_field([4, 4, 1]), np.zeros(15))
    assert e.value.code == abi.ERR_INVALID
    with pytest.raises(runtime.MinimGpuError):
        runtime.pf_setup(abi.phase_field([4, 4, 1], nfluid=5), np.zeros(80))
    with pytest.raises(runtime.MinimGpuError):
        runtime.bah_elements(abi.bar_and_hinge(triangulation=[[0, 1, 5]], rigidity=(1, 1)), np.zeros(9))


@pytest.mark.skipif(os.path.exists("/dev/nvidia0"), reason="host has a GPU")
def test_no_gpu_fails_loudly():
    with pytest.raises(runtime.MinimGpuError) as e:
        runtime.Instance(abi.lj(), [0, 0, 0, 2, 0, 0])
    assert e.value.code == abi.ERR_NO_DEVICE


def test_default_minimiser_and_python_mirror_agree():
    """minim_gpu_default_minimiser (the reference's constructor defaults, and
    Anneal's) against abi.minimiser, field by field."""
    import ctypes as C
    lib = runtime.load()
    for method, name in ((abi.LBFGS, "lbfgs"), (abi.FIRE, "fire"), (abi.GD, "gd"), (abi.ANNEAL, "anneal")):
        c = abi.MinimiserParams()
        lib.minim_gpu_default_minimiser(method, C.byref(c))
        py = abi.minimiser(name)
        for f, _ in abi.MinimiserParams._fields_:
            if f == "temp_schedule":
                assert not getattr(c, f) and not getattr(py, f)
                continue
            assert getattr(c, f) == getattr(py, f), (name, f)


def test_pfu_setup_errors():
    """PhaseFieldUnstructured's own argument checks (checkArraySizes, and the
    soft density element's three fluids)."""
    with pytest.raises(runtime.MinimGpuError):
        runtime.pf_setup(abi.phase_field_unstructured([4, 4, 1], nfluid=2, density_constraint="soft"),
                         np.full(32, 0.5))
    with pytest.raises(runtime.MinimGpuError):
        runtime.pf_setup(abi.phase_field_unstructured([4, 4, 1], surface_tension=np.ones(16)), np.zeros(16))
    with pytest.raises(runtime.MinimGpuError):
        runtime.pf_setup(abi.phase_field_unstructured([4, 4, 1], nfluid=3, interface_size=[1.0, 1.0]),
                         np.full(48, 1 / 3))
    info = runtime.pf_setup(abi.phase_field_unstructured([6, 5, 4]), np.zeros(120))
    assert info["kernel_variant"] == 3  # binary, no optional term: the PhaseField fast path
