"""Builds the engine library minim_gb300/libminim_gb300.so for sm_103a.

Translation units are compiled in parallel (one per kernel variant plus the
host runtime) and re-used while they are newer than every source they depend
on.  Only nvcc and g++ are needed; no GPU.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libminim_gb300.so")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU = ["engine_lj.cu", "engine_pf.cu", "engine_pf1.cu", "engine_bah.cu", "engine_misc.cu", "noalloc.cu", "stepped.cu", "topology.cu"]
CPP = ["setup.cpp", "capi.cpp"]
API = ["api_core.cpp", "api_minimisers.cpp", "api_potentials.cpp"]  # source-compatible C++ API
HEADERS = ["common.cuh", "potentials.cuh", "ljcells.cuh", "minimiser.cuh", "kernels.cuh", "engine.h", "setup.h"]
API_HEADERS = ["minim.h", "State.h", "Potential.h", "Minimiser.h", "Communicator.h", "minimisers/Lbfgs.h",
               "minimisers/Fire.h", "minimisers/GradDescent.h", "potentials/LjNd.h", "potentials/PhaseField.h",
               "potentials/BarAndHinge.h", "utils/vec.h", "utils/mpi.h", "utils/print.h"]


def _deps():
    return [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(REPO, "include", "minim_gpu.h")]


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    inc = ["-I" + os.path.join(REPO, "include"), "-I" + CSRC]
    # MINIM_GPU_LJ_MINB: minimum resident blocks per SM of the Lennard-Jones
    # batch kernel (its register budget); rebuild with force=True to change it
    defs = ["-DMG_LJ_MINB=" + os.environ["MINIM_GPU_LJ_MINB"]] if os.environ.get("MINIM_GPU_LJ_MINB") else []
    jobs = []
    objs = []
    for f in CU:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + _deps()):
            jobs.append([NVCC] + ARCH + ["-O3", "-lineinfo", "-std=c++20", "-Xcompiler", "-fPIC",
                                         "-Xptxas", "-v"] + defs + inc + ["-c", src, "-o", obj])
    for f in CPP:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + _deps()):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-I" + os.path.join(CUDA, "include")]
                        + inc + ["-c", src, "-o", obj])
    api_deps = [os.path.join(REPO, "include", "minim", h) for h in API_HEADERS] + _deps()
    for f in API:
        src = os.path.join(HERE, "cpp", f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + api_deps):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-I" + os.path.join(REPO, "include"),
                         "-I" + os.path.join(REPO, "include", "minim"), "-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            logs = list(ex.map(_run, jobs))
        with open(os.path.join(BUILD, "ptxas.log"), "w") as fh:
            fh.write("\n".join(logs))
        if verbose:
            print("\n".join(logs))
    if force or jobs or _stale(LIB, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
