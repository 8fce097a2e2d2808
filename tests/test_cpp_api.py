"""The source-compatible C++ API (include/minim/minim.h), driven by a C++
program that restates the reference's unit tests (tests/cpp/api_test.cpp).
Host potentials run anywhere; the built-in potentials need the GPU."""
import os
import subprocess

import pytest

from minim_gb300 import runtime

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def api_test(tmp_path_factory):
    runtime.load()  # builds the library if needed
    exe = str(tmp_path_factory.mktemp("cpp") / "api_test")
    lib = os.path.join(REPO, "minim_gb300")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + os.path.join(REPO, "include"),
                    "-I" + os.path.join(REPO, "include", "minim"),
                    os.path.join(REPO, "tests", "cpp", "api_test.cpp"), "-L" + lib, "-lminim_gb300",
                    "-Wl,-rpath," + lib, "-o", exe], check=True)
    return exe


def test_cpp_api_host_potentials(api_test):
    r = subprocess.run([api_test, "host"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr


@pytest.mark.gpu
def test_cpp_api_device_potentials(api_test):
    r = subprocess.run([api_test, "all"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
