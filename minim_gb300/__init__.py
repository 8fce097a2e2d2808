"""minim_gb300: GB300-native energy minimisation (LjNd, PhaseField and
BarAndHinge potentials with Lbfgs / Fire / GradDescent), device resident.

``abi`` holds the parameter structs of the C ABI; ``runtime`` binds the
engine library (include/minim_gpu.h) and raises when it or the GPU is absent.
"""
from . import abi  # noqa: F401

__all__ = ["abi", "runtime", "build"]
