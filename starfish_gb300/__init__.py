"""starfish_gb300: GB300 (sm_103a) implementation of Starfish's ES-PIC/DSMC hot path.

The compute lives in libstarfish_gpu.so (C ABI in include/starfish_gpu.h);
``plugin`` holds the host-side classes that mirror the reference's
KineticMaterial / PoissonSolver / DSMC / MCC plugin surface.
"""
from . import abi  # noqa: F401

__all__ = ["abi", "plugin", "workloads", "build"]
