"""pdgb — GB300-native projective-dynamics step engine (Python host side).

The compute path is ``_lib/libpdgb.so`` (CUDA kernels for sm_103a behind a C
ABI, declared in include/pdgb.h).  This package binds it with ctypes and
provides the synthetic soft bodies used by tests and benchmarks.
"""
from . import mesh, meshio, scene
from ._native import PdgbError, library_path
from .engine import PdSolver, SolverParams, SolverType, ccd_detect
from .server import PdServer

__all__ = ["mesh", "meshio", "scene", "PdSolver", "PdServer", "SolverParams", "SolverType", "PdgbError", "library_path",
           "ccd_detect"]
