"""ctypes wrapper of ``baseline/_build/librefgpu.so``: the reference's GPU PD
step (PdSolver::SolverStep + Update, src/simulation/solver/projective/
pdSolver.cu:141-232) restated with the same kernels' structure and cuSOLVER's
sparse Cholesky, used by bench.py and the GPU tests as a timed baseline.

It is not part of the engine and the engine never calls it.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_build" / "librefgpu.so"
_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is not built (run __graft_entry__.build())")
        L = C.CDLL(str(LIB_PATH))
        L.rg_last_error.restype = C.c_char_p
        L.rg_create.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                C.c_float, C.c_float, C.c_int, C.c_float, C.c_float, C.c_float, C.c_int,
                                C.POINTER(C.c_void_p)]
        L.rg_step.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_longlong)]
        L.rg_upload.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.rg_read.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.rg_system_nnz.argtypes = [C.c_void_p]
        L.rg_system_nnz.restype = C.c_longlong
        L.rg_destroy.argtypes = [C.c_void_p]
        L.rg_destroy.restype = None
        _lib = L
    return _lib


def _check(rc: int, what: str) -> None:
    if rc != 0:
        raise RuntimeError(f"{what}: {lib().rg_last_error().decode()}")


class ReferenceGpuPath:
    """One body on the restated reference path.  ``params`` is a
    ``pdgb.engine.SolverParams`` (solver 0 = Jacobi + Chebyshev, else the
    cuSOLVER Cholesky branch)."""

    def __init__(self, body, params):
        L = lib()
        self.nv, self.nt = body.num_verts, body.num_tets
        X = np.ascontiguousarray(body.X, dtype=np.float32)
        T = np.ascontiguousarray(body.tets, dtype=np.uint32)
        m = np.ascontiguousarray(body.mass, dtype=np.float32)
        w = np.ascontiguousarray(body.mu, dtype=np.float32)
        d = (np.zeros(self.nv, np.float32) if body.dbc is None
             else np.ascontiguousarray(body.dbc, dtype=np.float32))
        self._X0 = X
        h = C.c_void_p()
        _check(L.rg_create(self.nv, self.nt, X.ctypes.data, T.ctypes.data, m.ctypes.data, w.ctypes.data,
                           d.ctypes.data, params.dt, params.gravity, params.num_iterations, params.tol,
                           params.rho, params.positional_weight, 0 if params.solver == 0 else 1, C.byref(h)),
               "rg_create")
        self.h = h

    def step(self, nsteps: int = 1) -> tuple[float, int]:
        """Runs nsteps steps; returns (milliseconds between CUDA events on the
        default stream, local/global iterations run)."""
        ms, it = C.c_float(), C.c_longlong()
        _check(lib().rg_step(self.h, nsteps, C.byref(ms), C.byref(it)), "rg_step")
        return float(ms.value), int(it.value)

    def reset(self) -> None:
        _check(lib().rg_upload(self.h, self._X0.ctypes.data, None), "rg_upload")

    def state(self) -> tuple[np.ndarray, np.ndarray]:
        X = np.empty((self.nv, 3), np.float32)
        V = np.empty((self.nv, 3), np.float32)
        _check(lib().rg_read(self.h, X.ctypes.data, V.ctypes.data), "rg_read")
        return X, V

    def system_nnz(self) -> int:
        return int(lib().rg_system_nnz(self.h))

    def close(self) -> None:
        if self.h:
            lib().rg_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
