"""ctypes binding of the CPU oracle — TEST INFRASTRUCTURE ONLY.

Loaded by tests/, __graft_entry__.smoke() and the CPU-baseline leg of
bench.py, and nowhere else.  ``liboracle.so`` is the project's CPU
restatement of the reference's PD step (pd_oracle.h); ``_ref/libref_pd.so``
(present only where the reference sources were available to build it) runs
the reference's own PD kernels on the CPU.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_LIB = HERE / "_build" / "liboracle.so"
REF_LIB = HERE / "_ref" / "libref_pd.so"


class orc_params(C.Structure):
    _fields_ = [("dt", C.c_float), ("gravity", C.c_float), ("num_iterations", C.c_int), ("tol", C.c_float),
                ("rho", C.c_float), ("positional_weight", C.c_float), ("solver", C.c_int), ("reserved", C.c_int)]


_orc = None
_ref = None

_F32 = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_F64 = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_U32 = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_I32 = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_I64 = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")


def _load_oracle():
    global _orc
    if _orc is None:
        if not ORACLE_LIB.exists():
            raise RuntimeError(f"oracle not built: {ORACLE_LIB}")
        h = C.CDLL(str(ORACLE_LIB))
        h.orc_simulate.restype = C.c_int
        h.orc_simulate.argtypes = [C.c_int, C.c_int, _F32, _F32, _F32, _U32, _F32, _F32, C.c_void_p,
                                   C.POINTER(orc_params), C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        h.orc_rotations.restype = None
        h.orc_rotations.argtypes = [C.c_int, _F64, _F64, C.c_int]
        h.orc_local_rhs.restype = C.c_int
        h.orc_local_rhs.argtypes = [C.c_int, C.c_int, _F32, _U32, _F32, _F32, C.c_void_p, C.c_float, C.c_float,
                                    _F64, _F64, C.c_int, _F64]
        h.orc_system_csr.restype = C.c_long
        h.orc_system_csr.argtypes = [C.c_int, C.c_int, _F32, _U32, _F32, _F32, C.c_void_p, C.c_float, C.c_float,
                                     C.c_void_p, C.c_void_p, C.c_void_p]
        h.orc_solve3.restype = C.c_int
        h.orc_solve3.argtypes = [C.c_int, C.c_int, _F32, _U32, _F32, _F32, C.c_void_p, C.c_float, C.c_float,
                                 _F64, _F64]
        _orc = h
    return _orc


def reference_available() -> bool:
    return REF_LIB.exists()


def _load_ref():
    global _ref
    if _ref is None:
        if not REF_LIB.exists():
            raise RuntimeError(f"reference harness not built: {REF_LIB}")
        h = C.CDLL(str(REF_LIB))
        h.ref_simulate.restype = C.c_int
        h.ref_simulate.argtypes = [C.c_int, C.c_int, _F32, _F32, _F32, _U32, _F32, _F32, C.c_void_p, C.c_float,
                                   C.c_float, C.c_int, C.c_float, C.c_float, C.c_int, C.c_int, C.c_void_p]
        h.ref_rotation.restype = None
        h.ref_rotation.argtypes = [_F32, _F32]
        _ref = h
    return _ref


def _arr(body):
    X0 = np.ascontiguousarray(body.X, dtype=np.float32).reshape(-1)
    tets = np.ascontiguousarray(body.tets, dtype=np.uint32).reshape(-1)
    mass = np.ascontiguousarray(body.mass, dtype=np.float32)
    mu = np.ascontiguousarray(body.mu, dtype=np.float32)
    dbc = None if body.dbc is None else np.ascontiguousarray(body.dbc, dtype=np.float32)
    return X0, tets, mass, mu, dbc


def simulate(body, params, nsteps: int, precision: int = 64, nthreads: int = 0, X=None, V=None,
             timing: dict | None = None):
    """Runs the oracle; returns (X, V, iterations per step).  If `timing` is a
    dict it receives "step_seconds" (set-up excluded)."""
    h = _load_oracle()
    X0, tets, mass, mu, dbc = _arr(body)
    Xs = np.array(X0 if X is None else np.asarray(X, np.float32).reshape(-1), dtype=np.float32)
    Vs = np.zeros_like(Xs) if V is None else np.array(np.asarray(V, np.float32).reshape(-1), dtype=np.float32)
    p = orc_params(params.dt, params.gravity, params.num_iterations, params.tol, params.rho,
                   params.positional_weight, int(params.solver), 0)
    iters = np.zeros(max(nsteps, 1), dtype=np.int32)
    secs = C.c_double(0.0)
    st = h.orc_simulate(len(mass), len(mu), X0, Xs, Vs, tets, mass, mu,
                        None if dbc is None else dbc.ctypes.data, C.byref(p), precision, nsteps, nthreads,
                        iters.ctypes.data, C.addressof(secs))
    if st != 0:
        raise RuntimeError(f"orc_simulate failed ({st})")
    if timing is not None:
        timing["step_seconds"] = secs.value
    return Xs.reshape(-1, 3), Vs.reshape(-1, 3), iters[:nsteps]


def reference_simulate(body, params, nsteps: int, X=None, V=None):
    """Runs the reference's own PD kernels on the CPU (oracle/_ref)."""
    h = _load_ref()
    X0, tets, mass, mu, dbc = _arr(body)
    Xs = np.array(X0 if X is None else np.asarray(X, np.float32).reshape(-1), dtype=np.float32)
    Vs = np.zeros_like(Xs) if V is None else np.array(np.asarray(V, np.float32).reshape(-1), dtype=np.float32)
    iters = np.zeros(max(nsteps, 1), dtype=np.int32)
    st = h.ref_simulate(len(mass), len(mu), X0, Xs, Vs, tets, mass, mu, None if dbc is None else dbc.ctypes.data,
                        params.dt, params.gravity, params.num_iterations, params.tol, params.rho,
                        int(params.solver), nsteps, iters.ctypes.data)
    if st != 0:
        raise RuntimeError(f"ref_simulate failed ({st})")
    return Xs.reshape(-1, 3), Vs.reshape(-1, 3), iters[:nsteps]


def rotations(F: np.ndarray, precision: int = 64) -> np.ndarray:
    h = _load_oracle()
    F = np.ascontiguousarray(F, dtype=np.float64).reshape(-1, 9)
    R = np.empty_like(F)
    h.orc_rotations(F.shape[0], F.reshape(-1), R.reshape(-1), precision)
    return R.reshape(-1, 3, 3)


def reference_rotation(F: np.ndarray) -> np.ndarray:
    h = _load_ref()
    F = np.ascontiguousarray(F, dtype=np.float32).reshape(-1, 9)
    out = np.empty_like(F)
    for k in range(F.shape[0]):
        r = np.empty(9, np.float32)
        h.ref_rotation(np.ascontiguousarray(F[k]), r)
        out[k] = r
    return out.reshape(-1, 3, 3)


def local_rhs(body, dt: float, q: np.ndarray, s_old: np.ndarray, jacobi_form: bool,
              positional_weight: float = 1e6) -> np.ndarray:
    h = _load_oracle()
    X0, tets, mass, mu, dbc = _arr(body)
    b = np.empty(len(mass) * 3, dtype=np.float64)
    st = h.orc_local_rhs(len(mass), len(mu), X0, tets, mass, mu, None if dbc is None else dbc.ctypes.data, dt,
                         positional_weight, np.ascontiguousarray(q, np.float64).reshape(-1),
                         np.ascontiguousarray(s_old, np.float64).reshape(-1), int(jacobi_form), b)
    if st != 0:
        raise RuntimeError("orc_local_rhs failed")
    return b.reshape(-1, 3)


def system_csr(body, dt: float, positional_weight: float = 1e6):
    import scipy.sparse as sp
    h = _load_oracle()
    X0, tets, mass, mu, dbc = _arr(body)
    d = None if dbc is None else dbc.ctypes.data
    nnz = h.orc_system_csr(len(mass), len(mu), X0, tets, mass, mu, d, dt, positional_weight, None, None, None)
    rp = np.empty(len(mass) + 1, np.int64)
    ci = np.empty(nnz, np.int32)
    cv = np.empty(nnz, np.float64)
    h.orc_system_csr(len(mass), len(mu), X0, tets, mass, mu, d, dt, positional_weight, rp.ctypes.data,
                     ci.ctypes.data, cv.ctypes.data)
    return sp.csr_matrix((cv, ci, rp), shape=(len(mass), len(mass)))


def solve3(body, dt: float, b: np.ndarray, positional_weight: float = 1e6) -> np.ndarray:
    h = _load_oracle()
    X0, tets, mass, mu, dbc = _arr(body)
    x = np.empty(len(mass) * 3, np.float64)
    st = h.orc_solve3(len(mass), len(mu), X0, tets, mass, mu, None if dbc is None else dbc.ctypes.data, dt,
                      positional_weight, np.ascontiguousarray(b, np.float64).reshape(-1), x)
    if st != 0:
        raise RuntimeError("orc_solve3 failed")
    return x.reshape(-1, 3)
