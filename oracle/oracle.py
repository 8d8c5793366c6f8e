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


class orc_fixed_body(C.Structure):
    _fields_ = [("type", C.c_int), ("model", C.c_float * 16), ("radius", C.c_float), ("up", C.c_float * 3)]


class orc_scene(C.Structure):
    _fields_ = [("drag_w", C.c_void_p), ("drag_off", C.c_void_p), ("target", C.c_float * 3), ("nfixed", C.c_int),
                ("fixed", C.POINTER(orc_fixed_body)), ("mu_t", C.c_float), ("mu_n", C.c_float),
                ("XT", C.c_void_p)]


class RefFixedSpec(C.Structure):
    _fields_ = [("type", C.c_int), ("pos", C.c_float * 3), ("rot", C.c_float * 3), ("scale", C.c_float * 3)]


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
        h.orc_simulate_scene.restype = C.c_int
        h.orc_simulate_scene.argtypes = [C.c_int, C.c_int, _F32, _F32, _F32, _U32, _F32, _F32, C.c_void_p,
                                         C.POINTER(orc_params), C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                         C.POINTER(orc_scene)]
        h.orc_runner_create.restype = C.c_void_p
        h.orc_runner_create.argtypes = [C.c_int, C.c_int, _F32, _F32, _F32, _U32, _F32, _F32, C.c_void_p,
                                        C.POINTER(orc_params), C.c_int, C.c_int]
        h.orc_runner_run.restype = C.c_int
        h.orc_runner_run.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        h.orc_runner_state.restype = C.c_int
        h.orc_runner_state.argtypes = [C.c_void_p, _F32, _F32]
        h.orc_runner_destroy.restype = None
        h.orc_runner_destroy.argtypes = [C.c_void_p]
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
        h.orc_ccd_query.restype = C.c_float
        h.orc_ccd_query.argtypes = [C.c_int, _U32, _F32, _F32, _F32]
        h.orc_ccd_detect.restype = C.c_int
        h.orc_ccd_detect.argtypes = [C.c_int, C.c_int, _U32, _I32, _F32, _F32, _F32, _F32, _I64]
        h.orc_ccd_response.restype = None
        h.orc_ccd_response.argtypes = [C.c_int, _F32, _F32, _F32, _F32, _F32]
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
        h.ref_simulate_scene.restype = C.c_int
        h.ref_simulate_scene.argtypes = [C.c_int, C.c_int, _F32, _F32, _F32, _U32, _F32, _F32, C.c_void_p,
                                         C.c_float, C.c_float, C.c_int, C.c_float, C.c_float, C.c_int, C.c_int,
                                         C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int,
                                         C.POINTER(RefFixedSpec), C.c_float, C.c_float, C.c_void_p]
        h.ref_fixed_frame.restype = None
        h.ref_fixed_frame.argtypes = [C.c_int, _F32, _F32, _F32, _F32, _F32]
        h.ref_rotation.restype = None
        h.ref_rotation.argtypes = [_F32, _F32]
        h.ref_ccd_query.restype = C.c_float
        h.ref_ccd_query.argtypes = [C.c_int, _U32, _F32, _F32, _F32]
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


class Runner:
    """A persistent oracle simulation (set-up once, then timed steps)."""

    def __init__(self, body, params, precision: int = 32, nthreads: int = 0, X=None, V=None):
        self._h = _load_oracle()
        X0, tets, mass, mu, dbc = _arr(body)
        self._keep = (X0, tets, mass, mu, dbc)
        self.nv, self.nt = len(mass), len(mu)
        Xs = np.array(X0 if X is None else np.asarray(X, np.float32).reshape(-1), dtype=np.float32)
        Vs = np.zeros_like(Xs) if V is None else np.array(np.asarray(V, np.float32).reshape(-1), dtype=np.float32)
        p = _params(params)
        self._r = self._h.orc_runner_create(self.nv, self.nt, X0, Xs, Vs, tets, mass, mu,
                                            None if dbc is None else dbc.ctypes.data, C.byref(p), precision,
                                            nthreads)
        if not self._r:
            raise RuntimeError("orc_runner_create failed")

    def run(self, nsteps: int, num_iterations: int = 0) -> float:
        """Runs nsteps steps; returns their wall time in seconds."""
        secs = C.c_double(0.0)
        if self._h.orc_runner_run(self._r, nsteps, num_iterations, None, C.addressof(secs)) != 0:
            raise RuntimeError("orc_runner_run failed")
        return secs.value

    def state(self):
        X = np.empty(3 * self.nv, np.float32)
        V = np.empty(3 * self.nv, np.float32)
        self._h.orc_runner_state(self._r, X, V)
        return X.reshape(-1, 3), V.reshape(-1, 3)

    def close(self):
        if self._r:
            self._h.orc_runner_destroy(self._r)
            self._r = None

    def __del__(self):
        self.close()


def _params(params):
    return orc_params(params.dt, params.gravity, params.num_iterations, params.tol, params.rho,
                      params.positional_weight, int(params.solver), 0)


def simulate_scene(body, params, nsteps: int, precision: int = 64, drag_w=None, drag_off=None,
                   target=(0.0, 0.0, 0.0), fixed=(), mu_t: float = 0.5, mu_n: float = 0.5, X=None, V=None, XT=None,
                   nthreads: int = 0):
    """Oracle run with drag and fixed rigid bodies; returns (X, V, XTilde,
    iterations per step).  fixed: objects with type, model (4x4, glm
    column-major), radius and up."""
    h = _load_oracle()
    X0, tets, mass, mu, dbc = _arr(body)
    Xs = np.array(X0 if X is None else np.asarray(X, np.float32).reshape(-1), dtype=np.float32)
    Vs = np.zeros_like(Xs) if V is None else np.array(np.asarray(V, np.float32).reshape(-1), dtype=np.float32)
    XTs = np.array(Xs if XT is None else np.asarray(XT, np.float32).reshape(-1), dtype=np.float32)
    sc = orc_scene()
    keep = []
    if drag_w is not None:
        w = np.ascontiguousarray(drag_w, dtype=np.float32).reshape(-1)
        o = np.ascontiguousarray(drag_off, dtype=np.float32).reshape(-1)
        keep += [w, o]
        sc.drag_w, sc.drag_off = w.ctypes.data, o.ctypes.data
    for d in range(3):
        sc.target[d] = float(target[d])
    fb = (orc_fixed_body * max(1, len(fixed)))()
    for j, f in enumerate(fixed):
        fb[j].type = int(f.type)
        m = np.ascontiguousarray(f.model, dtype=np.float32).reshape(16)
        for k in range(16):
            fb[j].model[k] = float(m[k])
        fb[j].radius = float(f.radius)
        for k in range(3):
            fb[j].up[k] = float(f.up[k])
    sc.nfixed, sc.fixed = len(fixed), fb
    sc.mu_t, sc.mu_n = mu_t, mu_n
    sc.XT = XTs.ctypes.data
    iters = np.zeros(max(nsteps, 1), dtype=np.int32)
    p = _params(params)
    st = h.orc_simulate_scene(len(mass), len(mu), X0, Xs, Vs, tets, mass, mu,
                              None if dbc is None else dbc.ctypes.data, C.byref(p), precision, nsteps, nthreads,
                              iters.ctypes.data, None, C.byref(sc))
    if st != 0:
        raise RuntimeError(f"orc_simulate_scene failed ({st})")
    return Xs.reshape(-1, 3), Vs.reshape(-1, 3), XTs.reshape(-1, 3), iters[:nsteps]


def drag_select(X, dbc, select_v: int, control_mag: float = 10.0, radius_sq: float = 0.002, offsets=None):
    """The reference's drag selection (Control_Kernel, simulationContext.cu:
    201-218) in float32: every free vertex gets its offset from the grabbed
    vertex, and the weight control_mag when the squared distance is below
    radius_sq (compared in double, as the macro is a double literal).
    Returns (weights, offsets); pinned vertices keep `offsets`' rows."""
    X = np.asarray(X, np.float32).reshape(-1, 3)
    nv = X.shape[0]
    off = np.zeros((nv, 3), np.float32) if offsets is None else np.array(offsets, np.float32).reshape(nv, 3)
    w = np.zeros(nv, np.float32)
    if select_v < 0:
        return w, off
    free = np.ones(nv, bool) if dbc is None else (np.asarray(dbc) == 0)
    d = (X - X[select_v]).astype(np.float32)
    off[free] = d[free]
    dist2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]).astype(np.float32) + d[:, 2] * d[:, 2]
    w[free & (dist2.astype(np.float64) < radius_sq)] = np.float32(control_mag)
    return w, off


def reference_simulate_scene(body, params, nsteps: int, select_v: int = -1, reselect: bool = False, target=None,
                             fixed_specs=(), mu_t: float = 0.5, mu_n: float = 0.5, X=None, V=None):
    """The reference's own PD, drag and fixed-body kernels on the CPU
    (oracle/_ref).  fixed_specs: (type, pos, rot_deg, scale) as a scene file
    gives them (sphere radius = scale[0]).  Returns (X, V, XTilde, iters)."""
    h = _load_ref()
    X0, tets, mass, mu, dbc = _arr(body)
    Xs = np.array(X0 if X is None else np.asarray(X, np.float32).reshape(-1), dtype=np.float32)
    Vs = np.zeros_like(Xs) if V is None else np.array(np.asarray(V, np.float32).reshape(-1), dtype=np.float32)
    XTs = np.zeros_like(Xs)
    specs = (RefFixedSpec * max(1, len(fixed_specs)))()
    for j, (t, pos, rot, scale) in enumerate(fixed_specs):
        specs[j].type = int(t)
        for k in range(3):
            specs[j].pos[k], specs[j].rot[k], specs[j].scale[k] = float(pos[k]), float(rot[k]), float(scale[k])
    tgt = None if target is None else np.ascontiguousarray(target, dtype=np.float32)
    iters = np.zeros(max(nsteps, 1), dtype=np.int32)
    st = h.ref_simulate_scene(len(mass), len(mu), X0, Xs, Vs, tets, mass, mu,
                              None if dbc is None else dbc.ctypes.data, params.dt, params.gravity,
                              params.num_iterations, params.tol, params.rho, int(params.solver), nsteps,
                              iters.ctypes.data, int(select_v), int(bool(reselect)),
                              None if tgt is None else tgt.ctypes.data, len(fixed_specs), specs, mu_t, mu_n,
                              XTs.ctypes.data)
    if st != 0:
        raise RuntimeError(f"ref_simulate_scene failed ({st})")
    return Xs.reshape(-1, 3), Vs.reshape(-1, 3), XTs.reshape(-1, 3), iters[:nsteps]


def reference_fixed_frame(type_: int, pos, rot, scale):
    """The reference's model matrix (4x4, model[c][r]) and plane normal of one body."""
    h = _load_ref()
    model = np.zeros(16, np.float32)
    up = np.zeros(3, np.float32)
    h.ref_fixed_frame(int(type_), np.asarray(pos, np.float32), np.asarray(rot, np.float32),
                      np.asarray(scale, np.float32), model, up)
    return model.reshape(4, 4), up


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


# ------------------------------------------------------- continuous collision
def _f32(a, n=None):
    a = np.ascontiguousarray(a, dtype=np.float32).reshape(-1)
    return a


def ccd_query(face: bool, ids, X, XT):
    """Contact time and normal of one query (face: vertex ids[0] against face
    ids[1:4]; else edge ids[0:2] against edge ids[2:4]), float, restating the
    reference's ccdCollisionTest (intersections.cu:286-334)."""
    n = np.zeros(3, np.float32)
    t = _load_oracle().orc_ccd_query(1 if face else 0, np.ascontiguousarray(ids, np.uint32), _f32(X), _f32(XT), n)
    return float(t), n


def reference_ccd_query(face: bool, ids, X, XT):
    """The same query evaluated by the reference's own code (oracle/_ref)."""
    n = np.zeros(3, np.float32)
    t = _load_ref().ref_ccd_query(1 if face else 0, np.ascontiguousarray(ids, np.uint32), _f32(X), _f32(XT), n)
    return float(t), n


def ccd_detect(tris, tri_body, X, XT):
    """Collision detection between bodies (the reference's DetectCollision
    with ignoreSelfCollision): returns (tI [nv], normals [nv, 3], stats)
    where stats = (candidate pairs, vertices with a face contact, vertices
    marked)."""
    X = _f32(X)
    nv = X.size // 3
    tris = np.ascontiguousarray(tris, np.uint32).reshape(-1)
    body = np.ascontiguousarray(tri_body, np.int32)
    tI = np.empty(nv, np.float32)
    nrm = np.empty(3 * nv, np.float32)
    stats = np.zeros(3, np.int64)
    _load_oracle().orc_ccd_detect(nv, tris.size // 3, tris, body, X, _f32(XT), tI, nrm, stats)
    return tI, nrm.reshape(nv, 3), tuple(int(v) for v in stats)


def ccd_response(tI, normals, X, XT, V):
    """CCDKernel (collisionUtil.cu:50-70) on copies of X and V; returns them."""
    X = _f32(X).copy()
    V = _f32(V).copy()
    _load_oracle().orc_ccd_response(tI.size, np.ascontiguousarray(tI, np.float32), _f32(normals), X, _f32(XT), V)
    return X.reshape(-1, 3), V.reshape(-1, 3)
