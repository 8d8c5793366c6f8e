"""Python mirror of the reference's PD solver interface over the C ABI.

``PdSolver`` follows the reference's ``PdSolver`` (pdSolver.h:12-44) and
``Solver<float>`` (solver.h:11-28): construct from a system, ``update``
advances one step (prepares on first use), ``set_global_solver`` switches
between Jacobi+Chebyshev and Cholesky, ``reset`` restores the rest shape,
``get_performance_data`` reports timings.  All compute happens in
``libpdgb.so``; this module only moves numpy arrays across the C ABI.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native as N
from .mesh import SoftBody


class SolverType:
    """Mirrors PdSolver::SolverType (pdSolver.h:14-17)."""

    Jacobi = N.PDGB_SOLVER_JACOBI
    CuSolverCholesky = N.PDGB_SOLVER_CHOLESKY
    EigenCholesky = N.PDGB_SOLVER_CHOLESKY
    Cholesky = N.PDGB_SOLVER_CHOLESKY


@dataclass
class SolverParams:
    """Mirrors SolverParams<float> (def.h:82-100) for the fields PD reads."""

    dt: float = 1.0 / 120.0
    gravity: float = 9.8
    num_iterations: int = 10
    tol: float = 0.0
    rho: float = 0.9992
    positional_weight: float = 1e6
    solver: int = SolverType.Jacobi
    refine_steps: int = 0

    def to_c(self) -> N.pdgb_params:
        return N.pdgb_params(self.dt, self.gravity, self.num_iterations, self.tol, self.rho,
                             self.positional_weight, self.solver, self.refine_steps)


def _ptr(a: np.ndarray | None) -> int | None:
    return None if a is None else a.ctypes.data


def _host_desc(body: SoftBody, keep: list) -> N.pdgb_mesh_desc:
    X = np.ascontiguousarray(body.X, dtype=np.float32)
    tets = np.ascontiguousarray(body.tets, dtype=np.uint32)
    mass = np.ascontiguousarray(body.mass, dtype=np.float32)
    mu = np.ascontiguousarray(body.mu, dtype=np.float32)
    dbc = None if body.dbc is None else np.ascontiguousarray(body.dbc, dtype=np.float32)
    V = None if body.V is None else np.ascontiguousarray(body.V, dtype=np.float32)
    keep.extend([X, tets, mass, mu, dbc, V])
    return N.pdgb_mesh_desc(X.shape[0], tets.shape[0], _ptr(X), _ptr(V), _ptr(tets), _ptr(mass), _ptr(mu),
                            _ptr(dbc), N.PDGB_MEM_HOST)


class PdSolver:
    def __init__(self, body: SoftBody | list, params: SolverParams, stream: int | None = None):
        """One body, or a list of independent bodies advanced as one batch."""
        self._lib = N.lib()
        self.params = params
        self.body = body
        keep: list = []
        h = C.c_void_p()
        prm = params.to_c()
        if isinstance(body, (list, tuple)):
            descs = (N.pdgb_mesh_desc * len(body))(*[_host_desc(b, keep) for b in body])
            N.check(self._lib.pdgb_create_batch(len(body), descs, C.byref(prm), stream, C.byref(h)),
                    "pdgb_create_batch")
            self.body_verts = np.cumsum([0] + [b.num_verts for b in body])
            self.num_verts = int(self.body_verts[-1])
            self.num_tets = int(sum(b.num_tets for b in body))
        else:
            desc = _host_desc(body, keep)
            N.check(self._lib.pdgb_create(C.byref(desc), C.byref(prm), stream, C.byref(h)), "pdgb_create")
            self.body_verts = np.array([0, body.num_verts])
            self.num_verts = body.num_verts
            self.num_tets = body.num_tets
        self._h = h

    # -- Solver<float> interface
    def prepare(self) -> None:
        N.check(self._lib.pdgb_prepare(self._h), "pdgb_prepare")

    def update(self, nsteps: int = 1) -> None:
        N.check(self._lib.pdgb_step(self._h, int(nsteps)), "pdgb_step")

    def set_global_solver(self, solver: int) -> None:
        N.check(self._lib.pdgb_set_solver(self._h, int(solver)), "pdgb_set_solver")
        self.params.solver = int(solver)

    def set_params(self, params: SolverParams) -> None:
        prm = params.to_c()
        N.check(self._lib.pdgb_set_params(self._h, C.byref(prm)), "pdgb_set_params")
        self.params = params

    def set_ordering(self, ordering: int) -> None:
        """0 = AMD (default), 1 = geometric nested dissection."""
        N.check(self._lib.pdgb_set_ordering(self._h, int(ordering)), "pdgb_set_ordering")

    def set_rotation(self, mode: int) -> None:
        """0 = quaternion (default, converged), 1 = the reference's 4-sweep SVD."""
        N.check(self._lib.pdgb_set_rotation(self._h, int(mode)), "pdgb_set_rotation")

    def set_local_kernel(self, kind: int) -> None:
        """0 = one CTA per tile (default), 1 = pipelined persistent CTAs."""
        N.check(self._lib.pdgb_set_local_kernel(self._h, int(kind)), "pdgb_set_local_kernel")

    def local_kernel(self) -> int:
        k = C.c_int()
        N.check(self._lib.pdgb_get_local_kernel(self._h, C.byref(k)), "pdgb_get_local_kernel")
        return k.value

    def reset(self) -> None:
        N.check(self._lib.pdgb_reset(self._h), "pdgb_reset")

    def synchronize(self) -> None:
        N.check(self._lib.pdgb_synchronize(self._h), "pdgb_synchronize")

    def step_status(self) -> int:
        """PDGB_OK, or PDGB_ERR_NONFINITE once a step since the state was last
        set ended with a non-finite position or velocity (waits for the GPU)."""
        st = int(self._lib.pdgb_last_step_status(self._h))
        if st not in (N.PDGB_OK, N.PDGB_ERR_NONFINITE):
            N.check(st, "pdgb_last_step_status")
        return st

    def check_finite(self) -> None:
        """Raises PdgbError(PDGB_ERR_NONFINITE) if the iteration left the finite range."""
        N.check(self._lib.pdgb_last_step_status(self._h), "pdgb_last_step_status")

    # -- state
    def upload_state(self, X: np.ndarray, V: np.ndarray | None = None) -> None:
        X = np.ascontiguousarray(X, dtype=np.float32)
        V = None if V is None else np.ascontiguousarray(V, dtype=np.float32)
        N.check(self._lib.pdgb_upload_state(self._h, _ptr(X), _ptr(V), N.PDGB_MEM_HOST), "pdgb_upload_state")
        self.synchronize()

    def download_state(self) -> tuple[np.ndarray, np.ndarray]:
        X = np.empty((self.num_verts, 3), dtype=np.float32)
        V = np.empty((self.num_verts, 3), dtype=np.float32)
        N.check(self._lib.pdgb_download_state(self._h, _ptr(X), _ptr(V), N.PDGB_MEM_HOST), "pdgb_download_state")
        return X, V

    def download_xtilde(self) -> np.ndarray:
        """XTilde: positions after the fixed-body correction (= X without bodies)."""
        XT = np.empty((self.num_verts, 3), dtype=np.float32)
        N.check(self._lib.pdgb_download_xtilde(self._h, _ptr(XT), N.PDGB_MEM_HOST), "pdgb_download_xtilde")
        return XT

    def set_collision_surface(self, tris: np.ndarray, tri_body: np.ndarray | None = None) -> None:
        """Surface triangles (caller vertex ids) for continuous collision
        between bodies; tri_body: body of each triangle (None: from the
        engine's body ranges)."""
        t = np.ascontiguousarray(tris, dtype=np.uint32).reshape(-1, 3)
        b = None if tri_body is None else np.ascontiguousarray(tri_body, dtype=np.int32)
        N.check(self._lib.pdgb_set_collision_surface(self._h, t.ctypes.data, None if b is None else b.ctypes.data,
                                                     t.shape[0]), "pdgb_set_collision_surface")

    def enable_collision(self, on: bool = True) -> None:
        N.check(self._lib.pdgb_enable_collision(self._h, 1 if on else 0), "pdgb_enable_collision")

    def collision(self) -> tuple[np.ndarray, np.ndarray, dict]:
        """tI [nv], normals [nv, 3] and statistics of the last detection."""
        tI = np.empty(self.num_verts, np.float32)
        nrm = np.empty((self.num_verts, 3), np.float32)
        info = N.pdgb_collision_info()
        N.check(self._lib.pdgb_get_collision(self._h, tI.ctypes.data, nrm.ctypes.data, C.byref(info)),
                "pdgb_get_collision")
        return tI, nrm, {k: getattr(info, k) for k, _ in info._fields_}

    def render_surface(self, tris_ptr: int, num_tris: int, pos_ptr: int, nor_ptr: int) -> None:
        """Per-triangle corner positions (float[9 n]) and normals (float[12 n])
        of the current state into device buffers; tris_ptr: device uint32[3 n]
        caller vertex ids.  Stream-ordered on the engine's stream."""
        N.check(self._lib.pdgb_render_surface(self._h, C.c_void_p(tris_ptr), int(num_tris), C.c_void_p(pos_ptr),
                                              C.c_void_p(nor_ptr)), "pdgb_render_surface")

    # -- interactive drag (moreDBC / OffsetX / mouse target of SolverData)
    def set_drag(self, weights: np.ndarray, offsets: np.ndarray | None = None) -> None:
        w = np.ascontiguousarray(weights, dtype=np.float32).reshape(self.num_verts)
        o = None if offsets is None else np.ascontiguousarray(offsets, dtype=np.float32).reshape(self.num_verts, 3)
        N.check(self._lib.pdgb_set_drag(self._h, _ptr(w), _ptr(o), N.PDGB_MEM_HOST), "pdgb_set_drag")

    def drag_select(self, select_v: int, control_mag: float = 10.0, radius_sq: float = 0.002) -> None:
        """The reference's mouse selection (Control_Kernel) around vertex select_v."""
        N.check(self._lib.pdgb_drag_select(self._h, int(select_v), float(control_mag), float(radius_sq)),
                "pdgb_drag_select")

    def set_drag_target(self, target) -> None:
        t = (C.c_float * 3)(*[float(v) for v in target])
        N.check(self._lib.pdgb_set_drag_target(self._h, t), "pdgb_set_drag_target")

    def clear_drag(self) -> None:
        N.check(self._lib.pdgb_clear_drag(self._h), "pdgb_clear_drag")

    # -- fixed rigid bodies
    def set_fixed_bodies(self, bodies: list, mu_t: float = 0.5, mu_n: float = 0.5) -> None:
        arr = (N.pdgb_fixed_body * max(1, len(bodies)))(*[b.to_c() for b in bodies])
        N.check(self._lib.pdgb_set_fixed_bodies(self._h, arr, len(bodies), float(mu_t), float(mu_n)),
                "pdgb_set_fixed_bodies")

    def download_body(self, b: int) -> tuple[np.ndarray, np.ndarray]:
        n = int(self.body_verts[b + 1] - self.body_verts[b])
        X = np.empty((n, 3), dtype=np.float32)
        V = np.empty((n, 3), dtype=np.float32)
        N.check(self._lib.pdgb_download_body(self._h, int(b), _ptr(X), _ptr(V), N.PDGB_MEM_HOST), "pdgb_download_body")
        return X, V

    def get_performance_data(self) -> dict:
        p = N.pdgb_perf()
        N.check(self._lib.pdgb_get_perf(self._h, C.byref(p)), "pdgb_get_perf")
        return {"prepare_ms": p.prepare_ms, "steps": p.steps, "iterations": p.iterations,
                "factor_nnz": p.factor_nnz, "tiles": p.tiles, "patch_verts": p.patch_verts}

    def solve_levels(self) -> int:
        """Levels of the supernodal elimination tree (Cholesky path)."""
        f = N.pdgb_factor_info()
        N.check(self._lib.pdgb_get_factor_info(self._h, C.byref(f)), "pdgb_get_factor_info")
        return f.num_levels

    def factor_info(self) -> dict:
        f = N.pdgb_factor_info()
        N.check(self._lib.pdgb_get_factor_info(self._h, C.byref(f)), "pdgb_get_factor_info")
        return {k: getattr(f, k) for k, _ in f._fields_}

    def set_factor_device(self, device: int) -> None:
        """PDGB_FACTOR_GPU (default) or PDGB_FACTOR_HOST: where the one-time FP64
        numeric factorisation of the Cholesky path runs."""
        N.check(self._lib.pdgb_set_factor_device(self._h, int(device)), "pdgb_set_factor_device")

    def factor_blocks(self) -> np.ndarray:
        """The FP32 M_s blocks of the prepared factor (host copy)."""
        n = self.factor_info()["m_entries"]
        out = np.empty(max(int(n), 1), np.float32)
        N.check(self._lib.pdgb_get_factor_blocks(self._h, out.ctypes.data, int(out.size)), "pdgb_get_factor_blocks")
        return out[: int(n)]

    def last_step_iterations(self) -> int:
        it = C.c_int()
        N.check(self._lib.pdgb_last_step_iterations(self._h, C.byref(it)), "pdgb_last_step_iterations")
        return it.value

    # -- measurement hooks
    def enable_kernel_timing(self, on=True) -> None:
        """on: False/0 off, 1 step events only, True/2 step and local-kernel events."""
        mode = 2 if on is True else int(on)
        N.check(self._lib.pdgb_enable_kernel_timing(self._h, mode), "pdgb_enable_kernel_timing")

    def read_timing(self) -> dict:
        t = N.pdgb_timing()
        N.check(self._lib.pdgb_read_timing(self._h, C.byref(t)), "pdgb_read_timing")
        return {"step_ms": t.step_ms, "steps": t.steps, "local_ms": t.local_ms, "local_launches": t.local_launches,
                "solve_ms": t.solve_ms, "solves": t.solves}

    def local_step_bytes(self) -> float:
        b = C.c_double()
        N.check(self._lib.pdgb_local_step_bytes(self._h, C.byref(b)), "pdgb_local_step_bytes")
        return b.value

    def set_solve_mode(self, mode: int) -> None:
        """PDGB_SOLVE_AUTO / CTA / CLUSTER / LEVELS (schedule of the Cholesky solve)."""
        N.check(self._lib.pdgb_set_solve_mode(self._h, int(mode)), "pdgb_set_solve_mode")

    def time_local(self, launches: int = 100) -> float:
        """Average device ms of back-to-back local-step launches on the current state."""
        ms = C.c_double()
        N.check(self._lib.pdgb_time_local(self._h, int(launches), C.byref(ms)), "pdgb_time_local")
        return ms.value

    def set_tile_size(self, max_tets: int) -> None:
        """Most tets per local-step tile (32..512; 0 = 512)."""
        N.check(self._lib.pdgb_set_tile_size(self._h, int(max_tets)), "pdgb_set_tile_size")

    def autotune(self, steps: int = 5) -> dict:
        """Times tile sizes and solve schedules on this mesh, keeps the fastest
        (state restored; the simulation does not advance)."""
        r = N.pdgb_tune_report()
        N.check(self._lib.pdgb_autotune(self._h, int(steps), C.byref(r)), "pdgb_autotune")
        return {k: getattr(r, k) for k, _ in r._fields_ if k != "reserved"}

    def solve_mode(self) -> int:
        m = C.c_int()
        N.check(self._lib.pdgb_get_solve_mode(self._h, C.byref(m)), "pdgb_get_solve_mode")
        return m.value

    def solve_bytes(self) -> float:
        """Algorithmic bytes of one Cholesky solve (0 on the Jacobi path)."""
        b = C.c_double()
        N.check(self._lib.pdgb_solve_bytes(self._h, C.byref(b)), "pdgb_solve_bytes")
        return b.value

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.pdgb_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def ccd_detect(tris: np.ndarray, tri_body: np.ndarray, X: np.ndarray, XT: np.ndarray):
    """One continuous-collision detection on the GPU between start positions
    X and end positions XT (host arrays): (tI [nv], normals [nv, 3], info)."""
    lib = N.lib()
    X = np.ascontiguousarray(X, np.float32).reshape(-1, 3)
    XT = np.ascontiguousarray(XT, np.float32).reshape(-1, 3)
    t = np.ascontiguousarray(tris, np.uint32).reshape(-1, 3)
    b = np.ascontiguousarray(tri_body, np.int32)
    tI = np.empty(X.shape[0], np.float32)
    nrm = np.empty((X.shape[0], 3), np.float32)
    info = N.pdgb_collision_info()
    N.check(lib.pdgb_ccd_detect(X.shape[0], t.shape[0], t.ctypes.data, b.ctypes.data, X.ctypes.data, XT.ctypes.data,
                                tI.ctypes.data, nrm.ctypes.data, C.byref(info)), "pdgb_ccd_detect")
    return tI, nrm, {k: getattr(info, k) for k, _ in info._fields_}
