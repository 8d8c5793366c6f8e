"""Python wrapper of the serving loop (pdgb_server_* in include/pdgb.h)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .engine import SolverParams, _host_desc
from .mesh import SoftBody


class PdServer:
    """Continuous-batching PD server: submit bodies with step counts, call
    tick() to advance every resident request by one step."""

    def __init__(self, params: SolverParams, hbm_budget_bytes: int = 8 << 30, max_active: int = 0,
                 host_threads: int = 0, stream: int | None = None, cache_entries: int = 0):
        """params.solver selects the global solve of every request (Jacobi +
        Chebyshev, or the Cholesky factor computed on the GPU at admission);
        cache_entries: meshes whose layout and factor are kept (0 = 256, < 0 =
        none)."""
        self._lib = N.lib()
        cfg = N.pdgb_server_config()
        self._lib.pdgb_server_default_config(C.byref(cfg))
        cfg.params = params.to_c()
        cfg.hbm_budget_bytes = int(hbm_budget_bytes)
        cfg.max_active = int(max_active)
        cfg.host_threads = int(host_threads)
        cfg.cache_entries = int(cache_entries)
        h = C.c_void_p()
        N.check(self._lib.pdgb_server_create(C.byref(cfg), stream, C.byref(h)), "pdgb_server_create")
        self._h = h
        self._nv: dict[int, int] = {}

    def submit(self, body: SoftBody, nsteps: int) -> int:
        keep: list = []
        desc = _host_desc(body, keep)
        rid = C.c_longlong()
        N.check(self._lib.pdgb_server_submit(self._h, C.byref(desc), int(nsteps), C.byref(rid)), "pdgb_server_submit")
        self._nv[rid.value] = body.num_verts
        return rid.value

    def tick(self) -> tuple[int, int]:
        a, c = C.c_int(), C.c_int()
        N.check(self._lib.pdgb_server_tick(self._h, C.byref(a), C.byref(c)), "pdgb_server_tick")
        return a.value, c.value

    def poll(self, rid: int) -> tuple[int, int]:
        st, done = C.c_int(), C.c_int()
        N.check(self._lib.pdgb_server_poll(self._h, rid, C.byref(st), C.byref(done)), "pdgb_server_poll")
        return st.value, done.value

    def result(self, rid: int) -> tuple[np.ndarray, np.ndarray]:
        n = self._nv.pop(rid)
        X = np.empty((n, 3), np.float32)
        V = np.empty((n, 3), np.float32)
        N.check(self._lib.pdgb_server_result(self._h, rid, X.ctypes.data, V.ctypes.data), "pdgb_server_result")
        return X, V

    def stats(self) -> dict:
        s = N.pdgb_server_stats()
        N.check(self._lib.pdgb_server_get_stats(self._h, C.byref(s)), "pdgb_server_get_stats")
        return {k: getattr(s, k) for k, _ in s._fields_}

    def latencies_ms(self) -> np.ndarray:
        n = C.c_int()
        N.check(self._lib.pdgb_server_latencies(self._h, None, 0, C.byref(n)), "pdgb_server_latencies")
        out = np.empty(n.value, np.float64)
        N.check(self._lib.pdgb_server_latencies(self._h, out.ctypes.data, n.value, C.byref(n)), "pdgb_server_latencies")
        return out

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.pdgb_server_destroy(self._h)
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
