"""Host side of the Cholesky global solve (no GPU): system assembly, AMD / nested
dissection orderings, FP64 supernodal factorisation and the M_s blocks the GPU
applies, checked against the oracle's independent sparse solve."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_l2

import oracle as O
from pdgb import SolverParams, mesh
from pdgb import _native as N


def factor_check(body, ordering=0, b=None, dt=1 / 120, pw=1e6):
    lib = N.lib()
    X = np.ascontiguousarray(body.X, np.float32)
    T = np.ascontiguousarray(body.tets, np.uint32)
    m = np.ascontiguousarray(body.mass, np.float32)
    mu = np.ascontiguousarray(body.mu, np.float32)
    d = np.ascontiguousarray(body.dbc, np.float32)
    desc = N.pdgb_mesh_desc(X.shape[0], T.shape[0], X.ctypes.data, None, T.ctypes.data, m.ctypes.data,
                            mu.ctypes.data, d.ctypes.data, N.PDGB_MEM_HOST)
    prm = SolverParams(solver=1, dt=dt, positional_weight=pw).to_c()
    info = N.pdgb_factor_info()
    x = None if b is None else np.zeros_like(b)
    st = lib.pdgb_host_factor_check(C.byref(desc), C.byref(prm), ordering, None if b is None else b.ctypes.data,
                                    None if b is None else x.ctypes.data, C.byref(info))
    return st, info, x


@pytest.mark.parametrize("ordering", [N.PDGB_ORDER_AMD, N.PDGB_ORDER_ND, N.PDGB_ORDER_DENSE])
@pytest.mark.parametrize("case", ["tet", "grid3", "c1", "grid_aniso"])
def test_factor_solves_like_the_oracle(case, ordering):
    body = {"tet": lambda: mesh.single_tet(),
            "grid3": lambda: mesh.make_grid_body(3, 3, 3, jitter=0.1, seed=1),
            "c1": mesh.cube_c1,
            "grid_aniso": lambda: mesh.make_grid_body(12, 3, 7, young=3e6, jitter=0.15, seed=4)}[case]()
    rng = np.random.default_rng(3)
    b = rng.normal(size=(body.num_verts, 3))
    st, info, x = factor_check(body, ordering, b)
    assert st == N.PDGB_OK, N.lib().pdgb_last_error()
    xo = O.solve3(body, 1 / 120, b)
    # M_s is stored in float: ~1e-7 relative
    assert rel_l2(x, xo) < 1e-6
    assert info.num_levels >= 1 and info.fwd_items >= info.num_supernodes


def test_amd_fill_is_competitive():
    """AMD fill on a 3D grid stays within 1.3x of nested dissection, and after
    supernode amalgamation the solve has few levels (tree depth)."""
    body = mesh.make_grid_body(16, 16, 16)
    _, amd, _ = factor_check(body, N.PDGB_ORDER_AMD)
    _, nd, _ = factor_check(body, N.PDGB_ORDER_ND)
    n = body.num_verts
    assert amd.nnz_L < 1.3 * nd.nnz_L
    assert amd.nnz_L < n * (n + 1) // 2 / 10  # far from dense
    assert amd.num_levels <= max(16, 2 * nd.num_levels)


def test_not_spd_is_reported():
    body = mesh.make_grid_body(2, 2, 2)
    body.mass = -np.abs(body.mass) * 1e9  # negative inertia term dominates
    st, _, _ = factor_check(body, N.PDGB_ORDER_AMD)
    assert st == N.PDGB_ERR_NOT_SPD
    assert b"not positive definite" in N.lib().pdgb_last_error()
