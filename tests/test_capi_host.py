"""C ABI and host-side logic, no GPU needed: the library loads, exports every
symbol include/pdgb.h declares, and the host layout (Morton renumbering, tet
tiles and their vertex patches) is consistent."""
import ctypes as C
import re

import numpy as np
import pytest

from conftest import ROOT

from pdgb import _native as N
from pdgb import mesh


def declared_symbols():
    text = (ROOT / "include" / "pdgb.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pdgb_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(str(N.library_path()))
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the binding knows all of them
    assert set(names) <= set(N.SIGNATURES), set(names) - set(N.SIGNATURES)


def test_status_strings_and_defaults():
    lib = N.lib()
    assert lib.pdgb_status_string(N.PDGB_OK) == b"ok"
    assert lib.pdgb_status_string(N.PDGB_ERR_BAD_MESH) == b"bad mesh"
    assert lib.pdgb_version().startswith(b"pdgb")
    p = N.pdgb_params()
    lib.pdgb_default_params(C.byref(p))
    assert abs(p.dt - 1 / 120) < 1e-9 and p.positional_weight == 1e6 and p.solver == N.PDGB_SOLVER_JACOBI
    assert abs(p.rho - 0.9992) < 1e-6  # SolverParams<float>::rho default (def.h:97)


def test_null_arguments_are_rejected_without_gpu():
    lib = N.lib()
    out = C.c_void_p()
    assert lib.pdgb_create(None, None, None, C.byref(out)) == N.PDGB_ERR_INVALID_ARGUMENT
    assert out.value is None
    assert lib.pdgb_step(None, 1) == N.PDGB_ERR_INVALID_ARGUMENT
    assert lib.pdgb_destroy(None) == N.PDGB_ERR_INVALID_ARGUMENT


def inspect(body):
    lib = N.lib()
    X = np.ascontiguousarray(body.X, np.float32)
    T = np.ascontiguousarray(body.tets, np.uint32)
    m = np.ascontiguousarray(body.mass, np.float32)
    mu = np.ascontiguousarray(body.mu, np.float32)
    d = N.pdgb_mesh_desc(X.shape[0], T.shape[0], X.ctypes.data, None, T.ctypes.data, m.ctypes.data, mu.ctypes.data,
                         None, N.PDGB_MEM_HOST)
    info = N.pdgb_layout_info()
    vperm = np.empty(X.shape[0], np.int32)
    tperm = np.empty(T.shape[0], np.int32)
    st = lib.pdgb_inspect_layout(C.byref(d), C.byref(info), vperm.ctypes.data, tperm.ctypes.data)
    return st, info, vperm, tperm


@pytest.mark.parametrize("dims", [(1, 1, 1), (3, 4, 5), (16, 16, 16)])
def test_layout_is_a_valid_tiling(dims):
    body = mesh.make_grid_body(*dims, jitter=0.1, seed=1)
    st, info, vperm, tperm = inspect(body)
    assert st == N.PDGB_OK
    assert np.array_equal(np.sort(vperm), np.arange(body.num_verts))
    assert np.array_equal(np.sort(tperm), np.arange(body.num_tets))
    assert 1 <= info.num_tiles and info.max_patch <= 1024 and info.max_tile_tets <= 512
    assert info.num_tiles == -(-body.num_tets // 512) or info.max_patch == 1024
    # every tet corner is in its tile's patch: sum of patch sizes >= distinct verts
    assert info.patch_verts >= body.num_verts


def test_layout_patch_reuse_on_large_grid():
    """Morton tiles on a 32^3 grid: each vertex is staged by few tiles."""
    body = mesh.make_grid_body(32, 32, 32, jitter=0.1, seed=1)
    st, info, _, _ = inspect(body)
    assert st == N.PDGB_OK
    dup = info.patch_verts / body.num_verts
    assert dup < 2.5, dup


def test_bad_mesh_rejected_on_host():
    body = mesh.make_grid_body(2, 2, 2)
    body.tets = body.tets.copy()
    body.tets[3, 2] = body.num_verts + 7
    st, *_ = inspect(body)
    assert st == N.PDGB_ERR_BAD_MESH
    assert b"references vertex" in N.lib().pdgb_last_error()
    flat = mesh.make_grid_body(2, 2, 2)
    flat.tets = flat.tets.copy()
    flat.tets[0] = [0, 1, 2, 2]  # zero volume
    st, *_ = inspect(flat)
    assert st == N.PDGB_ERR_BAD_MESH


def test_chebyshev_schedule_matches_reference_host_loop():
    """omega per iteration as the reference computes it in float (pdSolver.cu:196-199)."""
    rho = np.float32(0.9995)
    om = np.float32(1.0)
    seq = []
    for i in range(20):
        if i <= 10:
            om = np.float32(1.0)
        elif i == 11:
            om = np.float32(2) / (np.float32(2) - rho * rho)
        else:
            om = np.float32(4) / (np.float32(4) - rho * rho * om)
        seq.append(om)
    assert seq[11] > 1.9 and all(1.0 <= w < 2.0 for w in seq)


def test_layout_splits_tiles_at_long_vertex_runs():
    """A vertex with 200 corners: a tile holds at most 64 corners of one
    vertex (the rank field of a corner record), so the 200 tets span at
    least 4 tiles; orders stay permutations."""
    from conftest import fan_body

    body = fan_body(100)
    st, info, vperm, tperm = inspect(body)
    assert st == N.PDGB_OK
    assert info.num_tiles >= 4
    assert info.max_tile_tets <= 64
    assert np.array_equal(np.sort(vperm), np.arange(body.num_verts))
    assert np.array_equal(np.sort(tperm), np.arange(body.num_tets))


def test_negative_weight_is_rejected():
    body = mesh.make_grid_body(2, 2, 2)
    body.mu = body.mu.copy()
    body.mu[3] = -1.0
    st, _, _, _ = inspect(body)
    assert st == N.PDGB_ERR_BAD_MESH
    assert "weight" in N.lib().pdgb_last_error().decode()
