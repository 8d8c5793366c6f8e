"""The allocation-free entry point pdgb_step_noalloc, through the C ABI.

It serves callers that must not allocate device memory while they advance a
body (a host application whose own allocator owns the GPU memory, a frame loop
where cudaMalloc/cudaFree would stall the device, a plugin handed only device
pointers).  Its results must match the regular entry points
(pdgb_create + pdgb_step, Jacobi + Chebyshev) within the parity tolerance, on
two calls in a row that share the library's fixed scratch array.

It is also held to the same bar as the engine on its own: the reference's
own kernels (golden fixtures) and the FP64 oracle, within 1e-4 relative L2 of
the positions.

This file is collected last on purpose; it allocates its test arrays with
torch, but the entry point itself allocates nothing.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden, rel_l2

import oracle as O
from pdgb import PdSolver, SolverParams, mesh
from pdgb import _native as N

pytestmark = pytest.mark.gpu

TOL = 1e-4


def _device_mesh(torch, body):
    dev = {k: torch.from_numpy(np.ascontiguousarray(getattr(body, k))).cuda()
           for k in ("X", "tets", "mass", "mu", "dbc")}
    m = N.pdgb_noalloc_mesh(body.num_verts, body.num_tets, dev["tets"].data_ptr(), dev["X"].data_ptr(),
                            dev["mass"].data_ptr(), dev["mu"].data_ptr(), dev["dbc"].data_ptr())
    return dev, m


def test_noalloc_matches_engine_on_two_calls():
    torch = pytest.importorskip("torch")
    lib = N.lib()
    body = mesh.make_grid_body(9, 7, 6, young=2e5, poisson=0.4, jitter=0.1, seed=12)
    params = SolverParams(num_iterations=20, rho=0.9995, solver=0)
    dev, m = _device_mesh(torch, body)
    X = dev["X"].clone()
    V = torch.zeros_like(X)
    prm = params.to_c()
    stream = torch.cuda.current_stream().cuda_stream
    results = []
    for _ in range(2):  # two calls in a row, 4 steps each
        st = lib.pdgb_step_noalloc(C.byref(m), C.byref(prm), X.data_ptr(), V.data_ptr(), 4, stream)
        assert st == N.PDGB_OK
        torch.cuda.synchronize()
        results.append((X.cpu().numpy().copy(), V.cpu().numpy().copy()))
    with PdSolver(body, params) as e:
        for k in range(2):
            e.update(4)
            Xe, Ve = e.download_state()
            Xn, Vn = results[k]
            assert np.isfinite(Xn).all()
            assert rel_l2(Xn, Xe) < TOL
            assert rel_l2(Xn - body.X, Xe - body.X) < 2e-3
            assert rel_l2(Vn, Ve) < 1e-2


@pytest.mark.parametrize("name", ["grid3_jacobi", "c1_jacobi"])
def test_noalloc_matches_reference_fixture_and_fp64_oracle(name):
    torch = pytest.importorskip("torch")
    lib = N.lib()
    body, params, steps, Xg, Vg, _ = load_golden(name)
    dev, m = _device_mesh(torch, body)
    X = dev["X"].clone()
    V = torch.zeros_like(X)
    prm = params.to_c()
    st = lib.pdgb_step_noalloc(C.byref(m), C.byref(prm), X.data_ptr(), V.data_ptr(), steps, None)
    assert st == N.PDGB_OK
    Xn = X.cpu().numpy()
    assert np.isfinite(Xn).all()
    assert rel_l2(Xn, Xg) < TOL
    assert rel_l2(Xn - body.X, Xg - body.X) < 2e-3
    Xo, _, _ = O.simulate(body, params, steps, precision=64)
    assert rel_l2(Xn, Xo) < TOL


def _bad_call(torch, lib, body, prm):
    """One call on a bad mesh: PDGB_ERR_BAD_MESH, with X and V untouched."""
    dev, m = _device_mesh(torch, body)
    X = dev["X"].clone()
    V = torch.full_like(X, 0.25)
    X_before, V_before = X.clone(), V.clone()
    st = lib.pdgb_step_noalloc(C.byref(m), C.byref(prm), X.data_ptr(), V.data_ptr(), 2, None)
    torch.cuda.synchronize()
    assert st == N.PDGB_ERR_BAD_MESH
    assert torch.equal(X, X_before) and torch.equal(V, V_before)


def test_noalloc_rejects_oversize_and_bad_meshes():
    torch = pytest.importorskip("torch")
    lib = N.lib()
    prm = SolverParams(num_iterations=5, solver=0).to_c()
    big = N.pdgb_noalloc_mesh(32769, 10, 1, 1, 1, 1, None)  # sizes are checked before any access
    assert lib.pdgb_step_noalloc(C.byref(big), C.byref(prm), 1, 1, 1, None) == N.PDGB_ERR_UNSUPPORTED
    big = N.pdgb_noalloc_mesh(10, 131073, 1, 1, 1, 1, None)
    assert lib.pdgb_step_noalloc(C.byref(big), C.byref(prm), 1, 1, 1, None) == N.PDGB_ERR_UNSUPPORTED
    # out-of-range index: found on the device, nothing is read there
    body = mesh.make_grid_body(2, 2, 2)
    body.tets = body.tets.copy()
    body.tets[1, 2] = body.num_verts + 5
    _bad_call(torch, lib, body, prm)
    # a tet whose double DmInv overflows float (edges of 1e-39 m, float
    # denormals): rejected like a flat one
    body = mesh.make_grid_body(2, 2, 2)
    nv = body.num_verts
    tiny = np.array([[0, 0, 0], [1e-39, 0, 0], [0, 1e-39, 0], [0, 0, 1e-39]], np.float32)
    assert tiny[1, 0] > 0.0
    body.X = np.concatenate([body.X, tiny])
    body.mass = np.concatenate([body.mass, np.ones(4, np.float32)])
    body.dbc = np.concatenate([body.dbc, np.zeros(4, np.float32)])
    body.tets = np.concatenate([body.tets, np.arange(nv, nv + 4, dtype=np.uint32)[None]])
    body.mu = np.concatenate([body.mu, body.mu[:1]])
    _bad_call(torch, lib, body, prm)
    # a negative weight
    body = mesh.make_grid_body(2, 2, 2)
    body.mu = body.mu.copy()
    body.mu[5] = -1.0
    _bad_call(torch, lib, body, prm)
    # and a good mesh still steps after the bad calls
    body = mesh.make_grid_body(2, 2, 2)
    dev, m = _device_mesh(torch, body)
    X = dev["X"].clone()
    V = torch.zeros_like(X)
    assert lib.pdgb_step_noalloc(C.byref(m), C.byref(prm), X.data_ptr(), V.data_ptr(), 2, None) == N.PDGB_OK
    assert torch.isfinite(X).all()
