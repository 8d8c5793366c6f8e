"""GPU parity of the Jacobi + Chebyshev PD path (libpdgb.so through the C ABI).

Bar: vertex positions after N steps within 1e-4 relative L2 of (a) the
reference's own kernels (golden fixtures) and (b) the FP64 oracle.
"""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden, rel_l2

import oracle as O
from pdgb import PdgbError, PdSolver, SolverParams, mesh
from pdgb import _native as N

pytestmark = pytest.mark.gpu

TOL = 1e-4


@pytest.mark.parametrize("name", [c for c in GOLDEN_CASES if c.endswith("jacobi")])
def test_engine_matches_reference_fixture(name):
    body, params, steps, Xg, Vg, _ = load_golden(name)
    with PdSolver(body, params) as e:
        e.update(steps)
        X, V = e.download_state()
    assert np.isfinite(X).all() and np.isfinite(V).all()
    assert rel_l2(X, Xg) < TOL
    assert rel_l2(X - body.X, Xg - body.X) < 2e-3
    Xo, _, _ = O.simulate(body, params, steps, precision=64)
    assert rel_l2(X, Xo) < TOL


def test_engine_vs_fp64_oracle_jittered_grid():
    body = mesh.make_grid_body(16, 12, 14, young=1e6, poisson=0.45, jitter=0.1, seed=21)
    params = SolverParams(num_iterations=20, rho=0.9995, solver=0)
    with PdSolver(body, params) as e:
        e.update(25)
        X, V = e.download_state()
    Xo, Vo, _ = O.simulate(body, params, 25, precision=64)
    assert rel_l2(X, Xo) < TOL
    assert rel_l2(X - body.X, Xo - body.X) < 1e-3
    assert rel_l2(V, Vo) < 1e-2


@pytest.mark.parametrize("solver", [0, 1])
def test_high_valence_vertex_vs_oracle(solver):
    """A centre vertex shared by 200 tets spans several tiles (at most 64
    of its corners per tile); the step still matches the FP64 oracle."""
    from conftest import fan_body

    body = fan_body(100, seed=5)
    params = SolverParams(num_iterations=20, rho=0.999, solver=solver)
    with PdSolver(body, params) as e:
        e.update(10)
        X, _ = e.download_state()
    Xo, _, _ = O.simulate(body, params, 10, precision=64)
    assert np.isfinite(X).all()
    assert rel_l2(X, Xo) < TOL


def test_vertices_outside_every_tet_vs_oracle():
    """Vertices that no tet references (free particles, one of them pinned)
    are in no tile: they keep the inertial iterate through the fused
    iterations and still get the final velocity / position update."""
    body = mesh.make_grid_body(4, 3, 5, young=1e5, poisson=0.4, jitter=0.1, seed=9)
    extra = np.array([[2.0, 0.5, 0.5], [-1.0, 0.2, 0.1], [0.5, 3.0, 0.5]], np.float32)
    body.X = np.concatenate([body.X, extra])
    body.mass = np.concatenate([body.mass, np.array([0.5, 2.0, 1.0], np.float32)])
    body.dbc = np.concatenate([body.dbc, np.array([0.0, 0.0, 1.0], np.float32)])
    body.V = np.zeros_like(body.X)
    body.V[-2] = (0.3, 0.0, -0.2)
    for solver, rho in ((0, 0.9995), (1, 0.9992)):
        params = SolverParams(num_iterations=20, rho=rho, solver=solver)
        with PdSolver(body, params) as e:
            e.update(12)
            X, V = e.download_state()
        Xo, Vo, _ = O.simulate(body, params, 12, precision=64, V=body.V)
        assert rel_l2(X, Xo) < TOL, solver
        assert np.allclose(X[-3:], Xo[-3:], rtol=0, atol=1e-5), solver
        # velocities are position changes / h: one float ulp of a 2 m
        # coordinate is 2.4e-7 m, i.e. 3e-5 m/s at h = 1/120
        assert np.allclose(V[-3:], Vo[-3:], rtol=0, atol=5e-4), solver


def test_large_grid_first_steps_vs_oracle():
    """64^3 cells (274,625 verts / 1,310,720 tets): 2 steps vs the FP64 oracle."""
    body = mesh.cube_c2()
    params = SolverParams(num_iterations=20, rho=0.9995, solver=0)
    with PdSolver(body, params) as e:
        e.update(2)
        X, V = e.download_state()
    Xo, Vo, _ = O.simulate(body, params, 2, precision=64)
    assert rel_l2(X, Xo) < TOL
    assert rel_l2(X - body.X, Xo - body.X) < 1e-3


def test_pinned_vertices_hold_and_body_sags():
    body = mesh.make_grid_body(8, 8, 8, young=1e5, poisson=0.4)
    params = SolverParams(num_iterations=20, rho=0.9995, solver=0)
    with PdSolver(body, params) as e:
        e.update(30)
        X, _ = e.download_state()
    pinned = body.dbc > 0
    assert np.abs(X[pinned] - body.X[pinned]).max() < 1e-5
    assert (X[~pinned, 1] <= body.X[~pinned, 1] + 1e-6).all()  # gravity pulls down
    assert (X[~pinned, 1] < body.X[~pinned, 1] - 1e-4).any()


def test_rigid_motion_is_preserved():
    """No gravity, no pins, rest shape rigidly rotated and moved: R = Q, F = Q, so
    every PD term is zero and the body must not move."""
    body = mesh.make_grid_body(5, 6, 7, jitter=0.1, seed=2, pin=None)
    rng = np.random.default_rng(4)
    Q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    if np.linalg.det(Q) < 0:
        Q[:, 0] *= -1
    Xm = (body.X.astype(np.float64) @ Q.T + np.array([0.3, -1.0, 2.0])).astype(np.float32)
    params = SolverParams(num_iterations=20, rho=0.9995, gravity=0.0, solver=0)
    with PdSolver(body, params) as e:
        e.upload_state(Xm, np.zeros_like(Xm))
        e.update(10)
        X, V = e.download_state()
    assert np.abs(X - Xm).max() < 2e-5
    assert np.abs(V).max() < 2e-3


def test_state_roundtrip_reset_and_reprepare():
    body = mesh.make_grid_body(4, 5, 6, jitter=0.1, seed=8)
    params = SolverParams(num_iterations=12, rho=0.999, solver=0)
    rng = np.random.default_rng(0)
    with PdSolver(body, params) as e:
        Xr = (body.X + rng.normal(scale=1e-3, size=body.X.shape)).astype(np.float32)
        Vr = rng.normal(scale=1e-2, size=body.X.shape).astype(np.float32)
        e.upload_state(Xr, Vr)
        X, V = e.download_state()
        assert np.array_equal(X, Xr) and np.array_equal(V, Vr)
        e.update(5)
        X1, _ = e.download_state()
        e.reset()
        X, V = e.download_state()
        assert np.array_equal(X, body.X) and not V.any()
        e.upload_state(Xr, Vr)
        e.update(5)
        X2, _ = e.download_state()
        assert rel_l2(X2, X1) < 1e-6  # same result after reset + re-prepare
        # changing params re-prepares: iterations change the result
        e.set_params(SolverParams(num_iterations=20, rho=0.999, solver=0))
        e.upload_state(Xr, Vr)
        e.update(5)
        X3, _ = e.download_state()
        Xo, _, _ = O.simulate(body, SolverParams(num_iterations=20, rho=0.999, solver=0), 5, 64, X=Xr, V=Vr)
        assert rel_l2(X3, Xo) < TOL


def test_bad_inputs_raise():
    body = mesh.make_grid_body(2, 2, 2)
    bad = mesh.make_grid_body(2, 2, 2)
    bad.tets = bad.tets.copy()
    bad.tets[0, 0] = 10_000
    with pytest.raises(PdgbError) as ei:
        PdSolver(bad, SolverParams())
    assert ei.value.status == N.PDGB_ERR_BAD_MESH
    with pytest.raises(PdgbError) as ei:
        PdSolver(body, SolverParams(dt=-1.0))
    assert ei.value.status == N.PDGB_ERR_INVALID_ARGUMENT
    with pytest.raises(PdgbError):
        PdSolver(body, SolverParams(num_iterations=0))


def test_mesh_from_device_memory():
    torch = pytest.importorskip("torch")
    body = mesh.make_grid_body(5, 5, 5, jitter=0.1, seed=5)
    params = SolverParams(num_iterations=20, rho=0.9995, solver=0)
    dev = {k: torch.from_numpy(np.ascontiguousarray(getattr(body, k))).cuda() for k in ("X", "tets", "mass", "mu", "dbc")}
    torch.cuda.synchronize()
    lib = N.lib()
    desc = N.pdgb_mesh_desc(body.num_verts, body.num_tets, dev["X"].data_ptr(), None, dev["tets"].data_ptr(),
                            dev["mass"].data_ptr(), dev["mu"].data_ptr(), dev["dbc"].data_ptr(), N.PDGB_MEM_DEVICE)
    h = C.c_void_p()
    prm = params.to_c()
    N.check(lib.pdgb_create(C.byref(desc), C.byref(prm), None, C.byref(h)), "create")
    try:
        N.check(lib.pdgb_step(h, 8), "step")
        Xd = torch.empty((body.num_verts, 3), dtype=torch.float32, device="cuda")
        N.check(lib.pdgb_download_state(h, Xd.data_ptr(), None, N.PDGB_MEM_DEVICE), "download")
        N.check(lib.pdgb_synchronize(h), "sync")
        X = Xd.cpu().numpy()
    finally:
        lib.pdgb_destroy(h)
    with PdSolver(body, params) as e:
        e.update(8)
        Xh, _ = e.download_state()
    assert rel_l2(X, Xh) < 1e-6


def test_independent_engines_do_not_interfere():
    a = mesh.make_grid_body(6, 6, 6, jitter=0.1, seed=1)
    b = mesh.make_grid_body(9, 4, 7, young=3e5, jitter=0.1, seed=2)
    pa = SolverParams(num_iterations=20, rho=0.9995, solver=0)
    pb = SolverParams(num_iterations=15, rho=0.999, solver=0)
    with PdSolver(a, pa) as ea, PdSolver(b, pb) as eb:
        for _ in range(6):
            ea.update(1)
            eb.update(1)
        Xa, _ = ea.download_state()
        Xb, _ = eb.download_state()
    Xa1, _, _ = O.simulate(a, pa, 6, 64)
    Xb1, _, _ = O.simulate(b, pb, 6, 64)
    assert rel_l2(Xa, Xa1) < TOL and rel_l2(Xb, Xb1) < TOL


def test_kernel_timing_hook_counts_launches():
    body = mesh.make_grid_body(8, 8, 8)
    params = SolverParams(num_iterations=7, rho=0.999, solver=0)
    with PdSolver(body, params) as e:
        e.enable_kernel_timing(True)
        e.update(3)
        t = e.read_timing()
        assert t["local_launches"] == 21 and t["steps"] == 3
        assert 0 < t["local_ms"] < t["step_ms"]
        assert e.local_step_bytes() == 56.0 * body.num_tets + 36.0 * body.num_verts
        # step events only: no per-local records, no wait inside pdgb_step
        e.enable_kernel_timing(1)
        e.update(4)
        t = e.read_timing()
        assert t["steps"] == 4 and t["local_launches"] == 0 and t["step_ms"] > 0
        assert e.read_timing()["steps"] == 0
        X, _ = e.download_state()
    Xo, _, _ = O.simulate(body, params, 7, 64)
    assert rel_l2(X, Xo) < TOL


@pytest.mark.parametrize("cap", [32, 64, 200, 512])
def test_tile_size_gives_same_step(cap):
    """Re-cut tiles (pdgb_set_tile_size) change only the float summation
    order of the local step."""
    body = mesh.make_grid_body(7, 6, 5, jitter=0.1, seed=21)
    params = SolverParams(num_iterations=15, rho=0.999, solver=0)
    with PdSolver(body, params) as e:
        e.update(2)
        e.set_tile_size(cap)
        e.update(4)
        X, _ = e.download_state()
        tiles = e.get_performance_data()["tiles"]
    assert tiles >= (body.num_tets + cap - 1) // cap
    Xo, _, _ = O.simulate(body, params, 6, precision=64)
    assert rel_l2(X, Xo) < TOL


@pytest.mark.parametrize("solver", [0, 1])
def test_autotune_keeps_state_and_result(solver):
    body = mesh.make_grid_body(8, 8, 8, jitter=0.1, seed=22, young=4e4)
    params = SolverParams(num_iterations=10 if solver else 20, rho=0.9995, solver=solver)
    with PdSolver(body, params) as e:
        e.update(3)
        X3, V3 = e.download_state()
        rep = e.autotune(steps=3)
        Xa, Va = e.download_state()
        assert np.array_equal(Xa, X3) and np.array_equal(Va, V3)  # tuning does not advance the state
        assert rep["candidates"] >= (9 if solver else 5)
        assert 0 < rep["best_ms"] <= rep["default_ms"] * 1.0001
        assert rep["tile_tets"] in (64, 128, 256, 512)
        e.update(3)
        X, _ = e.download_state()
    Xo, _, _ = O.simulate(body, params, 6, precision=64)
    assert rel_l2(X, Xo) < TOL


def _deformation_gradients(n, seed):
    """Rotations times stretches (singular values exp(U(-1.2, 1.2))), with
    inverted, nearly flat and near-identity cases mixed in."""
    rng = np.random.default_rng(seed)
    F = []
    for k in range(n):
        Q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        if np.linalg.det(Q) < 0:
            Q[:, 0] = -Q[:, 0]
        W, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        s = np.exp(rng.uniform(-1.2, 1.2, size=3))
        if k % 7 == 3:
            s[2] = -0.3 * s[2]                    # inverted
        if k % 11 == 5:
            s[2] = 1e-3                          # nearly flat
        if k % 5 == 1:
            s = 1.0 + rng.uniform(-0.05, 0.05, 3)  # mild
        F.append(Q @ np.diag(s) @ W.T)
    return np.asarray(F, dtype=np.float32)


@pytest.mark.parametrize("mode", [N.PDGB_ROTATION_QUAT, N.PDGB_ROTATION_SVD])
def test_device_rotation_accuracy(mode):
    """The local step's rotation on its own (pdgb_closest_rotations) against
    the exact closest proper rotation (FP64 oracle); the quaternion form is
    converged to float precision, the SVD form reproduces the reference's
    4-sweep scheme (golden rotations of the reference's own SVD)."""
    F = _deformation_gradients(4096, 31)
    R = np.empty_like(F)
    N.check(N.lib().pdgb_closest_rotations(len(F), F.ctypes.data, R.ctypes.data, mode), "rotations")
    Rx = O.rotations(F.astype(np.float64), precision=64).reshape(-1, 3, 3)
    err = np.abs(R - Rx).max(axis=(1, 2))
    assert np.isfinite(R).all()
    assert np.allclose(np.linalg.det(R.astype(np.float64)), 1.0, atol=1e-5)
    if mode == N.PDGB_ROTATION_QUAT:
        # The closest rotation maximises tr(R^T F).  Where the two largest
        # eigenvalues of Horn's matrix N(F) nearly coincide (inverted
        # elements with |sigma_3| close to sigma_2) the maximiser is not
        # unique: there only the objective is compared.
        F64 = F.astype(np.float64)
        obj = np.einsum("nij,nij->n", R.astype(np.float64), F64)
        objx = np.einsum("nij,nij->n", Rx, F64)
        scale = np.linalg.norm(F64.reshape(-1, 9), axis=1)
        gap = np.empty(len(F))
        top2 = np.empty(len(F))
        for n, f in enumerate(F64):
            Nm = np.array([[f[0, 0] + f[1, 1] + f[2, 2], f[2, 1] - f[1, 2], f[0, 2] - f[2, 0], f[1, 0] - f[0, 1]],
                           [f[2, 1] - f[1, 2], f[0, 0] - f[1, 1] - f[2, 2], f[0, 1] + f[1, 0], f[0, 2] + f[2, 0]],
                           [f[0, 2] - f[2, 0], f[0, 1] + f[1, 0], f[1, 1] - f[0, 0] - f[2, 2], f[1, 2] + f[2, 1]],
                           [f[1, 0] - f[0, 1], f[0, 2] + f[2, 0], f[1, 2] + f[2, 1], f[2, 2] - f[0, 0] - f[1, 1]]])
            ev = np.linalg.eigvalsh(Nm)
            gap[n] = (ev[3] - ev[2]) / max(ev[3] - ev[0], 1e-300)
            top2[n] = ev[3] - ev[2]
        # tr(R^T F) = q^T N q: never above the maximum, and at least the
        # second eigenvalue of N (q in the dominant eigenspace)
        assert (obj <= objx + 1e-5 * scale).all()
        assert (obj >= objx - top2 - 1e-5 * scale).all(), np.max(objx - obj - top2)
        well = gap > 1e-2
        assert well.mean() > 0.95
        # float arithmetic: a few ulp on mild deformations, up to ~5e-6 on
        # strongly stretched or flat elements (the reference's 4-sweep SVD is
        # off by up to 1.7e-2 there)
        assert np.median(err[well]) < 5e-7, np.median(err[well])
        assert err[well].max() < 1e-5, err[well].max()
    else:
        z = np.load(Path(__file__).resolve().parent / "golden" / "rotations.npz")
        Fg = np.ascontiguousarray(z["F"], dtype=np.float32)  # keep the array alive across the call
        Rg = np.empty_like(Fg)
        N.check(N.lib().pdgb_closest_rotations(len(Fg), Fg.ctypes.data, Rg.ctypes.data, mode), "rotations")
        # the reference's scheme in float on the GPU (contracted multiply-adds)
        # against its CPU build: agreement to a few float ulp of the products
        assert np.abs(Rg - z["R"]).max() < 2e-5


def test_time_local_leaves_state():
    body = mesh.make_grid_body(10, 10, 10, jitter=0.1, seed=23)
    params = SolverParams(num_iterations=12, rho=0.999, solver=0)
    with PdSolver(body, params) as e:
        e.update(2)
        X2, V2 = e.download_state()
        ms = e.time_local(20)
        X, V = e.download_state()
        assert ms > 0 and np.array_equal(X, X2) and np.array_equal(V, V2)
        e.update(2)
        X4, _ = e.download_state()
    Xo, _, _ = O.simulate(body, params, 4, precision=64)
    assert rel_l2(X4, Xo) < TOL


@pytest.mark.gpu
@pytest.mark.parametrize("solver,tile", [(0, 0), (1, 0), (0, 37), (1, 101)])
def test_pipelined_local_step_matches_tile_form(solver, tile):
    """The pipelined local step (persistent CTAs, next tile bulk-copied into
    shared memory) against the one-CTA-per-tile form: same per-tet arithmetic
    and run sums, so the states agree to the rounding of the cross-tile
    atomics.  Odd tile caps give tiles starting at odd tets and patch lists
    starting off the 16-byte grid (the copy ranges are rounded out)."""
    body = mesh.cube_c2(20)
    params = SolverParams(num_iterations=10, rho=0.9995, solver=solver)
    out = {}
    for kind in (N.PDGB_LOCAL_TILE, N.PDGB_LOCAL_PIPELINED):
        with PdSolver(body, params) as e:
            if tile:
                e.set_tile_size(tile)
            e.set_local_kernel(kind)
            assert e.local_kernel() == kind
            e.update(6)
            out[kind] = e.download_state()[0]
            assert e.step_status() == N.PDGB_OK
    assert np.isfinite(out[N.PDGB_LOCAL_PIPELINED]).all()
    assert rel_l2(out[N.PDGB_LOCAL_PIPELINED], out[N.PDGB_LOCAL_TILE]) < 1e-6
    Xo, _, _ = O.simulate(body, params, 6, precision=64)
    assert rel_l2(out[N.PDGB_LOCAL_PIPELINED], Xo) < 1e-4


@pytest.mark.gpu
def test_local_kernel_setting_checked():
    body = mesh.cube_c2(6)
    with PdSolver(body, SolverParams(num_iterations=5)) as e:
        assert e.local_kernel() == N.PDGB_LOCAL_TILE
        with pytest.raises(PdgbError):
            e.set_local_kernel(2)
