"""GPU parity of the Cholesky PD path: prefactored sparse Cholesky (AMD, FP64
factor, FP32 level-scheduled supernodal solves) behind the C ABI.

Bar: positions after N steps within 1e-4 relative L2 of the reference's own
kernels (golden fixtures) and of the FP64 oracle; with tol > 0 the per-step
iteration counts of the reference's error-based early exit."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden, rel_l2

import oracle as O
from pdgb import PdgbError, PdSolver, SolverParams, mesh
from pdgb import _native as N

pytestmark = pytest.mark.gpu

TOL = 1e-4


@pytest.mark.parametrize("name", [c for c in GOLDEN_CASES if "chol" in c])
@pytest.mark.parametrize("rotation", [N.PDGB_ROTATION_QUAT, N.PDGB_ROTATION_SVD])
def test_engine_matches_reference_fixture(name, rotation):
    body, params, steps, Xg, Vg, itg = load_golden(name)
    with PdSolver(body, params) as e:
        e.set_rotation(rotation)
        its = []
        for _ in range(steps):
            e.update(1)
            its.append(e.last_step_iterations())
        X, V = e.download_state()
    assert np.isfinite(X).all() and np.isfinite(V).all()
    assert rel_l2(X, Xg) < TOL
    assert rel_l2(X - body.X, Xg - body.X) < 2e-3
    if params.tol > 0:
        # the early exit depends on float rounding near the threshold: allow
        # a one-iteration difference on a few steps
        d = np.abs(np.asarray(its) - itg)
        assert d.max() <= 1 and (d > 0).sum() <= max(1, steps // 10), (its, list(itg))
    else:
        assert all(i == params.num_iterations for i in its)
    Xo, _, _ = O.simulate(body, params, steps, precision=64)
    assert rel_l2(X, Xo) < TOL


@pytest.mark.parametrize("ordering", [N.PDGB_ORDER_AMD, N.PDGB_ORDER_ND])
def test_heterogeneous_grid_vs_fp64_oracle(ordering):
    """Per-tet Young's modulus log-uniform 1e4..1e7 (the precision workload's
    material law) on a 14^3 grid."""
    body = mesh.cube_c3(n=14, seed=5)
    params = SolverParams(num_iterations=10, solver=1)
    with PdSolver(body, params) as e:
        e.set_ordering(ordering)
        e.update(20)
        X, V = e.download_state()
        perf = e.get_performance_data()
    assert perf["factor_nnz"] > body.num_verts
    Xo, Vo, _ = O.simulate(body, params, 20, precision=64)
    assert rel_l2(X, Xo) < TOL
    assert rel_l2(X - body.X, Xo - body.X) < 2e-3


def test_switch_solver_at_runtime():
    """SetGlobalSolver between steps (simulationContext.cpp:104-114)."""
    body = mesh.make_grid_body(6, 5, 4, jitter=0.1, seed=6)
    pj = SolverParams(num_iterations=20, rho=0.9995, solver=0)
    with PdSolver(body, pj) as e:
        e.update(3)
        e.set_global_solver(1)
        e.update(3)
        e.set_global_solver(0)
        e.update(3)
        X, _ = e.download_state()
    Xa, Va, _ = O.simulate(body, pj, 3, 64)
    pc = SolverParams(num_iterations=20, rho=0.9995, solver=1)
    Xb, Vb, _ = O.simulate(body, pc, 3, 64, X=Xa, V=Va)
    Xc, _, _ = O.simulate(body, pj, 3, 64, X=Xb, V=Vb)
    assert rel_l2(X, Xc) < TOL


def test_cholesky_and_jacobi_agree_when_converged():
    """With many iterations both global solvers approach the same PD fixed point."""
    body = mesh.make_grid_body(5, 5, 5, young=1e5, jitter=0.1, seed=7)
    with PdSolver(body, SolverParams(num_iterations=40, solver=1)) as e:
        e.update(5)
        Xc, _ = e.download_state()
    with PdSolver(body, SolverParams(num_iterations=200, rho=0.9995, solver=0)) as e:
        e.update(5)
        Xj, _ = e.download_state()
    assert rel_l2(Xc - body.X, Xj - body.X) < 5e-2


def test_fp64_residual_refinement_tightens_the_solve():
    """FP32 tri-solves of the FP64 factor plus 0..3 FP64-residual refinement
    steps (the precision workload): error vs the FP64 oracle within the bar,
    and refinement does not make it worse."""
    body = mesh.cube_c3(n=12, seed=9)
    errs = []
    for refine in range(4):
        params = SolverParams(num_iterations=10, solver=1, refine_steps=refine)
        with PdSolver(body, params) as e:
            e.update(8)
            X, _ = e.download_state()
        if refine == 0:
            Xo, _, _ = O.simulate(body, params, 8, precision=64)
        errs.append(rel_l2(X - body.X, Xo - body.X))
        assert rel_l2(X, Xo) < TOL
    assert errs[1] <= errs[0] * 1.05 + 1e-9, errs
    assert max(errs[1:]) <= errs[0] * 1.05 + 1e-9, errs


def test_solve_timing_and_bytes():
    """Kernel timing brackets every global solve of the Cholesky path; the
    solve's algorithmic bytes follow the factor size."""
    body = mesh.make_grid_body(6, 6, 6, jitter=0.1, seed=3)
    params = SolverParams(num_iterations=5, solver=1)
    with PdSolver(body, params) as e:
        e.enable_kernel_timing(True)
        e.update(3)
        t = e.read_timing()
        info = e.factor_info()
        nbytes = e.solve_bytes()
        X, _ = e.download_state()
    assert t["solves"] == 15 and t["local_launches"] == 15
    assert 0 < t["solve_ms"] < t["step_ms"]
    n = body.num_verts
    assert nbytes == 2 * (8.0 * info["nnz_L"] + 4.0 * (n + 1)) + 48.0 * n
    Xo, _, _ = O.simulate(body, params, 3, precision=64)
    assert rel_l2(X, Xo) < TOL


@pytest.mark.parametrize("mode", [N.PDGB_SOLVE_CTA, N.PDGB_SOLVE_CLUSTER, N.PDGB_SOLVE_LEVELS, N.PDGB_SOLVE_DSM])
def test_solve_schedules_agree(mode):
    """The four schedules of the same factor (one CTA, one cluster, one
    launch per level, one cluster with everything in distributed shared
    memory) give the FP64 oracle's positions; tol > 0 keeps the early exit
    working in each."""
    body = mesh.make_grid_body(9, 8, 7, jitter=0.1, seed=13, young=3e4)
    params = SolverParams(num_iterations=10, tol=1e-4, solver=1)
    with PdSolver(body, params) as e:
        e.set_solve_mode(mode)
        its = []
        for _ in range(6):
            e.update(1)
            its.append(e.last_step_iterations())
        assert e.solve_mode() == mode
        X, _ = e.download_state()
    Xo, _, ito = O.simulate(body, params, 6, precision=64)
    assert rel_l2(X, Xo) < TOL
    assert np.abs(np.asarray(its) - ito).max() <= 1



def test_dsm_solve_matches_cluster_and_refines():
    """The on-chip solve of the 10^3 cube (the C1 system) against the
    cluster schedule, with FP64-residual refinement steps in both."""
    body = mesh.cube_c1()
    out = {}
    for mode in (N.PDGB_SOLVE_CLUSTER, N.PDGB_SOLVE_DSM):
        params = SolverParams(num_iterations=10, solver=1, refine_steps=1)
        with PdSolver(body, params) as e:
            e.set_solve_mode(mode)
            e.update(5)
            assert e.solve_mode() == mode
            out[mode] = e.download_state()[0]
    assert rel_l2(out[N.PDGB_SOLVE_DSM], out[N.PDGB_SOLVE_CLUSTER]) < 1e-6


def test_dsm_solve_refuses_a_factor_too_large():
    body = mesh.make_grid_body(30, 30, 30)
    with PdSolver(body, SolverParams(num_iterations=2, solver=1)) as e:
        e.set_solve_mode(N.PDGB_SOLVE_DSM)
        with pytest.raises(PdgbError):
            e.update(1)


@pytest.mark.parametrize("case", ["c1", "hetero14", "batch"])
def test_gpu_factor_matches_host_factor(case):
    """The one-time FP64 numeric factorisation on the GPU (default) and on the
    host give the same M_s blocks (both FP64, rounded to FP32: a few entries
    may differ in their last float bit) and the same steps."""
    if case == "c1":
        body = mesh.make_grid_body(10, 10, 10, young=1e5, poisson=0.4)
    elif case == "hetero14":
        body = mesh.cube_c3(n=14, seed=5)
    else:
        body = mesh.batch_c4(nbodies=9, seed=11, lo=2, hi=9)
    params = SolverParams(num_iterations=10, solver=1)
    out = {}
    for dev in (N.PDGB_FACTOR_GPU, N.PDGB_FACTOR_HOST):
        with PdSolver(body, params) as e:
            e.set_factor_device(dev)
            e.update(3)
            info = e.factor_info()
            assert info["numeric_device"] == dev
            out[dev] = (e.factor_blocks(), e.download_state()[0], info)
    Mg, Xg, ig = out[N.PDGB_FACTOR_GPU]
    Mh, Xh, ih = out[N.PDGB_FACTOR_HOST]
    assert Mg.shape == Mh.shape and ig["m_entries"] == ih["m_entries"]
    assert ig["numeric_ms"] > 0 and ig["pool_bytes"] > 0
    assert np.isfinite(Mg).all()
    scale = np.abs(Mh).max()
    assert np.abs(Mg - Mh).max() <= 1e-6 * scale, np.abs(Mg - Mh).max() / scale
    rel = np.abs(Mg.astype(np.float64) - Mh) / np.maximum(np.abs(Mh), 1e-30 * scale)
    assert (rel > 2.5e-7).mean() < 1e-3
    assert rel_l2(Xg, Xh) < 1e-6


def test_gpu_factor_reports_not_positive_definite():
    body = mesh.make_grid_body(2, 2, 2)
    body.mass = -np.abs(body.mass) * 1e9  # negative inertia term dominates
    params = SolverParams(num_iterations=4, solver=1)
    with PdSolver(body, params) as e:
        with pytest.raises(PdgbError) as err:
            e.update(1)
        assert err.value.status == N.PDGB_ERR_NOT_SPD


@pytest.mark.parametrize("name", ["c1_chol", "grid3_chol_tol", "grid3_chol"])
def test_dense_supernode_ordering_matches_fixture(name):
    """The factor stored as one dense supernode (PDGB_ORDER_DENSE, for small
    single bodies) gives the same steps: the reference's own kernels'
    fixtures, the FP64 oracle and the early-exit iteration counts."""
    body, params, steps, Xg, Vg, itg = load_golden(name)
    with PdSolver(body, params) as e:
        e.set_ordering(N.PDGB_ORDER_DENSE)
        its = []
        for _ in range(steps):
            e.update(1)
            its.append(e.last_step_iterations())
        X, _ = e.download_state()
        info = e.factor_info()
    assert info["num_supernodes"] == 1 and info["num_levels"] == 1
    assert info["m_entries"] == body.num_verts * body.num_verts
    assert np.isfinite(X).all()
    assert rel_l2(X, Xg) < TOL
    if params.tol > 0:
        d = np.abs(np.asarray(its) - itg)
        assert d.max() <= 1 and (d > 0).sum() <= max(1, steps // 10), (its, list(itg))
    Xo, _, _ = O.simulate(body, params, steps, precision=64)
    assert rel_l2(X, Xo) < TOL


@pytest.mark.parametrize("kind", [N.PDGB_LOCAL_TILE, N.PDGB_LOCAL_PIPELINED])
def test_local_step_forms_with_early_exit(kind):
    """Both forms of the local step under the Cholesky tolerance rule: once
    the device flag says the step has converged, the remaining local launches
    of the step return at once (the pipelined form after its first copies
    have landed), and positions and iteration counts follow the FP64 oracle."""
    body = mesh.make_grid_body(12, 10, 9, jitter=0.1, seed=21, young=3e4)
    params = SolverParams(num_iterations=10, tol=1e-4, solver=1)
    with PdSolver(body, params) as e:
        e.set_local_kernel(kind)
        its = []
        for _ in range(6):
            e.update(1)
            its.append(e.last_step_iterations())
        assert e.step_status() == N.PDGB_OK
        X, _ = e.download_state()
    Xo, _, ito = O.simulate(body, params, 6, precision=64)
    assert min(its) < 10, its  # the early exit engaged
    assert rel_l2(X, Xo) < TOL
    assert np.abs(np.asarray(its) - ito).max() <= 1
