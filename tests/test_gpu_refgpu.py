"""The restated reference GPU path (baseline/refgpu.cu: the reference's
PdSolver kernels with cuSOLVER's FP32 sparse Cholesky), checked against the
golden fixtures made by the reference's own kernels, before bench.py times it
beside the engine.  A baseline that computed something else would be no
baseline."""
import sys

import numpy as np
import pytest

from conftest import GOLDEN_CASES, ROOT, load_golden, rel_l2

import oracle as O
from pdgb import PdSolver, SolverParams, mesh

sys.path.insert(0, str(ROOT / "baseline"))
import refgpu  # noqa: E402

pytestmark = pytest.mark.gpu

TOL = 1e-4


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from pdgb import build as B

    B.build_refgpu()
    yield


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_reference_path_matches_reference_fixture(name):
    body, params, steps, Xg, Vg, itg = load_golden(name)
    with refgpu.ReferenceGpuPath(body, params) as r:
        its = []
        for _ in range(steps):
            its.append(r.step(1)[1])
        X, V = r.state()
    err = rel_l2(X, Xg)
    print(f"{name}: rel L2 vs the reference's kernels {err:.3e}")
    assert np.isfinite(X).all() and np.isfinite(V).all()
    assert err < TOL
    if params.tol > 0:
        d = np.abs(np.asarray(its) - itg)
        assert d.max() <= 1 and (d > 0).sum() <= max(1, steps // 10), (its, list(itg))
    else:
        assert all(i == params.num_iterations for i in its)


@pytest.mark.parametrize("solver", [0, 1])
def test_reference_path_and_engine_agree(solver):
    """Same jittered body, same parameters: the restated reference path and
    the engine end within the parity bar of each other and of the FP64
    oracle."""
    body = mesh.make_grid_body(8, 8, 8, young=1e5, poisson=0.4, jitter=0.1, seed=11)
    params = SolverParams(num_iterations=20 if solver == 0 else 10, rho=0.9995, solver=solver)
    steps = 15
    with refgpu.ReferenceGpuPath(body, params) as r:
        r.step(steps)
        Xr, _ = r.state()
        nnz = r.system_nnz()
    with PdSolver(body, params) as e:
        e.update(steps)
        Xe, _ = e.download_state()
    Xo, _, _ = O.simulate(body, params, steps, precision=64)
    print(f"solver {solver}: ref vs fp64 {rel_l2(Xr, Xo):.3e}, engine vs fp64 {rel_l2(Xe, Xo):.3e}, nnz {nnz}")
    assert (nnz > 9 * body.num_verts) == (solver == 1)
    assert rel_l2(Xr, Xo) < TOL
    assert rel_l2(Xe, Xr) < TOL
