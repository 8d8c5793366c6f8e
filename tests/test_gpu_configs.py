"""GPU parity at the sizes the bench reports, against the FP64 oracle.

Each workload of the bench is asserted at its own size here, with the same
1e-4 bar on vertex positions (relative L2) as the small golden cases:

  - the 64^3 jittered Jacobi + Chebyshev cube (274,625 v / 1,310,720 t),
    20 steps from rest: the accuracy point the bench reports (past ~25 steps
    this iteration diverges in FP64 as in FP32, the reference's code included);
  - the 40^3 heterogeneous Cholesky cube (per-tet E over three decades),
    3 steps with 0..3 FP64-residual refinement steps; refinement must not
    worsen the displacement error;
  - the 512-body batch with its own size law (dims 4..24 per axis): 16 of its
    bodies, the largest among them, against the same body alone and against
    the oracle;
  - served requests of mid and large size (3e4 and 3e5 tets) next to small
    ones, with the Jacobi and with the Cholesky global solve (factors
    computed on the GPU at admission, resident while the request runs): each
    result equals the body run alone and matches the oracle.

Reference iteration: PdSolver::SolverStep, pdSolver.cu:141-208.
"""
import math
import os
import time

import numpy as np
import pytest

from conftest import rel_l2

import oracle as O
from pdgb import PdServer, PdSolver, SolverParams, mesh
from pdgb import _native as N

pytestmark = pytest.mark.gpu

TOL = 1e-4
NTHREADS = os.cpu_count() or 1


def _disp_err(X, Xo, X0):
    return float(np.linalg.norm(X.astype(np.float64) - Xo) / max(np.linalg.norm(Xo - X0.astype(np.float64)), 1e-30))


def test_c2_full_grid_twenty_steps():
    body = mesh.cube_c2(64)
    assert (body.num_verts, body.num_tets) == (274625, 1310720)
    params = SolverParams(num_iterations=20, rho=0.9995, solver=0)
    with PdSolver(body, params) as e:
        e.update(20)
        assert e.step_status() == N.PDGB_OK
        X, _ = e.download_state()
    Xo, _, _ = O.simulate(body, params, 20, precision=64, nthreads=NTHREADS)
    assert np.isfinite(X).all()
    err = rel_l2(X, Xo)
    assert err < TOL, err
    # displacements: the FP32 iteration follows the FP64 one to ~5e-4 here
    assert _disp_err(X, Xo, body.X) < 2e-3


def test_c3_full_grid_refinement_counts():
    body = mesh.cube_c3(40)
    assert (body.num_verts, body.num_tets) == (68921, 320000)
    steps = 3
    base = SolverParams(num_iterations=10, solver=1)
    Xo, _, _ = O.simulate(body, base, steps, precision=64, nthreads=NTHREADS)
    disp = []
    for r in range(4):
        params = SolverParams(num_iterations=10, solver=1, refine_steps=r)
        with PdSolver(body, params) as e:
            e.update(steps)
            X, _ = e.download_state()
        assert np.isfinite(X).all()
        err = rel_l2(X, Xo)
        assert err < TOL, (r, err)
        disp.append(_disp_err(X, Xo, body.X))
    for r in range(1, 4):
        assert disp[r] <= disp[0] * 1.05, disp


def test_c4_batch_sample_vs_alone_and_oracle():
    bodies = mesh.batch_c4()
    assert len(bodies) == 512
    sizes = np.array([b.num_tets for b in bodies])
    largest = int(np.argmax(sizes))
    pick = sorted(set([largest] + list(range(0, 512, 34))))[:16]
    if largest not in pick:
        pick[-1] = largest
    assert len(pick) == 16 and largest in pick
    params = SolverParams(num_iterations=10, solver=1)
    steps = 5
    with PdSolver(bodies, params) as e:
        e.update(steps)
        got = {b: e.download_body(b)[0] for b in pick}
    for b in pick:
        body = bodies[b]
        with PdSolver(body, params) as s:
            s.update(steps)
            Xs, _ = s.download_state()
        assert rel_l2(got[b], Xs) < 1e-5, (b, rel_l2(got[b], Xs))
        Xo, _, _ = O.simulate(body, params, steps, precision=64, nthreads=NTHREADS)
        assert rel_l2(got[b], Xo) < TOL, (b, rel_l2(got[b], Xo))
    assert sizes[largest] >= 5 * 20 ** 3


@pytest.mark.parametrize("solver", [0, 1])
def test_c5_mid_and_large_requests_alone_vs_mix(solver):
    params = SolverParams(num_iterations=10, rho=0.9995, solver=solver)
    rng = np.random.default_rng(8)
    big = [mesh.request_body(3e4, rng), mesh.request_body(3e5, rng)]
    small = [mesh.request_body(math.exp(rng.uniform(math.log(1e3), math.log(1e4))), rng) for _ in range(6)]
    steps = {0: 24, 1: 16}
    with PdServer(params) as srv:
        ids = {}
        for i, b in enumerate(small[:3]):
            ids[("s", i)] = srv.submit(b, 12)
        srv.tick()
        ids[("b", 0)] = srv.submit(big[0], steps[0])
        srv.tick()
        ids[("b", 1)] = srv.submit(big[1], steps[1])
        for i, b in enumerate(small[3:]):
            ids[("s", i + 3)] = srv.submit(b, 12)
        # layouts are built by host workers: tick until every request is
        # settled, bounded in time
        deadline = time.monotonic() + 180.0
        while time.monotonic() < deadline:
            if all(srv.poll(r)[0] in (N.PDGB_REQ_DONE, N.PDGB_REQ_FAILED) for r in ids.values()):
                break
            active, _ = srv.tick()
            if active == 0:
                time.sleep(0.005)
        assert all(srv.poll(r)[0] == N.PDGB_REQ_DONE for r in ids.values())
        res = {k: srv.result(r)[0] for k, r in ids.items()}
    assert big[1].num_tets > 2e5 and 2e4 < big[0].num_tets < 4e4
    for k, X in res.items():
        body = big[k[1]] if k[0] == "b" else small[k[1]]
        n = steps[k[1]] if k[0] == "b" else 12
        with PdSolver(body, params) as e:
            e.update(n)
            Xa, _ = e.download_state()
        assert rel_l2(X, Xa) < 1e-5, (k, rel_l2(X, Xa))
        if k[0] == "b":
            Xo, _, _ = O.simulate(body, params, n, precision=64, nthreads=NTHREADS)
            assert rel_l2(X, Xo) < TOL, (k, rel_l2(X, Xo))
