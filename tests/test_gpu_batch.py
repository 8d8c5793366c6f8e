"""GPU batches of independent bodies (one engine, per-body factors, one solve
launch per iteration with one CTA per body): every body's result equals the
same body simulated alone, and matches the FP64 oracle."""
import numpy as np
import pytest

from conftest import rel_l2

import oracle as O
from pdgb import PdSolver, SolverParams, mesh

pytestmark = pytest.mark.gpu

TOL = 1e-4


@pytest.mark.parametrize("solver", [0, 1])
def test_batch_equals_bodies_alone(solver):
    bodies = mesh.batch_c4(nbodies=9, seed=11, lo=2, hi=7)
    params = SolverParams(num_iterations=10 if solver else 20, rho=0.9995, solver=solver)
    with PdSolver(bodies, params) as e:
        e.update(6)
        batch = [e.download_body(b) for b in range(len(bodies))]
        Xall, _ = e.download_state()
    assert np.array_equal(np.concatenate([x for x, _ in batch]), Xall), "download_body != download_state slice"
    for b, body in enumerate(bodies):
        with PdSolver(body, params) as s:
            s.update(6)
            Xs, Vs = s.download_state()
        Xb, Vb = batch[b]
        # same arithmetic; only the float summation order of the tiles differs
        # (tiles and Morton keys of a body depend on the batch's bounding box)
        e_alone = rel_l2(Xb, Xs)
        assert e_alone < 1e-5, (b, e_alone)
        Xo, _, _ = O.simulate(body, params, 6, precision=64)
        assert rel_l2(Xb, Xo) < TOL, (b, rel_l2(Xb, Xo))
        # displacement diagnostic: stiff bodies placed ~1 m from the origin move
        # ~1e-4 m, and float32 rounding of the coordinates alone is ~1e-3 of
        # that motion, so the bound is relative or 1e-6 m rms, whichever is larger
        d_err = float(np.linalg.norm(Xb - Xo) / np.sqrt(body.num_verts))
        disp = float(np.linalg.norm(Xo - body.X) / np.sqrt(body.num_verts))
        assert d_err < max(2e-3 * disp, 1e-6), (b, d_err, disp)


def test_batch_uneven_sizes_cholesky():
    """Bodies from a handful of tets to ~10k tets in one batch."""
    sizes = [(1, 1, 1), (12, 10, 14), (2, 3, 2), (7, 7, 7), (1, 2, 1)]
    bodies = [mesh.make_grid_body(*d, young=1e5 * (i + 1), jitter=0.1, seed=i, size=(0.1 * d[0], 0.1 * d[1], 0.1 * d[2]))
              for i, d in enumerate(sizes)]
    params = SolverParams(num_iterations=10, solver=1)
    with PdSolver(bodies, params) as e:
        e.update(4)
        for b, body in enumerate(bodies):
            Xb, _ = e.download_body(b)
            Xo, _, _ = O.simulate(body, params, 4, precision=64)
            assert rel_l2(Xb, Xo) < TOL, b


def test_batch_solve_schedules():
    """One cluster of CTAs per body (PDGB_SOLVE_CLUSTER) and one launch per
    level across all bodies (PDGB_SOLVE_LEVELS) give the same bodies as one
    CTA per body."""
    from pdgb import _native as N

    bodies = mesh.batch_c4(nbodies=7, seed=17, lo=3, hi=9)
    params = SolverParams(num_iterations=10, solver=1)
    out = {}
    for mode in (N.PDGB_SOLVE_CTA, N.PDGB_SOLVE_CLUSTER, N.PDGB_SOLVE_LEVELS):
        with PdSolver(bodies, params) as e:
            e.set_solve_mode(mode)
            e.update(4)
            out[mode] = e.download_state()[0]
            assert e.solve_mode() == mode
    assert rel_l2(out[N.PDGB_SOLVE_CLUSTER], out[N.PDGB_SOLVE_CTA]) < 1e-5
    assert rel_l2(out[N.PDGB_SOLVE_LEVELS], out[N.PDGB_SOLVE_CTA]) < 1e-5
    for b, body in enumerate(bodies):
        Xo, _, _ = O.simulate(body, params, 4, precision=64)
        lo = sum(x.num_verts for x in bodies[:b])
        for mode in (N.PDGB_SOLVE_CLUSTER, N.PDGB_SOLVE_LEVELS):
            assert rel_l2(out[mode][lo:lo + body.num_verts], Xo) < TOL
