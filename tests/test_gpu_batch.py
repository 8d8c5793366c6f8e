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
        # that motion, so the bound is relative or 2e-6 m rms, whichever is
        # larger.  The floor is float32 noise: the cross-tile float atomics add
        # in no fixed order, and repeated runs of this batch put the rms error
        # of its last body anywhere from 5.8e-7 to 1.08e-6 m (30 float32 ulp
        # at 1 m at most).
        d_err = float(np.linalg.norm(Xb - Xo) / np.sqrt(body.num_verts))
        disp = float(np.linalg.norm(Xo - body.X) / np.sqrt(body.num_verts))
        assert d_err < max(2e-3 * disp, 2e-6), (b, d_err, disp)


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


@pytest.mark.parametrize("case", ["batch", "c1", "hetero14"])
def test_persistent_solve_matches_per_level_launches(case):
    """The whole Cholesky solve in one persistent cooperative launch (levels
    separated by a bounded grid barrier) gives the per-level launches'
    result, and the FP64 oracle's, on a batch and on single bodies."""
    from pdgb import _native as N

    if case == "batch":
        bodies = mesh.batch_c4(nbodies=9, seed=11, lo=2, hi=9)
    elif case == "c1":
        bodies = mesh.make_grid_body(10, 10, 10, young=1e5, poisson=0.4)
    else:
        bodies = mesh.cube_c3(n=14, seed=5)
    params = SolverParams(num_iterations=10, solver=1)
    out = {}
    for mode in (N.PDGB_SOLVE_LEVELS, N.PDGB_SOLVE_PERSISTENT):
        with PdSolver(bodies, params) as e:
            e.set_solve_mode(mode)
            e.update(4)
            assert e.solve_mode() == mode
            assert e.step_status() == N.PDGB_OK
            out[mode] = e.download_state()[0]
    assert rel_l2(out[N.PDGB_SOLVE_PERSISTENT], out[N.PDGB_SOLVE_LEVELS]) < 1e-5
    for b, body in enumerate(bodies if isinstance(bodies, list) else [bodies]):
        Xo, _, _ = O.simulate(body, params, 4, precision=64)
        lo = sum(x.num_verts for x in bodies[:b]) if isinstance(bodies, list) else 0
        assert rel_l2(out[N.PDGB_SOLVE_PERSISTENT][lo:lo + body.num_verts], Xo) < TOL


def test_grid_barrier_wait_is_bounded():
    """The persistent solve's grid barrier on its own: it completes when every
    CTA arrives; when one arrival can never come (a participant that nothing
    provides), every wait gives up after its bound, the kernel returns with a
    timeout status and the context stays usable."""
    from pdgb import _native as N

    lib = N.lib()
    assert lib.pdgb_grid_sync_check(0, 20, 0, 1 << 24) == N.PDGB_OK
    assert lib.pdgb_grid_sync_check(64, 3, 1, 20000) == N.PDGB_ERR_TIMEOUT
    assert lib.pdgb_grid_sync_check(64, 3, 0, 1 << 24) == N.PDGB_OK
    assert lib.pdgb_grid_sync_check(0, 5, 0, 1 << 24) == N.PDGB_OK


@pytest.mark.gpu
def test_bulk_copy_wait_is_bounded():
    """The pipelined local step's bulk-copy wait on its own: a copy that
    completes its phase is waited for and its data is intact; a phase that
    expects bytes nobody copies makes the wait give up after its bound with
    PDGB_ERR_TIMEOUT, and the context stays usable."""
    from pdgb import _native as N

    lib = N.lib()
    assert lib.pdgb_bulk_wait_check(0, 1_000_000_000) == N.PDGB_OK
    assert lib.pdgb_bulk_wait_check(16, 2_000_000) == N.PDGB_ERR_TIMEOUT
    assert lib.pdgb_bulk_wait_check(0, 1_000_000_000) == N.PDGB_OK
    assert lib.pdgb_bulk_wait_check(8, 2_000_000) == N.PDGB_ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("solver", [0, 1])
def test_pipelined_local_step_on_a_batch(solver):
    """The pipelined local step on a batch, whose tiles are cut at body
    boundaries (short tiles, patch lists and tet ranges starting anywhere):
    the same states as the one-CTA-per-tile form, to the rounding of the
    cross-tile atomics, and the FP64 oracle per body."""
    from pdgb import _native as N

    bodies = mesh.batch_c4(nbodies=13, seed=5, lo=2, hi=9)
    params = SolverParams(num_iterations=10, rho=0.9995, solver=solver)
    out = {}
    for kind in (N.PDGB_LOCAL_TILE, N.PDGB_LOCAL_PIPELINED):
        with PdSolver(bodies, params) as e:
            e.set_local_kernel(kind)
            e.update(5)
            out[kind] = e.download_state()[0]
            assert e.step_status() == N.PDGB_OK
    assert rel_l2(out[N.PDGB_LOCAL_PIPELINED], out[N.PDGB_LOCAL_TILE]) < 1e-5
    lo = 0
    for body in bodies:
        Xo, _, _ = O.simulate(body, params, 5, precision=64)
        assert rel_l2(out[N.PDGB_LOCAL_PIPELINED][lo:lo + body.num_verts], Xo) < TOL
        lo += body.num_verts
