"""Serving loop on the GPU: continuous batching with admission by HBM budget.

Every request's result must equal the same body simulated alone by a single
engine (same kernels; only the float summation order of atomics across tiles
may differ) and match the FP64 oracle within the parity bar."""
import time

import numpy as np
import pytest

from conftest import rel_l2

import oracle as O
from pdgb import PdServer, PdSolver, SolverParams, mesh
from pdgb import _native as N

pytestmark = pytest.mark.gpu

PARAMS = SolverParams(num_iterations=12, rho=0.999, solver=0)


def _bodies():
    rng = np.random.default_rng(3)
    out = []
    for i in range(6):
        d = tuple(int(v) for v in rng.integers(2, 9, size=3))
        out.append((mesh.make_grid_body(*d, young=float(10 ** rng.uniform(4.5, 6.5)), jitter=0.1, seed=i,
                                        size=(0.1 * d[0], 0.1 * d[1], 0.1 * d[2])), int(rng.integers(2, 9))))
    return out


def _alone(body, steps):
    with PdSolver(body, PARAMS) as e:
        e.update(steps)
        return e.download_state()


def _drain(srv, ids, timeout_s=120.0):
    """Ticks until every request is done or failed (layouts and factors are
    prepared by host workers meanwhile), bounded in time."""
    deadline = time.monotonic() + timeout_s
    while time.monotonic() < deadline:
        if all(srv.poll(i)[0] in (N.PDGB_REQ_DONE, N.PDGB_REQ_FAILED) for i in ids):
            return
        active, _ = srv.tick()
        if active == 0:
            time.sleep(0.002)
    raise AssertionError("requests did not finish")


def test_results_equal_alone_and_oracle():
    reqs = _bodies()
    with PdServer(PARAMS) as srv:
        ids = [srv.submit(b, s) for b, s in reqs]
        _drain(srv, ids)
        for (body, steps), rid in zip(reqs, ids):
            assert srv.poll(rid) == (N.PDGB_REQ_DONE, steps)
            X, V = srv.result(rid)
            Xa, Va = _alone(body, steps)
            assert rel_l2(X, Xa) < 1e-5
            Xo, _, _ = O.simulate(body, PARAMS, steps, precision=64)
            assert rel_l2(X, Xo) < 1e-4
        st = srv.stats()
        assert st["completed"] == len(reqs) and st["active"] == 0 and st["bytes_in_use"] == 0
        assert len(srv.latencies_ms()) == len(reqs)


def test_admission_by_budget_and_late_arrivals():
    """A budget that holds about two requests: the rest wait and are admitted
    as memory frees up; requests submitted mid-flight join the next ticks."""
    reqs = _bodies()
    with PdServer(PARAMS, hbm_budget_bytes=1) as probe:  # too small for anything
        rid = probe.submit(*reqs[0])
        probe.tick()
        probe.tick()
    budget = 2 * 600_000
    with PdServer(PARAMS, hbm_budget_bytes=budget) as srv:
        ids = [srv.submit(b, s) for b, s in reqs[:3]]
        max_active = 0
        for _ in range(3):
            a, _ = srv.tick()
            max_active = max(max_active, a)
            assert srv.stats()["bytes_in_use"] <= budget
        ids += [srv.submit(b, s) for b, s in reqs[3:]]
        for _ in range(200):
            if all(srv.poll(i)[0] == N.PDGB_REQ_DONE for i in ids):
                break
            a, _ = srv.tick()
            max_active = max(max_active, a)
            assert srv.stats()["bytes_in_use"] <= budget
        for (body, steps), rid in zip(reqs, ids):
            X, _ = srv.result(rid)
            Xa, _ = _alone(body, steps)
            assert rel_l2(X, Xa) < 1e-5
    assert max_active >= 1


def test_slot_limit_and_bad_request():
    reqs = _bodies()
    bad = mesh.make_grid_body(2, 2, 2)
    bad.tets = bad.tets.copy()
    bad.tets[0, 1] = 999
    with PdServer(PARAMS, max_active=2) as srv:
        ids = [srv.submit(b, s) for b, s in reqs[:4]]
        bad_id = srv.submit(bad, 3)
        # the bad request fails in a layout worker, possibly after the good
        # ones have finished: tick until both are settled (bounded in time)
        deadline = time.monotonic() + 60.0
        while time.monotonic() < deadline:
            a, _ = srv.tick()
            assert a <= 2
            if (all(srv.poll(i)[0] == N.PDGB_REQ_DONE for i in ids)
                    and srv.poll(bad_id)[0] == N.PDGB_REQ_FAILED):
                break
            if a == 0:
                time.sleep(0.01)
        assert srv.poll(bad_id)[0] == N.PDGB_REQ_FAILED
        with pytest.raises(Exception):
            srv.result(bad_id)
        for (body, steps), rid in zip(reqs[:4], ids):
            X, _ = srv.result(rid)
            Xa, _ = _alone(body, steps)
            assert rel_l2(X, Xa) < 1e-5


def test_layout_cache_reuse():
    """The same mesh submitted again reuses the cached host layout; each
    request still gets its own device state and result."""
    body, _ = _bodies()[1]
    other, _ = _bodies()[2]
    with PdServer(PARAMS) as srv:
        first = srv.submit(body, 3)
        _drain(srv, [first])
        ids = [srv.submit(body, s) for s in (2, 5)] + [srv.submit(other, 4)]
        _drain(srv, ids)
        assert srv.stats()["layout_cache_hits"] >= 2
        for rid, b, s in zip([first] + ids, [body, body, body, other], [3, 2, 5, 4]):
            X, _ = srv.result(rid)
            Xa, _ = _alone(b, s)
            assert rel_l2(X, Xa) < 1e-5


CHOL = SolverParams(num_iterations=10, solver=1)


def _alone_with(body, steps, params):
    with PdSolver(body, params) as e:
        e.update(steps)
        return e.download_state()


def test_cholesky_requests_equal_alone_and_oracle():
    """Cholesky requests: each request's FP64 factor is computed on the GPU at
    admission and stays resident; the per-level solve launches cover every
    active request.  Results equal the engine alone and the FP64 oracle."""
    reqs = _bodies()
    with PdServer(CHOL) as srv:
        ids = [srv.submit(b, s) for b, s in reqs[:3]]
        srv.tick()
        ids += [srv.submit(b, s) for b, s in reqs[3:]]  # join while the others run
        _drain(srv, ids)
        for (body, steps), rid in zip(reqs, ids):
            assert srv.poll(rid) == (N.PDGB_REQ_DONE, steps)
            X, V = srv.result(rid)
            Xa, _ = _alone_with(body, steps, CHOL)
            assert rel_l2(X, Xa) < 1e-5
            Xo, _, _ = O.simulate(body, CHOL, steps, precision=64)
            assert rel_l2(X, Xo) < 1e-4
        st = srv.stats()
        assert st["completed"] == len(reqs) and st["active"] == 0 and st["bytes_in_use"] == 0
        assert st["factors"] == len(reqs) and st["factor_ms"] > 0


def test_cholesky_factor_cache_and_no_cache():
    """A mesh submitted again reuses its cached layout and numeric factor
    (uploaded, not recomputed); with the cache off every request factors."""
    body, _ = _bodies()[1]
    other, _ = _bodies()[4]
    for cache in (0, -1):
        with PdServer(CHOL, cache_entries=cache) as srv:
            first = srv.submit(body, 3)
            _drain(srv, [first])
            ids = [srv.submit(body, s) for s in (2, 5)] + [srv.submit(other, 4)]
            _drain(srv, ids)
            st = srv.stats()
            if cache == 0:
                assert st["factor_cache_hits"] >= 2 and st["factors"] == 2 and st["layout_cache_hits"] >= 2
            else:
                assert st["factor_cache_hits"] == 0 and st["factors"] == 4 and st["layout_cache_hits"] == 0
            for rid, b, s in zip([first] + ids, [body, body, body, other], [3, 2, 5, 4]):
                X, _ = srv.result(rid)
                Xa, _ = _alone_with(b, s, CHOL)
                assert rel_l2(X, Xa) < 1e-5


@pytest.mark.parametrize("solver", [0, 1])
def test_nonfinite_request_fails(solver):
    """A request whose state leaves the finite range (here a NaN initial
    velocity) fails with PDGB_ERR_NONFINITE instead of returning NaN; the
    requests beside it are unaffected."""
    params = PARAMS if solver == 0 else CHOL
    reqs = _bodies()[:3]
    bad, _ = _bodies()[3]
    bad.V = np.zeros_like(bad.X)
    bad.V[5, 1] = np.nan
    with PdServer(params) as srv:
        ids = [srv.submit(b, s) for b, s in reqs]
        bad_id = srv.submit(bad, 3)
        _drain(srv, ids + [bad_id])
        assert srv.poll(bad_id)[0] == N.PDGB_REQ_FAILED
        with pytest.raises(Exception) as err:
            srv.result(bad_id)
        assert getattr(err.value, "status", None) == N.PDGB_ERR_NONFINITE
        st = srv.stats()
        assert st["nonfinite"] == 1 and st["failed"] == 1 and st["completed"] == len(reqs)
        for (body, steps), rid in zip(reqs, ids):
            X, _ = srv.result(rid)
            Xa, _ = _alone_with(body, steps, params)
            assert rel_l2(X, Xa) < 1e-5
