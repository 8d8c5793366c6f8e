"""GPU parity of the scene terms behind the C ABI: interactive drag
(pdgb_drag_select / pdgb_set_drag / pdgb_set_drag_target) and fixed rigid
bodies (pdgb_set_fixed_bodies), against the reference's own kernels (golden
fixtures) and the FP64 oracle.  Bar: X and XTilde within 1e-4 relative L2."""
import numpy as np
import pytest

from conftest import SCENE_CASES, load_scene_golden, rel_l2, scene_fixed_bodies
from test_scene_oracle import oracle_replay

from pdgb import PdSolver, PdgbError, SolverParams, mesh
from pdgb import _native as N

pytestmark = pytest.mark.gpu

TOL = 1e-4


def engine_replay(body, params, steps, sc, solver_cls=PdSolver):
    with solver_cls(body, params) as e:
        fixed = scene_fixed_bodies(sc["fixed"])
        if fixed:
            e.set_fixed_bodies(fixed, sc["mu_t"], sc["mu_n"])
        if sc["select_v"] >= 0:
            e.set_drag_target(sc["target"])
        for k in range(steps):
            if sc["select_v"] >= 0 and (k == 0 or sc["reselect"]):
                e.drag_select(sc["select_v"])
            e.update(1)
        X, V = e.download_state()
        XT = e.download_xtilde()
    return X, V, XT


@pytest.mark.parametrize("name", SCENE_CASES)
def test_engine_matches_reference_scene(name):
    body, params, steps, Xg, Vg, sc = load_scene_golden(name)
    X, V, XT = engine_replay(body, params, steps, sc)
    assert np.isfinite(X).all() and np.isfinite(V).all()
    assert rel_l2(X, Xg) < TOL
    assert rel_l2(XT, sc["XT"]) < TOL
    assert rel_l2(V, Vg) < 5e-3
    Xo, Vo, XTo = oracle_replay(body, params, steps, sc, 64)
    assert rel_l2(X, Xo) < TOL
    assert rel_l2(XT, XTo) < TOL


def test_set_drag_arrays_equal_selection():
    """Caller-given weights/offsets (pdgb_set_drag) give the same step as the
    built-in selection."""
    import oracle as O

    body, params, steps, _, _, sc = load_scene_golden("drag_chol")
    w, off = O.drag_select(body.X, body.dbc, sc["select_v"])
    with PdSolver(body, params) as e:
        e.set_drag_target(sc["target"])
        e.set_drag(w, off)
        e.update(5)
        Xa, _ = e.download_state()
    with PdSolver(body, params) as e:
        e.set_drag_target(sc["target"])
        e.drag_select(sc["select_v"])
        e.update(5)
        Xb, _ = e.download_state()
    assert rel_l2(Xa, Xb) < 1e-6
    Xo, _, _, _ = O.simulate_scene(body, params, 5, 64, drag_w=w, drag_off=off, target=sc["target"])
    assert rel_l2(Xa, Xo) < TOL


def test_clear_drag_and_reset():
    body, params, _, _, _, sc = load_scene_golden("drag_jacobi")
    with PdSolver(body, params) as e:
        e.set_drag_target(sc["target"])
        e.drag_select(sc["select_v"])
        e.update(3)
        e.clear_drag()
        e.update(2)
        X1, V1 = e.download_state()
        e.reset()
        e.update(2)
        X2, _ = e.download_state()
    import oracle as O

    w, off = O.drag_select(body.X, body.dbc, sc["select_v"])
    Xa, Va, XTa, _ = O.simulate_scene(body, params, 3, 64, drag_w=w, drag_off=off, target=sc["target"])
    Xb, Vb, _, _ = O.simulate_scene(body, params, 2, 64, X=Xa, V=Va, XT=XTa)
    assert rel_l2(X1, Xb) < TOL
    Xr, _, _ = O.simulate(body, params, 2, 64)
    assert rel_l2(X2, Xr) < TOL  # reset clears the drag and restores X0


def test_drag_rejects_pinned_and_bad_vertex():
    body = mesh.make_grid_body(3, 3, 3)
    with PdSolver(body, SolverParams()) as e:
        w = np.zeros(body.num_verts, np.float32)
        w[np.argmax(body.dbc)] = 10.0
        with pytest.raises(PdgbError):
            e.set_drag(w)
        with pytest.raises(PdgbError):
            e.drag_select(body.num_verts)


def test_fixed_bodies_in_a_batch():
    """Fixed bodies apply to every body of a batch (one context)."""
    body, params, steps, _, _, sc = load_scene_golden("fixed_chol")
    shifted = mesh.SoftBody(X=body.X + np.float32([0.6, 0.0, 0.0]), tets=body.tets, mass=body.mass, mu=body.mu,
                            dbc=body.dbc)
    fixed = scene_fixed_bodies(sc["fixed"])
    with PdSolver([body, shifted], params) as e:
        e.set_fixed_bodies(fixed, sc["mu_t"], sc["mu_n"])
        e.update(20)
        Xa, _ = e.download_body(0)
        Xb, _ = e.download_body(1)
    import oracle as O

    for b, X in ((body, Xa), (shifted, Xb)):
        Xo, _, _, _ = O.simulate_scene(b, params, 20, 64, fixed=fixed, mu_t=sc["mu_t"], mu_n=sc["mu_n"])
        assert rel_l2(X, Xo) < TOL


def test_remove_fixed_bodies_keeps_xtilde():
    body, params, _, _, _, sc = load_scene_golden("fixed_jacobi")
    fixed = scene_fixed_bodies(sc["fixed"])
    with PdSolver(body, params) as e:
        e.set_fixed_bodies(fixed, sc["mu_t"], sc["mu_n"])
        e.update(40)
        e.set_fixed_bodies([], sc["mu_t"], sc["mu_n"])
        e.update(5)
        X, _ = e.download_state()
    import oracle as O

    Xa, Va, XTa, _ = O.simulate_scene(body, params, 40, 64, fixed=fixed, mu_t=sc["mu_t"], mu_n=sc["mu_n"])
    Xb, _, _, _ = O.simulate_scene(body, params, 5, 64, X=Xa, V=Va, XT=XTa)
    assert rel_l2(X, Xb) < TOL
