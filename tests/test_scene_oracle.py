"""Drag and fixed rigid bodies: the oracle against the reference's own
kernels (golden fixtures made by oracle/_ref), and the engine-side model
matrices against the reference's.

The reference applies drag inside the PD step (setMDt_2MoreDBC, computeSn,
computeDBCLocal, getErrorKern, updateVelPos; pdUtil.cu:56-205), selects the
dragged vertices with Control_Kernel (simulationContext.cu:201-231) and
projects XTilde out of fixed bodies after each step (fixedBodyData.cu:66-148,
pdSolver.cu:218-232).  Bar: positions, XTilde within 1e-4 relative L2."""
import numpy as np
import pytest

from conftest import SCENE_CASES, load_scene_golden, rel_l2, scene_fixed_bodies

import oracle as O

TOL = 1e-4


def oracle_replay(body, params, steps, sc, precision):
    """Step-by-step oracle run of a scene case: the drag selection before the
    first step (and before every step when reselect is set), then one step."""
    fixed = scene_fixed_bodies(sc["fixed"])
    X = body.X.astype(np.float32).copy()
    V = np.zeros_like(X)
    XT = X.copy()
    w = off = None
    for k in range(steps):
        if sc["select_v"] >= 0 and (k == 0 or sc["reselect"]):
            w, off = O.drag_select(X, body.dbc, sc["select_v"], offsets=off)
        X, V, XT, _ = O.simulate_scene(body, params, 1, precision, drag_w=w, drag_off=off, target=sc["target"],
                                       fixed=fixed, mu_t=sc["mu_t"], mu_n=sc["mu_n"], X=X, V=V, XT=XT)
    return X, V, XT


@pytest.mark.parametrize("name", SCENE_CASES)
@pytest.mark.parametrize("precision", [32, 64])
def test_oracle_matches_reference_scene(name, precision):
    body, params, steps, Xg, Vg, sc = load_scene_golden(name)
    X, V, XT = oracle_replay(body, params, steps, sc, precision)
    assert rel_l2(X, Xg) < TOL
    assert rel_l2(XT, sc["XT"]) < TOL
    assert rel_l2(V, Vg) < 5e-3
    # the scene terms matter: a plain run ends far away
    X0, _, _ = O.simulate(body, params, steps, precision=64)
    assert rel_l2(X0, Xg) > 100 * TOL


def test_scene_cases_exercise_the_terms():
    body, _, _, _, _, sc = load_scene_golden("drag_jacobi")
    w, _ = O.drag_select(body.X, body.dbc, sc["select_v"])
    assert (w > 0).sum() >= 8                       # a patch of vertices is dragged
    body, _, _, Xg, _, sc = load_scene_golden("fixed_chol")
    assert np.abs(sc["XT"] - Xg).max() > 1e-3       # the correction moved XTilde away from X
    assert {int(t) for t in sc["fixed"][:, 0]} == {0, 1, 2}


def test_drag_select_rules():
    X = np.array([[0, 0, 0], [0.01, 0, 0], [0.03, 0.03, 0], [0.02, 0, 0], [1, 1, 1]], np.float32)
    dbc = np.array([0, 0, 0, 1, 0], np.float32)
    w, off = O.drag_select(X, dbc, 0)
    # |d|^2: 0, 1e-4, 1.8e-3 (inside 0.002), pinned, 3
    assert list(w) == [10, 10, 10, 0, 0]
    assert np.allclose(off[4], [1, 1, 1]) and np.allclose(off[3], 0)
    w, _ = O.drag_select(X, dbc, -1)
    assert not w.any()


@pytest.mark.skipif(not O.reference_available(), reason="reference harness not built (no reference sources)")
@pytest.mark.parametrize("spec", [(0, (0.1, -0.5, 0.2), (0, 0, 0), (0.3, 0.3, 0.3)),
                                  (1, (0, -0.2, 0), (10, 20, 30), (4, 4, 4)),
                                  (1, (0.5, 0.0, -1.0), (0, 0, 0), (450, 450, 450)),
                                  (2, (0.5, 0.1, 0.5), (90, 0, 0), (0.2, 3, 0.2)),
                                  (2, (0.0, 10.0, 0.0), (90.0, 0.0, 0.0), (10.0, 75.0, 10.0))])
def test_model_matrices_match_reference(spec):
    """pdgb.scene rebuilds utilityCore::modelMatrix and Plane::m_floorUp."""
    from pdgb import scene

    t, pos, rot, sc = spec
    m_ref, up_ref = O.reference_fixed_frame(t, pos, rot, sc)
    body = scene_fixed_bodies(np.array([[t, *pos, *rot, *sc]], np.float32))[0]
    assert np.abs(body.model - m_ref).max() <= 1e-6 * max(1.0, np.abs(m_ref).max())
    if t == 1:
        assert np.abs(np.asarray(body.up) - up_ref).max() < 1e-6
    assert body.type == t
