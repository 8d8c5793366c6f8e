"""Continuous collision between bodies: the CPU oracle against the
reference's own query code (golden vectors from oracle/_ref, and live when
the reference is built here), plus the detection and response rules
(src/collision/*.cu, src/simulation/collisionUtil.cu:50-70,
src/simulation/solver/projective/pdSolver.cu:218-224)."""
import numpy as np
import pytest

from conftest import GOLDEN, ccd_scene

import oracle as O


def test_queries_match_reference_golden():
    z = np.load(GOLDEN / "ccd_queries.npz")
    ids = np.arange(4, dtype=np.uint32)
    hits = 0
    for k in range(z["toi"].size):
        t, n = O.ccd_query(bool(z["face"][k]), ids, z["X"][k], z["XT"][k])
        assert t == z["toi"][k], k  # bit-identical float arithmetic
        if t < 1.0:
            hits += 1
            assert np.array_equal(n, z["normal"][k]), k
    assert hits > 100


@pytest.mark.skipif(not O.reference_available(), reason="reference harness not built here")
def test_queries_match_reference_live():
    rng = np.random.default_rng(23)
    ids = np.arange(4, dtype=np.uint32)
    hits = 0
    for k in range(4000):
        X = rng.uniform(-1, 1, (4, 3)).astype(np.float32)
        XT = (X + rng.uniform(-1, 1, (4, 3)) * rng.uniform(0.1, 2.0)).astype(np.float32)
        t1, n1 = O.ccd_query(bool(k % 2), ids, X, XT)
        t2, n2 = O.reference_ccd_query(bool(k % 2), ids, X, XT)
        assert t1 == t2
        if t1 < 1.0:
            hits += 1
            assert np.array_equal(n1, n2)
    assert hits > 100


def test_point_through_face_and_crossing_edges():
    # a point moving straight down through a horizontal triangle at t = 0.5
    X = np.array([[0.2, 1.0, 0.2], [0, 0, 0], [1, 0, 0], [0, 0, 1]], np.float32)
    XT = X.copy()
    XT[0, 1] = -1.0
    t, n = O.ccd_query(True, np.arange(4, dtype=np.uint32), X, XT)
    assert abs(t - 0.5) < 1e-6
    assert abs(abs(n[1]) - 1.0) < 1e-6
    # two edges crossing: (x along, at y=1 moving down) vs (z along, at y=0)
    X = np.array([[-1, 1, 0.1], [1, 1, 0.1], [0.2, 0, -1], [0.2, 0, 1]], np.float32)
    XT = X.copy()
    XT[:2, 1] = -1.0
    t, n = O.ccd_query(False, np.arange(4, dtype=np.uint32), X, XT)
    assert abs(t - 0.5) < 1e-6
    # missing the face: no contact
    X = np.array([[3.0, 1.0, 3.0], [0, 0, 0], [1, 0, 0], [0, 0, 1]], np.float32)
    XT = X.copy()
    XT[0, 1] = -1.0
    t, _ = O.ccd_query(True, np.arange(4, dtype=np.uint32), X, XT)
    assert t == 1.0


def test_detection_marks_the_contact_region_only():
    tris, tri_body, X, XT, body = ccd_scene("drop")
    tI, nrm, (pairs, vf, marked) = O.ccd_detect(tris, tri_body, X, XT)
    assert pairs > 0 and marked > 0
    hit = tI < 1.0
    assert set(np.unique(tI)) <= {0.5, 1.0}
    # contacts happen where body 1's bottom meets body 0's top (y ~ 0.2):
    # marked vertices lie within one cell (0.1) of it, edge contacts marking
    # both ends of an edge
    assert np.all(np.abs(X[hit, 1] - 0.215) < 0.13)
    assert np.any(np.abs(X[hit, 1] - 0.215) < 0.03)
    assert np.allclose(np.linalg.norm(nrm[hit], axis=1), 1.0, atol=1e-5)
    assert np.all(nrm[~hit] == 0.0)
    # interior vertices (in no surface triangle) are never marked
    on_surface = np.zeros(X.shape[0], bool)
    on_surface[tris.reshape(-1)] = True
    assert not np.any(hit & ~on_surface)


def test_same_body_and_separating_bodies_give_no_contacts():
    tris, tri_body, X, XT, _ = ccd_scene("drop")
    tI, _, stats = O.ccd_detect(tris, np.zeros_like(tri_body), X, XT)  # one body: self-collision is ignored
    assert np.all(tI == 1.0) and stats[0] == 0
    tris, tri_body, X, XT, _ = ccd_scene("apart")
    tI, _, stats = O.ccd_detect(tris, tri_body, X, XT)
    assert np.all(tI == 1.0)


def test_response_keeps_colliding_vertices_and_reflects_normal_motion():
    tris, tri_body, X, XT, _ = ccd_scene("shear", seed=2)
    tI, nrm, _ = O.ccd_detect(tris, tri_body, X, XT)
    V = np.full_like(X, 7.0)
    Xn, Vn = O.ccd_response(tI, nrm, X, XT, V)
    hit = tI < 1.0
    assert hit.any() and (~hit).any()
    assert np.array_equal(Xn[hit], X[hit]) and np.array_equal(Xn[~hit], XT[~hit])
    d = (XT - X)[hit]
    vn = np.sum(d * nrm[hit], axis=1, keepdims=True) * nrm[hit]
    assert np.allclose(Vn[hit], -vn, atol=1e-6)
    assert np.all(Vn[~hit] == 7.0)
