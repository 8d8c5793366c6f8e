"""Continuous collision between bodies on the GPU against the CPU oracle
(which is pinned to the reference's own query code): the standalone
detection on seeded scenes, and the engine's step with collision handling
on (detection on the engine's own X -> XTilde, the CCDKernel response)."""
import numpy as np
import pytest

from conftest import ccd_scene, rel_l2

import oracle as O
from pdgb import PdSolver, SolverParams, ccd_detect, mesh
from pdgb.meshio import surface_triangles

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,seed", [("drop", 0), ("drop", 3), ("shear", 1), ("shear", 4), ("apart", 2)])
def test_detection_matches_oracle(kind, seed):
    tris, tri_body, X, XT, _ = ccd_scene(kind, seed)
    tI, nrm, info = ccd_detect(tris, tri_body, X, XT)
    tIo, nrmo, (pairs, _, marked) = O.ccd_detect(tris, tri_body, X, XT)
    assert info["candidate_pairs"] == pairs
    assert info["vertices_hit"] == marked
    assert np.array_equal(tI, tIo)  # same IEEE operations: identical decisions
    assert np.abs(nrm - nrmo).max() <= 1e-6
    if kind != "apart":
        assert marked > 0


def test_detection_random_triangle_soup_matches_oracle():
    """Many small triangles of 4 bodies tumbling through each other."""
    rng = np.random.default_rng(8)
    nb, per = 4, 150
    cent = rng.uniform(-0.5, 0.5, (nb * per, 1, 3))
    X = (cent + rng.uniform(-0.06, 0.06, (nb * per, 3, 3))).reshape(-1, 3).astype(np.float32)
    XT = (X + rng.uniform(-0.08, 0.08, X.shape)).astype(np.float32)
    tris = np.arange(X.shape[0], dtype=np.uint32).reshape(-1, 3)
    body = np.repeat(np.arange(nb, dtype=np.int32), per)
    tI, nrm, info = ccd_detect(tris, body, X, XT)
    tIo, nrmo, (pairs, _, marked) = O.ccd_detect(tris, body, X, XT)
    assert info["candidate_pairs"] == pairs and pairs > 1000
    assert np.array_equal(tI, tIo) and marked > 10
    assert np.abs(nrm - nrmo).max() <= 1e-6


def _two_bodies():
    a = mesh.make_grid_body(6, 2, 6, size=(0.6, 0.2, 0.6), jitter=0.05, seed=1, pin="top")
    b = mesh.make_grid_body(3, 3, 3, size=(0.3, 0.3, 0.3), origin=(0.15, 0.21, 0.15), jitter=0.05, seed=2, pin=None)
    body = mesh.concat([a, b])
    tris = np.concatenate([surface_triangles(a.tets), surface_triangles(b.tets) + a.num_verts])
    tri_body = np.concatenate([np.zeros(len(tris) - len(surface_triangles(b.tets)), np.int32),
                               np.ones(len(surface_triangles(b.tets)), np.int32)])
    V = np.zeros_like(body.X)
    V[a.num_verts:] = (0.0, -6.0, 0.0)  # body b thrown down onto body a
    body.V = V
    return body, tris.astype(np.uint32), tri_body


@pytest.mark.parametrize("solver", [0, 1])
def test_engine_step_with_collision(solver):
    body, tris, tri_body = _two_bodies()
    params = SolverParams(num_iterations=10, rho=0.999, solver=solver)
    hits = 0
    with PdSolver(body, params) as e:
        e.set_collision_surface(tris, tri_body)
        e.enable_collision(True)
        for step in range(8):
            X0, V0 = e.download_state()
            e.update(1)
            X1, V1 = e.download_state()
            XT = e.download_xtilde()
            tI, nrm, info = e.collision()
            # detection on the engine's own X -> XTilde
            tIo, nrmo, (pairs, _, marked) = O.ccd_detect(tris, tri_body, X0, XT)
            assert info["candidate_pairs"] == pairs
            assert np.array_equal(tI, tIo), step
            assert np.abs(nrm - nrmo).max() <= 1e-6
            # response: colliding vertices keep X and get v = -(d.n) n
            Xr, Vr = O.ccd_response(tIo, nrmo, X0, XT, V1)
            hit = tI < 1.0
            assert np.array_equal(X1[hit], X0[hit]) and np.array_equal(X1[~hit], XT[~hit])
            assert np.allclose(V1[hit], Vr[hit], atol=1e-6)
            hits += int(hit.sum())
    assert hits > 0


def test_collision_surface_of_one_body_changes_nothing():
    body = mesh.make_grid_body(4, 3, 4, jitter=0.1, seed=3)
    tris = surface_triangles(body.tets)
    params = SolverParams(num_iterations=20, rho=0.9995, solver=0)
    with PdSolver(body, params) as e:
        e.update(5)
        Xa, Va = e.download_state()
    with PdSolver(body, params) as e:
        e.set_collision_surface(tris)  # one body: self-collision is ignored, as in the reference
        e.enable_collision(True)
        e.update(5)
        Xb, Vb = e.download_state()
        tI, _, info = e.collision()
    assert info["candidate_pairs"] == 0 and np.all(tI == 1.0)
    assert rel_l2(Xb, Xa) < 1e-6 and rel_l2(Vb, Va) < 1e-5
