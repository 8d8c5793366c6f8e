import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "soft-body-simulation-cuda_gb300", ROOT / "oracle"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds the engine, oracle (and reference harness if possible) once."""
    from pdgb import build as B

    B.build_all()
    yield


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def load_golden(name: str):
    from pdgb.mesh import SoftBody
    from pdgb.engine import SolverParams

    z = np.load(GOLDEN / f"{name}.npz")
    body = SoftBody(X=z["X0"], tets=z["tets"], mass=z["mass"], mu=z["mu"], dbc=z["dbc"])
    params = SolverParams(dt=float(z["dt"]), gravity=float(z["gravity"]), num_iterations=int(z["num_iterations"]),
                          tol=float(z["tol"]), rho=float(z["rho"]), solver=int(z["solver"]))
    return body, params, int(z["steps"]), z["X"], z["V"], z["iters"]


GOLDEN_CASES = ["tet1_jacobi", "grid3_jacobi", "grid3_chol", "grid3_chol_tol", "grid435_soft_jacobi", "c1_chol",
                "c1_jacobi"]


# Cases with the reference's interactive drag and fixed rigid bodies
# (tests/golden/make_golden.py, make_scene_case).
SCENE_CASES = ["drag_jacobi", "drag_chol", "drag_chol_nopin", "fixed_jacobi", "fixed_chol"]


def load_scene_golden(name: str):
    """(body, params, steps, X, V, scene) with scene = select_v, reselect,
    target, fixed (rows type, pos, rot, scale), mu_t, mu_n, XT."""
    body, params, steps, X, V, _ = load_golden(name)
    z = np.load(GOLDEN / f"{name}.npz")
    sc = {"select_v": int(z["select_v"]), "reselect": bool(z["reselect"]), "target": z["target"],
          "fixed": z["fixed"], "mu_t": float(z["mu_t"]), "mu_n": float(z["mu_n"]), "XT": z["XT"]}
    return body, params, steps, X, V, sc


def scene_fixed_bodies(rows):
    """Fixed bodies of a case, built as a scene file would (pdgb.scene)."""
    from pdgb import scene

    out = []
    for r in np.asarray(rows, np.float32).reshape(-1, 10):
        t, pos, rot, sc = int(r[0]), r[1:4], r[4:7], r[7:10]
        if t == 0:
            out.append(scene.sphere(pos, float(sc[0]), rot))
        elif t == 1:
            out.append(scene.plane(pos, rot, sc))
        else:
            out.append(scene.cylinder(pos, rot, sc))
    return out


def fan_body(n: int = 100, seed: int = 0):
    """Bicone of 2n tets around one centre vertex (valence 2n): a ring of n
    vertices, an apex above and below; the upper apex is pinned.  Used to
    exercise a vertex with more corners than one tile run holds."""
    from pdgb import mesh

    rng = np.random.default_rng(seed)
    ang = np.sort(rng.uniform(0.0, 2.0 * np.pi, n))
    rad = rng.uniform(0.8, 1.2, n)
    ring = np.stack([rad * np.cos(ang), rng.uniform(-0.05, 0.05, n), rad * np.sin(ang)], axis=1)
    X = np.concatenate([[[0.0, 0.0, 0.0]], ring, [[0.0, 1.0, 0.0], [0.0, -1.0, 0.0]]]).astype(np.float64)
    c, top, bot = 0, n + 1, n + 2
    tets = []
    for i in range(n):
        a, b = 1 + i, 1 + (i + 1) % n
        tets.append([c, a, b, top])
        tets.append([c, b, a, bot])
    tets = mesh.orient_positive(X, np.array(tets, np.uint32))
    mass = mesh.lumped_mass(X, tets, 1000.0)
    mu = np.full(tets.shape[0], mesh.lame_mu(1e5, 0.4), np.float32)
    dbc = np.zeros(X.shape[0], np.float32)
    dbc[top] = 1.0
    return mesh.SoftBody(X=X.astype(np.float32), tets=tets.astype(np.uint32), mass=mass.astype(np.float32), mu=mu,
                         dbc=dbc)


def ccd_scene(kind: str, seed: int = 0):
    """Two-body continuous-collision scenes: (tris [m, 3], tri_body [m], X,
    XT, bodies).  X are start positions, XT end positions of one step.
      "drop"  : body 1 (a 3x2x3-cell block) falls through the top of body 0
      "apart" : the same bodies moving away from each other
      "shear" : body 1 slides sideways across body 0 while sinking into it
    """
    from pdgb import mesh
    from pdgb.meshio import surface_triangles

    rng = np.random.default_rng(seed)
    a = mesh.make_grid_body(4, 2, 4, size=(0.4, 0.2, 0.4), jitter=0.05, seed=seed, pin=None)
    b = mesh.make_grid_body(3, 2, 3, size=(0.3, 0.2, 0.3), origin=(0.05, 0.23, 0.05), jitter=0.05,
                            seed=seed + 1, pin=None)
    body = mesh.concat([a, b])
    nva = a.num_verts
    tris = np.concatenate([surface_triangles(a.tets), surface_triangles(b.tets) + nva])
    tri_body = np.concatenate([np.zeros(len(surface_triangles(a.tets)), np.int32),
                               np.ones(len(surface_triangles(b.tets)), np.int32)])
    X = body.X.astype(np.float32)
    D = np.zeros_like(X)
    noise = rng.uniform(-0.004, 0.004, X.shape).astype(np.float32)
    if kind == "drop":
        D[nva:] = (0.0, -0.12, 0.0)
    elif kind == "apart":
        D[nva:] = (0.0, 0.12, 0.0)
        D[:nva] = (0.0, -0.05, 0.0)
    elif kind == "shear":
        D[nva:] = (0.15, -0.08, 0.05)
    else:
        raise ValueError(kind)
    XT = (X + D + noise).astype(np.float32)
    return tris.astype(np.uint32), tri_body, X, XT, body
