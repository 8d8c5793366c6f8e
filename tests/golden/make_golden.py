"""Generates the golden PD fixtures in this directory.

Each case runs the REFERENCE's own PD kernels (src/simulation/solver/
projective/pdUtil.cu, compiled for the CPU into oracle/_ref by
oracle/build_ref.sh) through its PdSolver step order, on a small seeded
synthetic body, and stores inputs and outputs:

  X0, tets, mass, mu, dbc        the system (SolverData<float> arrays)
  params                         dt, gravity, iterations, tol, rho, solver
  X, V                           state after `steps` steps
  iters                          local/global iterations run per step

Scene cases (drag_*, fixed_*) add the reference's interactive drag and
fixed rigid bodies (see make_scene_case).

Also `rotations.npz`: random deformation gradients (including inverted and
nearly flat ones) with the reference's rotation R = U V^T (svd.cuh:7-14 +
pdUtil.cu:113-122), and `ccd_queries.npz`: random continuous-collision
queries with the reference's contact times and normals
(src/collision/intersections.cu:286-334).

The reference's Cholesky branch calls cuSOLVER; the CPU harness solves the
same 3n x 3n system exactly in double instead.

Usage (needs the reference sources to build oracle/_ref):
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "soft-body-simulation-cuda_gb300"))
sys.path.insert(0, str(ROOT / "oracle"))

from pdgb import mesh  # noqa: E402
from pdgb.engine import SolverParams  # noqa: E402
import oracle as O  # noqa: E402

CASES = {
    # name: (body factory, params, steps)
    "tet1_jacobi": (lambda: mesh.single_tet(mass=0.5, mu=2e3),
                    SolverParams(num_iterations=20, rho=0.9992, solver=0), 40),
    "grid3_jacobi": (lambda: mesh.make_grid_body(3, 3, 3, young=1e5, poisson=0.4, jitter=0.1, seed=11),
                     SolverParams(num_iterations=20, rho=0.9995, solver=0), 30),
    "grid3_chol": (lambda: mesh.make_grid_body(3, 3, 3, young=1e5, poisson=0.4, jitter=0.1, seed=11),
                   SolverParams(num_iterations=10, solver=1), 30),
    "grid3_chol_tol": (lambda: mesh.make_grid_body(3, 3, 3, young=1e5, poisson=0.4, jitter=0.1, seed=11),
                       SolverParams(num_iterations=10, tol=2e-4, solver=1), 30),
    "grid435_soft_jacobi": (lambda: mesh.make_grid_body(4, 3, 5, young=2e4, poisson=0.3, jitter=0.15, seed=5,
                                                        size=(0.4, 0.3, 0.5)),
                            SolverParams(num_iterations=14, rho=0.999, solver=0), 40),
    "c1_chol": (mesh.cube_c1, SolverParams(num_iterations=10, solver=1), 10),
    "c1_jacobi": (mesh.cube_c1, SolverParams(num_iterations=20, rho=0.9995, solver=0), 10),
}


def _small_body(pin):
    # 6^3 cells of 2 cm: the reference's drag radius (sqrt(0.002) m) covers
    # a few dozen vertices
    return mesh.make_grid_body(6, 6, 6, size=(0.12, 0.12, 0.12), young=2e4, poisson=0.4, jitter=0.1, seed=21,
                               pin=pin)


def _falling_body():
    return mesh.make_grid_body(5, 5, 5, size=(0.5, 0.5, 0.5), origin=(0.0, 0.05, 0.0), young=1e5, poisson=0.4,
                               jitter=0.1, seed=4, pin=None)


# (type, pos, rot_deg, scale) as a scene file gives them; sphere radius = scale[0]
_FIXED = [(0, (0.25, -0.1, 0.25), (0.0, 0.0, 0.0), (0.12, 0.12, 0.12)),
          (1, (0.0, 0.0, 0.0), (5.0, 0.0, 3.0), (4.0, 4.0, 4.0)),
          (2, (0.25, 0.05, 0.25), (0.0, 0.0, 90.0), (0.05, 2.0, 0.05))]

SCENE_CASES = {
    # name: (body factory, params, steps, select_v, reselect, target offset from X[select_v], fixed, mu_t, mu_n)
    "drag_jacobi": (lambda: _small_body("top"), SolverParams(num_iterations=20, rho=0.9995, solver=0), 30,
                    0, True, (0.05, -0.04, 0.03), [], 0.5, 0.5),
    "drag_chol": (lambda: _small_body("top"), SolverParams(num_iterations=10, solver=1), 30,
                  0, True, (0.05, -0.04, 0.03), [], 0.5, 0.5),
    "drag_chol_nopin": (lambda: _small_body(None), SolverParams(num_iterations=10, solver=1), 20,
                        0, False, (0.02, 0.03, -0.01), [], 0.5, 0.5),
    "fixed_jacobi": (_falling_body, SolverParams(num_iterations=20, rho=0.9995, solver=0), 60,
                     -1, False, (0.0, 0.0, 0.0), _FIXED, 0.5, 0.3),
    "fixed_chol": (_falling_body, SolverParams(num_iterations=10, solver=1), 60,
                   -1, False, (0.0, 0.0, 0.0), _FIXED, 0.5, 0.3),
}


def make_scene_case(name: str) -> Path:
    """Drag (the reference's Control_Kernel selection, re-run before every
    step when `reselect`, as its mouse-move callback does) and fixed rigid
    bodies (FixedBodyData kernels after every step).  Adds to the case file:
    select_v, reselect, target, fixed (rows type, pos, rot, scale), mu_t,
    mu_n and XT (XTilde after the last step)."""
    factory, params, steps, sel, reselect, toff, fixed, mu_t, mu_n = SCENE_CASES[name]
    body = factory()
    target = (np.zeros(3, np.float32) if sel < 0 else body.X[sel] + np.asarray(toff, np.float32)).astype(np.float32)
    X, V, XT, iters = O.reference_simulate_scene(body, params, steps, select_v=sel, reselect=reselect,
                                                 target=target, fixed_specs=fixed, mu_t=mu_t, mu_n=mu_n)
    rows = np.array([[t, *pos, *rot, *sc] for (t, pos, rot, sc) in fixed], dtype=np.float32).reshape(-1, 10)
    out = HERE / f"{name}.npz"
    np.savez_compressed(
        out, X0=body.X, tets=body.tets, mass=body.mass, mu=body.mu, dbc=body.dbc,
        dt=np.float32(params.dt), gravity=np.float32(params.gravity), num_iterations=np.int32(params.num_iterations),
        tol=np.float32(params.tol), rho=np.float32(params.rho), solver=np.int32(params.solver),
        steps=np.int32(steps), X=X, V=V, iters=iters, XT=XT, select_v=np.int32(sel),
        reselect=np.int32(reselect), target=target, fixed=rows, mu_t=np.float32(mu_t), mu_n=np.float32(mu_n))
    return out


def make_case(name: str) -> Path:
    factory, params, steps = CASES[name]
    body = factory()
    X, V, iters = O.reference_simulate(body, params, steps)
    out = HERE / f"{name}.npz"
    np.savez_compressed(
        out, X0=body.X, tets=body.tets, mass=body.mass, mu=body.mu, dbc=body.dbc,
        dt=np.float32(params.dt), gravity=np.float32(params.gravity), num_iterations=np.int32(params.num_iterations),
        tol=np.float32(params.tol), rho=np.float32(params.rho), solver=np.int32(params.solver),
        steps=np.int32(steps), X=X, V=V, iters=iters)
    return out


def make_rotations() -> Path:
    rng = np.random.default_rng(7)
    n = 256
    F = []
    for k in range(n):
        Q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        if np.linalg.det(Q) < 0:
            Q[:, 0] = -Q[:, 0]
        W, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        s = np.exp(rng.uniform(-1.0, 1.0, size=3))
        if k % 8 == 3:
            s[2] = -s[2] * 0.3  # inverted
        if k % 16 == 7:
            s[2] = 1e-4        # nearly flat
        if k % 32 == 5:
            s = np.array([1.0, 1.0, 1.0]) + rng.uniform(-1e-3, 1e-3, 3)  # near-rotation
        F.append(Q @ np.diag(s) @ W.T)
    F = np.asarray(F, dtype=np.float32)
    R = O.reference_rotation(F)
    out = HERE / "rotations.npz"
    np.savez_compressed(out, F=F, R=R)
    return out


def make_ccd_queries() -> Path:
    """Random point-face and edge-edge continuous-collision queries (4 points
    moving from X to XT each) with the reference's own contact time and normal
    (ccdCollisionTest, intersections.cu:286-334).  About 1 in 14 collides."""
    rng = np.random.default_rng(17)
    q = 2048
    X = rng.uniform(-1.0, 1.0, (q, 4, 3)).astype(np.float32)
    D = (rng.uniform(-1.0, 1.0, (q, 4, 3)) * rng.uniform(0.2, 2.0, (q, 1, 1))).astype(np.float32)
    XT = (X + D).astype(np.float32)
    face = (np.arange(q) % 2).astype(np.int32)
    toi = np.empty(q, np.float32)
    nrm = np.empty((q, 3), np.float32)
    ids = np.arange(4, dtype=np.uint32)
    for k in range(q):
        toi[k], nrm[k] = O.reference_ccd_query(bool(face[k]), ids, X[k], XT[k])
    out = HERE / "ccd_queries.npz"
    np.savez_compressed(out, X=X, XT=XT, face=face, toi=toi, normal=nrm)
    return out


def main() -> None:
    if not O.reference_available():
        raise SystemExit("oracle/_ref/libref_pd.so is missing: build it with oracle/build_ref.sh")
    for name in CASES:
        p = make_case(name)
        print("wrote", p.relative_to(ROOT), p.stat().st_size, "bytes")
    for name in SCENE_CASES:
        p = make_scene_case(name)
        print("wrote", p.relative_to(ROOT), p.stat().st_size, "bytes")
    p = make_rotations()
    print("wrote", p.relative_to(ROOT), p.stat().st_size, "bytes")
    p = make_ccd_queries()
    print("wrote", p.relative_to(ROOT), p.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
