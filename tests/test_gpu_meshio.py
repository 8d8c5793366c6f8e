"""Bodies loaded from files step on the GPU exactly like generated ones, and
the render-side surface buffers (pdgb_render_surface) match the state."""
import numpy as np
import pytest

from conftest import rel_l2
from test_meshio import write_tetgen

import oracle as O
from pdgb import PdSolver, SolverParams, mesh, meshio

pytestmark = pytest.mark.gpu


def test_loaded_body_steps_like_the_oracle(tmp_path):
    src = mesh.make_grid_body(6, 5, 4, jitter=0.1, seed=12, young=5e4)
    node, ele, _ = write_tetgen(tmp_path, src)
    pinned = [int(i) for i in np.nonzero(src.dbc)[0]]
    body = meshio.load_body(node, ele, start_index=1, pos=(0.5, 1.0, 0.0), scale=(1.0, 1.0, 1.0),
                            rot=(0.0, 30.0, 0.0), mass=0.05, mu=2e4, dbc=pinned)
    for solver, iters in ((0, 20), (1, 10)):
        params = SolverParams(num_iterations=iters, rho=0.9995, solver=solver)
        with PdSolver(body, params) as e:
            e.update(20)
            X, _ = e.download_state()
        Xo, _, _ = O.simulate(body, params, 20, precision=64)
        assert rel_l2(X, Xo) < 1e-4
        assert rel_l2(X - body.X, Xo - body.X) < 2e-3


def test_render_surface_buffers(tmp_path):
    torch = pytest.importorskip("torch")
    src = mesh.make_grid_body(4, 4, 4, jitter=0.1, seed=3)
    node, ele, _ = write_tetgen(tmp_path, src)
    body = meshio.load_body(node, ele, start_index=1, scale=(1.0, 1.0, 1.0), dbc=np.nonzero(src.dbc)[0])
    tris = body.meta["tris"]
    n = tris.shape[0]
    bad = np.vstack([tris, [[0, 1, body.num_verts]]]).astype(np.uint32)  # last one out of range
    with PdSolver(body, SolverParams(num_iterations=10)) as e:
        e.update(5)
        X, _ = e.download_state()
        dev = torch.device("cuda")
        t = torch.from_numpy(bad.view(np.int32).copy()).to(dev)
        pos = torch.full(((n + 1) * 9,), 7.0, dtype=torch.float32, device=dev)
        nor = torch.full(((n + 1) * 12,), 7.0, dtype=torch.float32, device=dev)
        torch.cuda.synchronize()
        e.render_surface(t.data_ptr(), n + 1, pos.data_ptr(), nor.data_ptr())
        e.synchronize()
        P = pos.cpu().numpy().reshape(n + 1, 3, 3)
        Nn = nor.cpu().numpy().reshape(n + 1, 3, 4)
    want = X[tris[:, [0, 2, 1]]]
    assert np.array_equal(P[:n], want)
    X64 = want.astype(np.float64)
    cr = np.cross(X64[:, 1] - X64[:, 0], X64[:, 2] - X64[:, 0])
    cr /= np.linalg.norm(cr, axis=1, keepdims=True)
    assert np.abs(Nn[:n, :, :3] - cr[:, None, :]).max() < 1e-4
    assert (Nn[:n, :, 3] == 0).all()
    assert (P[n] == 0).all() and (Nn[n] == 0).all()
    # outward: normals point away from the body's centre on average
    c = X.mean(axis=0)
    assert (np.einsum("ij,ij->i", cr, X64.mean(axis=1) - c) > 0).mean() > 0.95
