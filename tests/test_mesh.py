"""Synthetic soft bodies: sizes, conformity, mass lumping, pinning."""
import numpy as np
import pytest

from pdgb import mesh


def test_c1_sizes_and_totals():
    b = mesh.cube_c1()
    assert (b.num_verts, b.num_tets) == (1331, 5000)
    assert abs(float(b.mass.astype(np.float64).sum()) - 1000.0) < 1e-2  # rho * 1 m^3
    assert int(b.dbc.sum()) == 121  # top face 11 x 11
    assert np.allclose(b.mu, 1e5 / (2 * 1.4))
    assert abs(mesh.tet_volumes(b.X, b.tets).sum() - 1.0) < 1e-9


def test_c2_c3_sizes_formula():
    for n, nv, nt in ((64, 274625, 1310720), (40, 68921, 320000)):
        assert (n + 1) ** 3 == nv and 5 * n ** 3 == nt


@pytest.mark.parametrize("dims", [(1, 1, 1), (2, 3, 2), (4, 4, 4)])
def test_grid_is_conforming_and_positive(dims):
    b = mesh.make_grid_body(*dims, jitter=0.1, seed=3)
    x = b.X.astype(np.float64)
    t = b.tets.astype(np.int64)
    det = np.einsum("ij,ij->i", np.cross(x[t[:, 1]] - x[t[:, 0]], x[t[:, 2]] - x[t[:, 0]]), x[t[:, 3]] - x[t[:, 0]])
    assert (det > 0).all()
    faces = np.sort(np.concatenate([t[:, [0, 1, 2]], t[:, [0, 1, 3]], t[:, [0, 2, 3]], t[:, [1, 2, 3]]]), axis=1)
    _, counts = np.unique(faces, axis=0, return_counts=True)
    assert counts.max() == 2  # every face shared by at most two tets
    nx, ny, nz = dims
    boundary_faces = 2 * 2 * (nx * ny + ny * nz + nx * nz)
    assert (counts == 1).sum() == boundary_faces


def test_c3_material_ranges():
    b = mesh.cube_c3(n=6, seed=3)
    E_over = b.mu * 2 * (1 + 0.3)
    assert b.mu.min() > 1e4 / (2 * 1.45) * 0.99 and b.mu.max() < 1e7 / (2 * 1.3) * 1.01
    assert E_over.size == 5 * 6 ** 3
