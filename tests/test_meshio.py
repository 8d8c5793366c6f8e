"""Tet-mesh files: TetGen .node/.ele/.face and Gmsh 2.x .msh loading,
placement, surface extraction (pdgb_load_body_file, pdgb_surface_triangles).

Behaviour follows the reference's DataLoader (src/simulation/dataLoader.cu:
38-378).  Where the reference's own assets are present (this container),
the extracted surfaces are checked against the TetGen .face files that ship
with them."""
import struct
from pathlib import Path

import numpy as np
import pytest

from pdgb import PdgbError, mesh, meshio
from pdgb.build import reference_root

# the reference's asset files, where its sources are present (the root that
# oracle/_ref was built from, or $PDGB_REFERENCE_ROOT); the tests that read
# them skip elsewhere
_REF = reference_root()
REF_ASSETS = (_REF / "assets") if _REF is not None else Path("reference-assets-absent")


def write_tetgen(tmp: Path, body, start=1, faces=None, comments=False):
    node, ele = tmp / "b.node", tmp / "b.ele"
    with open(node, "w") as f:
        if comments:
            f.write("# a TetGen node file\n\n")
        f.write(f"{body.num_verts}  3  0  0\n")
        for i, p in enumerate(body.X):
            f.write(f"{i + start} {p[0]:.9g} {p[1]:.9g} {p[2]:.9g}\n")
    with open(ele, "w") as f:
        f.write(f"{body.num_tets}  4  0\n")
        for i, t in enumerate(body.tets):
            f.write(f"{i + start} {t[0] + start} {t[1] + start} {t[2] + start} {t[3] + start}\n")
        if comments:
            f.write("# generated\n")
    face = None
    if faces is not None:
        face = tmp / "b.face"
        with open(face, "w") as f:
            f.write(f"{len(faces)}  1\n")
            for i, t in enumerate(faces):
                f.write(f"{i + start} {t[0] + start} {t[1] + start} {t[2] + start} -1\n")
    return node, ele, face


def boundary_numpy(tets):
    """Faces (0,1,2), (0,2,3), (0,3,1), (1,3,2) of each tet used exactly once,
    ascending by sorted corners, oriented as the tet lists them."""
    count, orient = {}, {}
    for t in np.asarray(tets):
        for f in ((t[0], t[1], t[2]), (t[0], t[2], t[3]), (t[0], t[3], t[1]), (t[1], t[3], t[2])):
            k = tuple(sorted(int(v) for v in f))
            count[k] = count.get(k, 0) + 1
            orient[k] = tuple(int(v) for v in f)
    keys = sorted(k for k, c in count.items() if c % 2 == 1)
    return np.array([orient[k] for k in keys], dtype=np.uint32).reshape(-1, 3)


def test_tetgen_round_trip_and_surface(tmp_path):
    body = mesh.make_grid_body(4, 3, 5, jitter=0.1, seed=2)
    node, ele, _ = write_tetgen(tmp_path, body, comments=True)
    m = meshio.load_mesh(node, ele, start_index=1)
    assert np.array_equal(m["X"], body.X)
    assert np.array_equal(m["tets"], body.tets)
    ref = boundary_numpy(body.tets)
    assert np.array_equal(m["tris"], ref)
    assert np.array_equal(meshio.surface_triangles(body.tets), ref)
    # a 4x3x5 box has 2*(4*3 + 3*5 + 4*5) * 2 boundary triangles
    assert m["tris"].shape[0] == 4 * (12 + 15 + 20)
    # edges: distinct triangle edges, ascending
    e = {tuple(sorted((int(t[i]), int(t[(i + 1) % 3])))) for t in ref for i in range(3)}
    assert [tuple(r) for r in m["edges"]] == sorted(e)
    # start index -1: the first .node id is the base
    m2 = meshio.load_mesh(node, ele, start_index=-1)
    assert np.array_equal(m2["tets"], body.tets)


def test_surface_faces_point_into_their_tet():
    """Every extracted face (a, b, c) of a positively oriented mesh has its
    tet's fourth corner on the side of (b - a) x (c - a): the reference's
    render step flips the winding to face outward."""
    body = mesh.make_grid_body(3, 3, 3, jitter=0.15, seed=8)
    tris = meshio.surface_triangles(body.tets)
    X = body.X.astype(np.float64)
    owner = {}
    for t in body.tets:
        for f in ((0, 1, 2), (0, 2, 3), (0, 3, 1), (1, 3, 2)):
            k = tuple(sorted(int(t[i]) for i in f))
            owner.setdefault(k, []).append(int(sum(int(v) for v in t) - sum(int(t[i]) for i in f)))
    for a, b, c in tris:
        d = owner[tuple(sorted((int(a), int(b), int(c))))][0]
        n = np.cross(X[b] - X[a], X[c] - X[a])
        assert np.dot(n, X[d] - X[a]) > 0


def test_face_file_is_used_and_placement(tmp_path):
    body = mesh.make_grid_body(2, 2, 2, jitter=0.0)
    faces = boundary_numpy(body.tets)[::2]  # any list: the file wins over extraction
    node, ele, face = write_tetgen(tmp_path, body, faces=faces)
    m = meshio.load_mesh(node, ele, face, pos=(1.0, -2.0, 0.5), scale=(2.0, 3.0, 0.5), rot=(30.0, -45.0, 60.0),
                         start_index=1)
    assert np.array_equal(m["tris"], faces)

    def rot(axis, deg):
        a = np.radians(deg)
        c, s = np.cos(a), np.sin(a)
        R = np.eye(4)
        i, j = (axis + 1) % 3, (axis + 2) % 3
        R[i, i], R[j, j], R[j, i], R[i, j] = c, c, s, -s
        return R

    T = np.eye(4)
    T[:3, 3] = (1.0, -2.0, 0.5)
    M = T @ np.diag([2.0, 3.0, 0.5, 1.0]) @ rot(0, 30.0) @ rot(1, -45.0) @ rot(2, 60.0)
    Xh = np.c_[body.X.astype(np.float64), np.ones(body.num_verts)]
    Xr = (Xh @ M.T)[:, :3]
    assert np.abs(m["X"] - Xr).max() < 2e-6 * np.abs(Xr).max()


def test_centralize(tmp_path):
    body = mesh.make_grid_body(3, 2, 4, origin=(5.0, 1.0, -2.0), jitter=0.05, seed=1)
    node, ele, _ = write_tetgen(tmp_path, body)
    m = meshio.load_mesh(node, ele, centralize=True, start_index=1)
    Xc = body.X.astype(np.float64) - body.X.astype(np.float64).mean(axis=0)
    assert np.abs(m["X"] - Xc[:, [0, 2, 1]]).max() < 1e-5


def write_msh(path: Path, body, binary: bool, extra_tris=True):
    nv, nt = body.num_verts, body.num_tets
    tris = boundary_numpy(body.tets)[:5] if extra_tris else np.zeros((0, 3), np.uint32)
    with open(path, "wb") as f:
        f.write(b"$MeshFormat\n2.2 %d 8\n" % (1 if binary else 0))
        if binary:
            f.write(struct.pack("<i", 1) + b"\n")
        f.write(b"$EndMeshFormat\n$PhysicalNames\n1\n3 1 \"body\"\n$EndPhysicalNames\n")
        f.write(b"$Nodes\n%d\n" % nv)
        for i, p in enumerate(body.X.astype(np.float64)):
            if binary:
                f.write(struct.pack("<i3d", i + 1, *p))
            else:
                f.write(b"%d %.17g %.17g %.17g\n" % (i + 1, p[0], p[1], p[2]))
        if binary:
            f.write(b"\n")
        f.write(b"$EndNodes\n$Elements\n%d\n" % (nt + len(tris)))
        if binary:
            if len(tris):
                f.write(struct.pack("<3i", 2, len(tris), 2))
                for i, t in enumerate(tris):
                    f.write(struct.pack("<6i", i + 1, 1, 1, *(int(v) + 1 for v in t)))
            f.write(struct.pack("<3i", 4, nt, 2))
            for i, t in enumerate(body.tets):
                f.write(struct.pack("<7i", len(tris) + i + 1, 1, 1, *(int(v) + 1 for v in t)))
            f.write(b"\n")
        else:
            for i, t in enumerate(tris):
                f.write(b"%d 2 2 1 1 %d %d %d\n" % (i + 1, *(int(v) + 1 for v in t)))
            for i, t in enumerate(body.tets):
                f.write(b"%d 4 2 1 1 %d %d %d %d\n" % (len(tris) + i + 1, *(int(v) + 1 for v in t)))
        f.write(b"$EndElements\n$NodeData\n1\n\"t\"\n1\n0.0\n3\n0\n1\n1\n1 0.5\n$EndNodeData\n")


@pytest.mark.parametrize("binary", [False, True])
def test_gmsh(tmp_path, binary):
    body = mesh.make_grid_body(3, 3, 2, jitter=0.1, seed=4)
    path = tmp_path / ("b_bin.msh" if binary else "b.msh")
    write_msh(path, body, binary)
    m = meshio.load_mesh(msh_file=path, scale=(1.0, 1.0, 1.0))
    assert np.array_equal(m["X"], body.X)
    assert np.array_equal(m["tets"], body.tets)  # only the tetrahedra
    assert m["tris"].shape == (0, 3)


def test_load_errors(tmp_path):
    with pytest.raises(PdgbError):
        meshio.load_mesh(tmp_path / "missing.node", tmp_path / "missing.ele")
    body = mesh.make_grid_body(1, 1, 1)
    node, ele, _ = write_tetgen(tmp_path, body)
    with pytest.raises(PdgbError):
        meshio.load_mesh(node, ele, start_index=0)  # ids are 1-based: n is out of range
    (tmp_path / "bad.ele").write_text("3 4 0\n1 1 2 3 4\n")
    with pytest.raises(PdgbError):
        meshio.load_mesh(node, tmp_path / "bad.ele", start_index=1)  # fewer tets than declared
    with pytest.raises(PdgbError):
        meshio.load_mesh()


def test_scene_bodies(tmp_path):
    body = mesh.make_grid_body(2, 2, 2)
    write_tetgen(tmp_path, body)
    defs = {"box": {"nodeFile": "b.node", "eleFile": "b.ele", "start index": 1, "mass": 2.0, "mu": 500.0,
                    "scale": [1.0, 1.0, 1.0], "DBC": [0, 1]}}
    inst = [{"name": "box", "pos": [0.0, 3.0, 0.0]}, {"name": "box", "mu": 800.0, "DBC": [5]}]
    a, b = meshio.load_scene_bodies(inst, defs, tmp_path)
    assert np.allclose(a.X, body.X + np.float32([0, 3, 0]))
    assert (a.mass == 2.0).all() and (a.mu == 500.0).all() and list(np.nonzero(a.dbc)[0]) == [0, 1]
    assert (b.mu == 800.0).all() and list(np.nonzero(b.dbc)[0]) == [5]
    assert a.meta["tris"].shape[0] == 2 * 2 * 6 * 2


@pytest.mark.skipif(not REF_ASSETS.exists(), reason="reference assets not present")
@pytest.mark.parametrize("name,start", [("cube/cube.1", 1), ("sphere/sphere.1", 1), ("bunny/bunny.1", 1),
                                        ("armadillo0/armadillo0.1", 0)])
def test_reference_assets_surface_equals_face_file(name, start):
    base = REF_ASSETS / name
    node, ele, face = (Path(str(base) + s) for s in (".node", ".ele", ".face"))
    with_face = meshio.load_mesh(node, ele, face, start_index=start)
    extracted = meshio.load_mesh(node, ele, start_index=start)
    nv = int(node.read_text().split()[0])
    nt = int(ele.read_text().split()[0])
    assert with_face["X"].shape == (nv, 3) and with_face["tets"].shape == (nt, 4)
    s1 = {tuple(sorted(t)) for t in with_face["tris"].tolist()}
    s2 = {tuple(sorted(t)) for t in extracted["tris"].tolist()}
    assert s1 == s2 and len(s2) == extracted["tris"].shape[0]


@pytest.mark.skipif(not REF_ASSETS.exists(), reason="reference assets not present")
def test_reference_single_tet():
    """The scene's single tet (no face file; the .face beside it belongs to
    the cube): four boundary faces."""
    m = meshio.load_mesh(REF_ASSETS / "tet/tet.node", REF_ASSETS / "tet/tet.ele", start_index=1,
                         pos=(0.0, 10.0, 25.0), scale=(4.0, 4.0, 4.0))
    assert m["tets"].tolist() == [[3, 1, 0, 2]] and m["tris"].shape == (4, 3)
    assert np.allclose(m["X"][0], [4.0, 14.0, 21.0])


@pytest.mark.skipif(not REF_ASSETS.exists(), reason="reference assets not present")
def test_reference_scene_house_centralized():
    m = meshio.load_mesh(REF_ASSETS / "house2/house2.node", REF_ASSETS / "house2/house2.ele", centralize=True,
                         start_index=1, scale=(4.0, 4.0, 4.0))
    assert m["X"].shape == (400, 3) and m["tets"].shape == (1389, 4)
    assert np.abs(m["X"].mean(axis=0)).max() < 1e-4 * np.abs(m["X"]).max()
    assert m["tris"].shape[0] > 0
