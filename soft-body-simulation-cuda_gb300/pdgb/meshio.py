"""Soft bodies from tet-mesh files (TetGen .node/.ele/.face, Gmsh 2.x .msh).

``load_body`` mirrors what the reference's scene loading does for one soft
body (SimulationCUDAContext::Impl::Init, simulationContext.cu:60-104, and
DataLoader::CollectData / AllocData, dataLoader.cu:202-378): read and place
the mesh (native, ``pdgb_load_body_file``), give every vertex the body's
constant ``mass`` and every tet its ``mu`` (the PD weight), and pin the
vertices listed in ``dbc``.  ``load_scene_bodies`` resolves per-instance
values against body definitions the way the scene file's "softBodies" block
does (instance value, else definition value, else the default).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import _native as N
from .mesh import SoftBody


def _cstr(p) -> bytes | None:
    return None if p is None or p == "" else str(p).encode()


def load_mesh(node_file=None, ele_file=None, face_file=None, msh_file=None, pos=(0.0, 0.0, 0.0),
              scale=(1.0, 1.0, 1.0), rot=(0.0, 0.0, 0.0), centralize: bool = False, start_index: int = 0) -> dict:
    """Placed mesh arrays: X (nv, 3) float32, tets (nt, 4), tris (ntri, 3),
    edges (ne, 2) uint32."""
    lib = N.lib()
    f = N.pdgb_body_file()
    f.node_file, f.ele_file, f.face_file, f.msh_file = (_cstr(node_file), _cstr(ele_file), _cstr(face_file),
                                                        _cstr(msh_file))
    for d in range(3):
        f.pos[d], f.scale[d], f.rot[d] = float(pos[d]), float(scale[d]), float(rot[d])
    f.centralize = int(bool(centralize))
    f.start_index = int(start_index)
    out = C.POINTER(N.pdgb_tet_mesh)()
    N.check(lib.pdgb_load_body_file(C.byref(f), C.byref(out)), "pdgb_load_body_file")
    try:
        m = out.contents

        def arr(ptr, n, k, dt):
            if n == 0:
                return np.zeros((0, k), dtype=dt)
            return np.ctypeslib.as_array(ptr, shape=(n * k,)).astype(dt, copy=True).reshape(n, k)

        return {"X": arr(m.X, m.num_verts, 3, np.float32), "tets": arr(m.tets, m.num_tets, 4, np.uint32),
                "tris": arr(m.tris, m.num_tris, 3, np.uint32), "edges": arr(m.edges, m.num_edges, 2, np.uint32)}
    finally:
        lib.pdgb_free_tet_mesh(out)


def load_body(node_file=None, ele_file=None, face_file=None, msh_file=None, pos=(0.0, 0.0, 0.0),
              scale=(1.0, 1.0, 1.0), rot=(0.0, 0.0, 0.0), centralize: bool = False, start_index: int = 0,
              mass: float = 1.0, mu: float = 1000.0, dbc=()) -> SoftBody:
    """A SoftBody from files; defaults are the scene file's (mass 1, mu 1000)."""
    m = load_mesh(node_file, ele_file, face_file, msh_file, pos, scale, rot, centralize, start_index)
    nv, nt = m["X"].shape[0], m["tets"].shape[0]
    pins = np.zeros(nv, np.float32)
    idx = np.asarray(list(dbc), dtype=np.int64)
    if idx.size and (idx.min() < 0 or idx.max() >= nv):
        raise ValueError("DBC vertex index out of range")
    pins[idx] = 1.0
    return SoftBody(X=m["X"], tets=m["tets"], mass=np.full(nv, mass, np.float32), mu=np.full(nt, mu, np.float32),
                    dbc=pins, meta={"tris": m["tris"], "edges": m["edges"]})


def surface_triangles(tets: np.ndarray) -> np.ndarray:
    """Boundary triangles of a tet list (faces used by exactly one tet)."""
    t = np.ascontiguousarray(tets, dtype=np.uint32).reshape(-1, 4)
    lib = N.lib()
    cap = 4 * t.shape[0]
    out = np.empty((max(cap, 1), 3), np.uint32)
    n = C.c_int(0)
    N.check(lib.pdgb_surface_triangles(t.shape[0], t.ctypes.data, out.ctypes.data, cap, C.byref(n)),
            "pdgb_surface_triangles")
    return out[: n.value].copy()


_VEC_KEYS = ("pos", "scale", "rot")


def load_scene_bodies(instances: list, definitions: dict, base_dir=".") -> list:
    """Bodies of a scene's "softBodies" list.  Each instance names a
    definition; pos/scale/rot/mass/mu/DBC come from the instance, else the
    definition, else the defaults (vectors 0, mass 1, mu 1000); files,
    "centralize" and "start index" come from the definition."""
    base = Path(base_dir)
    out = []
    for inst in instances:
        d = definitions[inst["name"]]

        def pick(key, default):
            return inst[key] if key in inst else d.get(key, default)

        vec = {k: tuple(float(v) for v in pick(k, (0.0, 0.0, 0.0))) for k in _VEC_KEYS}
        files = {k: (str(base / d[k]) if d.get(k) else None) for k in ("nodeFile", "eleFile", "faceFile", "mshFile")}
        dbc = pick("DBC", None) or ()
        out.append(load_body(node_file=None if files["mshFile"] else files["nodeFile"],
                             ele_file=files["eleFile"], face_file=files["faceFile"], msh_file=files["mshFile"],
                             pos=vec["pos"], scale=vec["scale"], rot=vec["rot"],
                             centralize=bool(d.get("centralize", False)), start_index=int(d.get("start index", 0)),
                             mass=float(pick("mass", 1.0)), mu=float(pick("mu", 1000.0)), dbc=dbc))
    return out
