"""Fixed rigid bodies of a scene, in the form the engine takes them.

The reference describes each fixed body in its scene file by type, position,
rotation (degrees about x, then y, then z) and scale or radius
(src/context.cpp:262-307), builds a glm model matrix from them
(utilityCore::modelMatrix, src/utilities.cpp:141-149) and keeps, per kind:
sphere -- centre (model translation) and radius; plane -- a point (model
translation) and the normal m_floorUp = normalize((model^-1)^T (0,1,0,0))
(src/collision/rigid/plane.cpp:9); cylinder -- centre, axis = the model's
second column normalised, radius = scale[0] (cylinder.cpp:9,
fixedBodyData.cu:116).  These helpers rebuild the same matrices in float32.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import _native as N

_DEG = np.float32(0.01745329251994329576923690768489)


@dataclass
class FixedBody:
    type: int                 # N.PDGB_FIXED_SPHERE / PLANE / CYLINDER
    model: np.ndarray         # (4, 4) float32, model[c] = column c (glm layout)
    radius: float = 1.0
    up: tuple = (0.0, 1.0, 0.0)

    def to_c(self) -> N.pdgb_fixed_body:
        fb = N.pdgb_fixed_body()
        fb.type = int(self.type)
        flat = np.ascontiguousarray(self.model, dtype=np.float32).reshape(16)
        for k in range(16):
            fb.model[k] = float(flat[k])
        fb.radius = float(self.radius)
        for k in range(3):
            fb.up[k] = float(self.up[k])
        return fb


def _rotate(m: np.ndarray, angle: np.float32, axis) -> np.ndarray:
    """m * R(angle, axis): rotation about a unit axis, Rodrigues form."""
    c, s = np.float32(np.cos(angle)), np.float32(np.sin(angle))
    a = np.asarray(axis, dtype=np.float32)
    a = a / np.float32(np.sqrt(np.dot(a, a)))
    t = (np.float32(1) - c) * a
    R = np.empty((3, 3), dtype=np.float32)  # R[col][row]
    R[0] = [c + t[0] * a[0], t[0] * a[1] + s * a[2], t[0] * a[2] - s * a[1]]
    R[1] = [t[1] * a[0] - s * a[2], c + t[1] * a[1], t[1] * a[2] + s * a[0]]
    R[2] = [t[2] * a[0] + s * a[1], t[2] * a[1] - s * a[0], c + t[2] * a[2]]
    out = m.copy()
    for j in range(3):
        out[j] = m[0] * R[j][0] + m[1] * R[j][1] + m[2] * R[j][2]
    return out


def model_matrix(pos, rot_deg=(0.0, 0.0, 0.0), scale=(1.0, 1.0, 1.0)) -> np.ndarray:
    """translate(pos) * rotate_x * rotate_y * rotate_z * scale, column-major
    (4, 4) float32 with model[3] = translation column."""
    m = np.eye(4, dtype=np.float32)
    p = np.asarray(pos, dtype=np.float32)
    m[3] = m[0] * p[0] + m[1] * p[1] + m[2] * p[2] + m[3]
    r = np.asarray(rot_deg, dtype=np.float32) * _DEG
    m = _rotate(m, r[0], (1.0, 0.0, 0.0))
    m = _rotate(m, r[1], (0.0, 1.0, 0.0))
    m = _rotate(m, r[2], (0.0, 0.0, 1.0))
    sc = np.asarray(scale, dtype=np.float32)
    out = m.copy()
    for j in range(3):
        out[j] = m[j] * sc[j]
    return out


def plane_up(model: np.ndarray) -> tuple:
    """normalize(vec3(transpose(inverse(model)) * (0, 1, 0, 0)))."""
    M = np.asarray(model, dtype=np.float64).T      # row-major matrix
    n = np.linalg.inv(M).T @ np.array([0.0, 1.0, 0.0, 0.0])
    n = n[:3] / np.linalg.norm(n[:3])
    return tuple(float(v) for v in n.astype(np.float32))


def sphere(pos, radius: float, rot_deg=(0.0, 0.0, 0.0)) -> FixedBody:
    r = float(radius)
    return FixedBody(N.PDGB_FIXED_SPHERE, model_matrix(pos, rot_deg, (r, r, r)), radius=r)


def plane(pos, rot_deg=(0.0, 0.0, 0.0), scale=(1.0, 1.0, 1.0)) -> FixedBody:
    m = model_matrix(pos, rot_deg, scale)
    return FixedBody(N.PDGB_FIXED_PLANE, m, up=plane_up(m))


def cylinder(pos, rot_deg=(0.0, 0.0, 0.0), scale=(1.0, 1.0, 1.0)) -> FixedBody:
    """scale = (radius, height, unused): the model is scaled (s0, s1, s0)."""
    s = np.asarray(scale, dtype=np.float32)
    return FixedBody(N.PDGB_FIXED_CYLINDER, model_matrix(pos, rot_deg, (s[0], s[1], s[0])), radius=float(s[0]))
