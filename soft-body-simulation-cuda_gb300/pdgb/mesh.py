"""Synthetic soft bodies: hex grids split into 5 tets per cell.

A system is the data the reference's ``SolverData<float>`` holds for PD
(def.h:21-56): positions X (rest = X0), tets, per-vertex mass, per-tet PD
weight ``mu`` and per-vertex pin flags ``DBC``.  The reference fills them
from TetGen files (dataLoader.cu:291-378); the synthetic bodies here are
generated directly.

Cell split: each hex cell is cut into 5 tets (4 corner tets + 1 central);
cells alternate the cut by the parity of (i + j + k) so that neighbouring
cells share face diagonals (a conforming mesh).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

# Corner (i, j, k) offsets of a hex cell and its 5-tet split for even cells;
# odd cells use the mirrored split.  Tets are listed by corner numbers
# c = i + 2 j + 4 k.
_EVEN = [(1, 0, 3, 5), (2, 0, 3, 6), (4, 0, 5, 6), (7, 3, 6, 5), (0, 3, 5, 6)]
_ODD = [(0, 1, 2, 4), (3, 1, 2, 7), (5, 1, 4, 7), (6, 2, 4, 7), (1, 2, 4, 7)]


@dataclass
class SoftBody:
    X: np.ndarray            # (nv, 3) float32 positions (also the rest shape)
    tets: np.ndarray         # (nt, 4) uint32
    mass: np.ndarray         # (nv,) float32
    mu: np.ndarray           # (nt,) float32 PD weight
    dbc: np.ndarray          # (nv,) float32 pin flags 0/1
    V: np.ndarray | None = None
    meta: dict = field(default_factory=dict)

    @property
    def num_verts(self) -> int:
        return int(self.X.shape[0])

    @property
    def num_tets(self) -> int:
        return int(self.tets.shape[0])


def grid_tets(nx: int, ny: int, nz: int) -> np.ndarray:
    """Tets of an nx x ny x nz hex grid, vertex id = i + (nx+1)(j + (ny+1) k)."""
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    i, j, k = i.ravel(order="F"), j.ravel(order="F"), k.ravel(order="F")
    sx, sy = nx + 1, (nx + 1) * (ny + 1)
    corners = np.stack([(i + di) + sx * (j + dj) + sy * (k + dk)
                        for dk in (0, 1) for dj in (0, 1) for di in (0, 1)], axis=1)  # c = di + 2dj + 4dk
    odd = ((i + j + k) & 1).astype(bool)
    out = np.empty((corners.shape[0], 5, 4), dtype=np.int64)
    for t, (ev, od) in enumerate(zip(_EVEN, _ODD)):
        out[:, t, :] = np.where(odd[:, None], corners[:, list(od)], corners[:, list(ev)])
    return out.reshape(-1, 4).astype(np.uint32)


def grid_positions(nx: int, ny: int, nz: int, size=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0)) -> np.ndarray:
    xs = origin[0] + np.linspace(0.0, size[0], nx + 1)
    ys = origin[1] + np.linspace(0.0, size[1], ny + 1)
    zs = origin[2] + np.linspace(0.0, size[2], nz + 1)
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)


def orient_positive(X: np.ndarray, tets: np.ndarray) -> np.ndarray:
    """Swaps two corners of every tet with negative signed volume."""
    x = X.astype(np.float64)
    d = np.einsum("ij,ij->i", np.cross(x[tets[:, 1]] - x[tets[:, 0]], x[tets[:, 2]] - x[tets[:, 0]]),
                  x[tets[:, 3]] - x[tets[:, 0]])
    out = tets.copy()
    neg = d < 0
    out[neg, 2], out[neg, 3] = tets[neg, 3], tets[neg, 2]
    return out


def tet_volumes(X: np.ndarray, tets: np.ndarray) -> np.ndarray:
    x = X.astype(np.float64)
    d = np.einsum("ij,ij->i", np.cross(x[tets[:, 1]] - x[tets[:, 0]], x[tets[:, 2]] - x[tets[:, 0]]),
                  x[tets[:, 3]] - x[tets[:, 0]])
    return np.abs(d) / 6.0


def lumped_mass(X: np.ndarray, tets: np.ndarray, density) -> np.ndarray:
    """rho V_t / 4 to each corner; density scalar or per tet."""
    vol = tet_volumes(X, tets) * np.broadcast_to(np.asarray(density, dtype=np.float64), (tets.shape[0],))
    m = np.zeros(X.shape[0], dtype=np.float64)
    for c in range(4):
        np.add.at(m, tets[:, c], vol / 4.0)
    return m


def lame_mu(E, nu):
    return np.asarray(E, dtype=np.float64) / (2.0 * (1.0 + np.asarray(nu, dtype=np.float64)))


def make_grid_body(nx: int, ny: int, nz: int, *, size=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0),
                   young=1e5, poisson=0.4, density=1000.0, jitter=0.0, seed=0,
                   pin="top") -> SoftBody:
    """Hex-grid soft body.

    young/poisson: scalars or per-tet arrays; the PD weight is mu = E/(2(1+nu)).
    jitter: uniform displacement of every vertex in [-jitter, jitter] cells per axis.
    pin: "top" pins the y = max face (reference DBC flags), None pins nothing.
    """
    X = grid_positions(nx, ny, nz, size, origin)
    rng = np.random.default_rng(seed)
    if jitter > 0.0:
        cell = np.array([size[0] / nx, size[1] / ny, size[2] / nz])
        X = X + rng.uniform(-jitter, jitter, size=X.shape) * cell
    tets = orient_positive(X, grid_tets(nx, ny, nz))
    nt = tets.shape[0]
    E = np.broadcast_to(np.asarray(young, dtype=np.float64), (nt,))
    nu = np.broadcast_to(np.asarray(poisson, dtype=np.float64), (nt,))
    mass = lumped_mass(X, tets, density)
    dbc = np.zeros(X.shape[0], dtype=np.float32)
    if pin == "top":
        j = (np.arange(X.shape[0]) // (nx + 1)) % (ny + 1)
        dbc[j == ny] = 1.0
    elif pin is not None:
        raise ValueError(f"unknown pin mode {pin!r}")
    return SoftBody(X=X.astype(np.float32), tets=tets.astype(np.uint32), mass=mass.astype(np.float32),
                    mu=lame_mu(E, nu).astype(np.float32), dbc=dbc,
                    meta={"dims": (nx, ny, nz), "size": size, "jitter": jitter, "seed": seed})


def single_tet(mass=1.0, mu=1e4) -> SoftBody:
    X = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=np.float32)
    tets = np.array([[0, 1, 2, 3]], dtype=np.uint32)
    return SoftBody(X=X, tets=tets, mass=np.full(4, mass, np.float32), mu=np.array([mu], np.float32),
                    dbc=np.array([0, 0, 1, 0], np.float32))


# ---------------------------------------------------------------- workloads
# Named configurations (sizes, materials and step counts).
def cube_c1() -> SoftBody:
    """1 m cube, 10^3 cells (1,331 verts / 5,000 tets), E=1e5, nu=0.4, rho=1000, top face pinned."""
    return make_grid_body(10, 10, 10, young=1e5, poisson=0.4, density=1000.0)


def cube_c2(n: int = 64, seed: int = 2024) -> SoftBody:
    """1 m cube, n^3 cells jittered +-0.1 cell, E=1e6, nu=0.45, rho=1000, top face pinned.

    n=64 gives 274,625 verts / 1,310,720 tets."""
    return make_grid_body(n, n, n, young=1e6, poisson=0.45, density=1000.0, jitter=0.1, seed=seed)


def batch_c4(nbodies: int = 512, seed: int = 4, lo: int = 4, hi: int = 24, cell: float = 1.0 / 16.0) -> list:
    """Independent hex-grid bodies, dims uniform lo..hi per axis (seeded),
    E log-uniform 1e4..1e7, nu uniform 0.3..0.45, density uniform 800..1200,
    cells of `cell` metres, top faces pinned; bodies laid out on a square
    grid in the x-z plane (they never touch; there is no collision)."""
    rng = np.random.default_rng(seed)
    side = int(math.ceil(math.sqrt(nbodies)))
    bodies = []
    for b in range(nbodies):
        nx, ny, nz = (int(v) for v in rng.integers(lo, hi + 1, size=3))
        E = float(np.exp(rng.uniform(math.log(1e4), math.log(1e7))))
        nu = float(rng.uniform(0.3, 0.45))
        rho = float(rng.uniform(800.0, 1200.0))
        ox, oz = (b % side) * (hi + 4) * cell, (b // side) * (hi + 4) * cell
        bodies.append(make_grid_body(nx, ny, nz, size=(nx * cell, ny * cell, nz * cell), origin=(ox, 0.0, oz),
                                     young=E, poisson=nu, density=rho, seed=seed * 100003 + b))
    return bodies


def request_body(target_tets: float, rng, cell: float = 1.0 / 16.0) -> SoftBody:
    """A near-cubic hex-grid body with about target_tets tets (5 nx ny nz),
    material drawn as in the batch workload."""
    n = max(1.0, (target_tets / 5.0) ** (1.0 / 3.0))
    base = int(n)
    dims = [base, base, base]
    k = 0
    while 5 * dims[0] * dims[1] * dims[2] < target_tets and k < 3:
        dims[k] += 1
        k += 1
    nx, ny, nz = (max(1, d) for d in dims)
    E = float(np.exp(rng.uniform(math.log(1e4), math.log(1e7))))
    nu = float(rng.uniform(0.3, 0.45))
    rho = float(rng.uniform(800.0, 1200.0))
    return make_grid_body(nx, ny, nz, size=(nx * cell, ny * cell, nz * cell), young=E, poisson=nu, density=rho,
                          seed=int(rng.integers(1 << 30)))


def concat(bodies: list) -> SoftBody:
    """One disconnected system holding all bodies (vertex ids offset per body):
    the reference's multi-body layout (dataLoader.cu:291-378)."""
    offs = np.cumsum([0] + [b.num_verts for b in bodies])
    return SoftBody(X=np.concatenate([b.X for b in bodies]).astype(np.float32),
                    tets=np.concatenate([b.tets + np.uint32(o) for b, o in zip(bodies, offs[:-1])]).astype(np.uint32),
                    mass=np.concatenate([b.mass for b in bodies]).astype(np.float32),
                    mu=np.concatenate([b.mu for b in bodies]).astype(np.float32),
                    dbc=np.concatenate([b.dbc for b in bodies]).astype(np.float32),
                    meta={"bodies": len(bodies), "vstart": offs})


def cube_c3(n: int = 40, seed: int = 3) -> SoftBody:
    """1 m cube, n^3 cells, per-tet E log-uniform [1e4, 1e7], nu uniform [0.3, 0.45]."""
    rng = np.random.default_rng(seed)
    nt = 5 * n ** 3
    E = np.exp(rng.uniform(math.log(1e4), math.log(1e7), size=nt))
    nu = rng.uniform(0.3, 0.45, size=nt)
    return make_grid_body(n, n, n, young=E, poisson=nu, density=1000.0)
