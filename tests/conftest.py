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
