"""Device-side detection of a step that leaves the finite range.

The reference has no such check: SolverStep returns true unconditionally
(pdSolver.cu:207) and a diverged state stays silently NaN.  The engine's step
epilogue sets a device word when a vertex ends a step with a non-finite
position or velocity; pdgb_last_step_status reads it (PDGB_ERR_NONFINITE) and
setting the state again clears it.
"""
import numpy as np
import pytest

from pdgb import PdgbError, PdSolver, SolverParams, mesh
from pdgb import _native as N

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("solver", [0, 1])
def test_nan_position_is_reported(solver):
    body = mesh.make_grid_body(4, 3, 5, young=1e5, poisson=0.4, jitter=0.1, seed=4)
    params = SolverParams(num_iterations=10, rho=0.9995, solver=solver)
    with PdSolver(body, params) as e:
        e.update(2)
        assert e.step_status() == N.PDGB_OK
        X, V = e.download_state()
        Xbad = X.copy()
        Xbad[7, 1] = np.nan
        e.upload_state(Xbad, V)
        assert e.step_status() == N.PDGB_OK  # nothing stepped yet
        e.update(1)
        assert e.step_status() == N.PDGB_ERR_NONFINITE
        with pytest.raises(PdgbError) as err:
            e.check_finite()
        assert err.value.status == N.PDGB_ERR_NONFINITE
        e.update(1)  # sticky until the state is set again
        assert e.step_status() == N.PDGB_ERR_NONFINITE
        e.upload_state(X, V)
        e.update(1)
        assert e.step_status() == N.PDGB_OK
        Xinf = X.copy()
        Xinf[3, 0] = np.inf
        e.upload_state(Xinf, V)
        e.update(1)
        assert e.step_status() == N.PDGB_ERR_NONFINITE
        e.reset()
        e.update(1)
        assert e.step_status() == N.PDGB_OK
