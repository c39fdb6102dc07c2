"""The longest lines the passes take (8192 points) against the oracle: Wigner-Moyal grids of 8192 x 32
and 32 x 8192, so that the 8192-point transform runs once in the row pass (a row tile of 16 elements a
thread) and once in the column pass (a column tile of one 128 KB column), with the Ehrenfest observables
of every step (wigner_moyal_cuda_1d.py:543-606).  The complex128 forms are held to the parity tolerance;
complex64 to the rounding of its FP32 arithmetic over five steps (measured: W 6.6e-7, observables up to
6.4e-6, as on a 128 x 64 grid).

The amplitudes keep the observables' weights moderate: with X_amplitude 60 the quartic term of V and of
the energy weighs the grid's edges by 6.5e5, and the absolute rounding of the tails then moves the
energy by 5e-11 even between native FP64 and the NumPy oracle (double-float 1.8e-10) while W still
agrees to 1.7e-15 (3.6e-14)."""
import numpy as np
import pytest

from conftest import obs_close, rel_l2
from _cases import WM_ANHARMONIC, WM_INIT

pytestmark = pytest.mark.gpu

NAMES = ("X_average", "X_average_RHS", "P_average", "P_average_RHS", "hamiltonian_average")
GRIDS = [(8192, 32, 12.0, 4.0), (32, 8192, 6.0, 16.0)]  # X_gridDIM, P_gridDIM, X_amplitude, P_amplitude
TOL = {"c128": 1e-10, "c128-fp64": 1e-10, "c64": 2e-5}
STEPS = 5


def _params(grid):
    nx, npn, xa, pa = grid
    return dict(WM_ANHARMONIC, X_gridDIM=nx, P_gridDIM=npn, X_amplitude=xa, P_amplitude=pa)


@pytest.fixture(scope="module")
def oracle_runs():
    from oracle.propagators import WignerMoyalOracle

    out = {}
    for grid in GRIDS:
        c = WignerMoyalOracle(**_params(grid))
        c.set_wignerfunction(WM_INIT)
        c.propagate(STEPS)
        out[grid] = (c.wignerfunction.copy(), c.rho.copy(), {k: np.array(getattr(c, k)) for k in NAMES},
                     c.get_purity(), c.t)
    return out


@pytest.mark.parametrize("precision", ["c128", "c128-fp64", "c64"])
@pytest.mark.parametrize("grid", GRIDS, ids=["8192x32", "32x8192"])
def test_wigner_moyal_8192_point_lines_against_oracle(oracle_runs, grid, precision):
    from accuratewigner_gb300 import WignerMoyalCUDA1D

    W, rho, obs, purity, t = oracle_runs[grid]
    tol = TOL[precision]
    g = WignerMoyalCUDA1D(precision=precision, **_params(grid))
    g.set_wignerfunction(WM_INIT)
    g.propagate(STEPS)
    assert g.t == t
    assert rel_l2(g.wignerfunction.get(), W) < tol
    assert rel_l2(g.rho.get(), rho) < tol
    for k in NAMES:
        assert len(getattr(g, k)) == STEPS
        assert obs_close(getattr(g, k), obs[k], tol), k
    assert abs(g.get_purity() - purity) < tol
    g.close()
