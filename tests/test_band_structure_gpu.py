"""rho-Bloch on the GPU against the band Gibbs states of the same lattice (the reference's own check,
band_structure_gibbs_state.py:182-202): known answers independent of the split-operator method."""
import numpy as np
import pytest

from test_band_structure import V0, V_C, XA, lattice, mathieu_levels

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("c128_engine")]

BASE = dict(t=0.0, X_gridDIM=256, X_amplitude=XA, V0=V0, K="0.5 * P * P", V=V_C, quasimomentum=0.0, dt=0.01)


def test_gibbs_state_is_the_band_gibbs_state_to_second_order_in_dbeta():
    from accuratewigner_gb300 import RhoBlochCUDA1D

    q = lattice(256)
    exact = q.get_gibbs(0.0, 0.5, n=256)
    err = []
    for dbeta in (0.005, 0.0025):
        s = RhoBlochCUDA1D(kT=0.5, dbeta=dbeta, **BASE)
        r = s.get_gibbs_state().get()
        s.close()
        r = r / np.trace(r)
        err.append(np.linalg.norm(r - exact) / np.linalg.norm(exact))
    # splitting error of exp(-H / kT): 7.3e-8 at dbeta = 0.005 in the FP64 oracle
    assert err[0] < 1.5e-7
    assert 3.6 < err[0] / err[1] < 4.4


def test_ground_state_is_the_lowest_band_and_stays_put():
    from accuratewigner_gb300 import RhoBlochCUDA1D

    s = RhoBlochCUDA1D(kT=0.5, dbeta=0.005, **BASE)
    s.get_ground_state(dbeta=1e-3)
    r = s.rho.get()
    r = r / np.trace(r)
    q = lattice(256)
    # splitting error of the imaginary-time step that the dbeta halvings ended on (3e-9 in the FP64
    # oracle, 2e-8 with double-float passes, whose purity test stops at another step).  The search
    # (rb:163-223) halves dbeta whenever an energy fails to decrease, and near convergence those
    # comparisons are decided by rounding: where it stops moves the energy by up to 1.5e-8 between
    # summation orders of the same observables.
    assert np.linalg.norm(r - q.get_gibbs(0.0, 0.5, n=1)) < 1e-7
    assert abs(q.get_energy(r) - mathieu_levels(False, 1)[0]) < 3e-8
    # a stationary state: real-time propagation leaves it in place (bsg:190-192), up to the
    # splitting error of the real-time step (the exact band state drifts by 1.8e-6 over these 200
    # steps of dt = 0.01 in the FP64 oracle)
    s.propagate(200)
    r2 = s.rho.get()
    s.close()
    r2 = r2 / np.trace(r2)
    assert np.linalg.norm(r2 - r) < 5e-6
