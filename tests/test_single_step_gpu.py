"""The public single-step and per-call observable methods against the oracle: single_step_propagation
of the three real-time classes (one unnormalised step at the current t), the Schrodinger
get_Ehrenfest and projectout_stationary_states."""
import numpy as np
import pytest

from conftest import obs_close, rel_l2
from _cases import SW, VN, VN_INIT, WM_ANHARMONIC, WM_INIT, WM_STRONG_FIELD, e_field

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("c128_engine")]

TOL = 1e-10


def _steps(g, c, n):
    for _ in range(n):
        g.t += g.dt
        c.t += c.dt
        g.single_step_propagation()
        c.single_step_propagation()


@pytest.mark.parametrize("case", ["anharmonic", "strong_field"])
def test_wigner_moyal_single_steps(case):
    from accuratewigner_gb300 import WignerMoyalCUDA1D
    from oracle.propagators import WignerMoyalOracle

    if case == "anharmonic":
        p, extra = dict(WM_ANHARMONIC), {}
    else:
        p, extra = dict(WM_STRONG_FIELD), {"py_functions": {"E": e_field}}
    g = WignerMoyalCUDA1D(**p)
    c = WignerMoyalOracle(**p, **extra)
    g.set_wignerfunction(WM_INIT)
    c.set_wignerfunction(WM_INIT)
    _steps(g, c, 3)
    assert g.t == c.t
    assert rel_l2(g.rho.get(), c.rho) < TOL
    # not normalised: the reference leaves that to propagate / normalize_rho_wigner
    g.normalize_rho_wigner()
    c.normalize_rho_wigner()
    assert rel_l2(g.wignerfunction.get(), c.wignerfunction) < TOL
    g.close()


def test_von_neumann_single_steps():
    from accuratewigner_gb300 import RhoVNeumannCUDA1D
    from oracle.propagators import RhoVNeumannOracle

    g = RhoVNeumannCUDA1D(**VN)
    c = RhoVNeumannOracle(**VN)
    g.set_rho(VN_INIT)
    c.set_rho(VN_INIT)
    _steps(g, c, 3)
    assert rel_l2(g.rho.get(), c.rho) < TOL
    assert abs(np.trace(g.rho.get()) - np.trace(c.rho)) < 1e-10 * abs(np.trace(c.rho))
    g.close()


def test_schrodinger_single_steps_and_get_ehrenfest():
    from accuratewigner_gb300 import SchrodingerWignerCUDA1D
    from oracle.propagators import SchrodingerWignerOracle

    g = SchrodingerWignerCUDA1D(**SW)
    c = SchrodingerWignerOracle(**SW)
    init = "exp(-pow(X - 1., 2) + cuda_complex(0., 0.5) * X)"
    g.set_wavefunction(init)
    c.set_wavefunction(init)
    _steps(g, c, 4)
    assert rel_l2(g.wavefunction.get(), c.wavefunction) < TOL
    g.get_Ehrenfest(g.t)
    c.get_Ehrenfest(c.t)
    for name in ("X_average", "X_average_RHS", "P_average", "P_average_RHS", "hamiltonian_average"):
        assert len(getattr(g, name)) == 1
        assert obs_close(getattr(g, name), getattr(c, name), TOL), name
    g.close()


def test_schrodinger_projectout_stationary_states():
    from accuratewigner_gb300 import SchrodingerWignerCUDA1D
    from oracle.propagators import SchrodingerWignerOracle

    p = dict(t=0.0, dt=0.01, X_gridDIM=256, X_amplitude=10.0, K="0.5 * P * P", V="0.5 * X * X")
    g = SchrodingerWignerCUDA1D(**p)
    c = SchrodingerWignerOracle(**p)
    g.get_stationary_states(2, nsteps=300)
    c.get_stationary_states(2, nsteps=300)
    x = np.linspace(-10.0, 10.0 - 20.0 / 256, 256)
    psi = (np.exp(-0.5 * (x - 1.0) ** 2) * (1.0 + 0.3 * x)).astype(np.complex128).reshape(1, -1)
    a = g.projectout_stationary_states(psi.copy())
    b = c.projectout_stationary_states(psi.copy().reshape(c.wavefunction.shape))
    assert rel_l2(a.reshape(-1), np.asarray(b).reshape(-1)) < 1e-9
    for phi in g.stationary_states:
        assert abs(np.vdot(phi.reshape(-1), a.reshape(-1))) < 1e-9
    # a device array of the package is projected in place and returned
    g.set_wavefunction(psi)
    out = g.projectout_stationary_states(g.wavefunction)
    assert out is g.wavefunction
    assert rel_l2(g.wavefunction.get().reshape(-1), a.reshape(-1)) < 1e-12
    g.close()
