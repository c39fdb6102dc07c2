"""Zero and negative step counts, as the reference's loops over xrange(steps) run them: no step, the time
unchanged and no observable recorded.  Wigner-Moyal without Ehrenfest observables still ends with
normalize_rho_wigner (wigner_moyal_cuda_1d.py:563-582); von Neumann and the Schrodinger propagator leave
the state as it was (rho_vneumann_cuda_1d.py:429-448, schrodinger_wigner_cuda_1d.py:371-390).  A step
count after them continues as if they had not been made."""
import numpy as np
import pytest

from conftest import obs_close, rel_l2
from _cases import SW, VN, VN_INIT, WM_ANHARMONIC, WM_INIT

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("c128_engine")]

TOL = 1e-10
NAMES = ("X_average", "X_average_RHS", "P_average", "P_average_RHS", "hamiltonian_average")


@pytest.mark.parametrize("ehrenfest", [True, False])
@pytest.mark.parametrize("steps", [0, -3])
def test_wigner_moyal_no_steps(steps, ehrenfest):
    from accuratewigner_gb300 import WignerMoyalCUDA1D
    from oracle.propagators import WignerMoyalOracle

    p = dict(WM_ANHARMONIC)
    if not ehrenfest:
        p.pop("diff_K")
        p.pop("diff_V")
    g = WignerMoyalCUDA1D(**p)
    c = WignerMoyalOracle(**p)
    g.set_wignerfunction(WM_INIT)
    c.set_wignerfunction(WM_INIT)
    # an unnormalised rho, so that a normalisation shows (set_wignerfunction normalises)
    g.rho.set(3.0 * g.rho.get())
    c.rho = 3.0 * c.rho
    g.propagate(steps)
    c.propagate(steps)
    assert g.t == c.t == 0.0
    assert rel_l2(g.wignerfunction.get(), c.wignerfunction) < TOL
    assert rel_l2(g.rho.get(), c.rho) < TOL
    # without Ehrenfest observables the call still normalised rho (and recomputed W); with them not
    trace = float(np.sum(np.abs(g.rho.get()) ** 2))
    assert (abs(trace - float(np.sum(np.abs(c.rho) ** 2))) < TOL * trace)
    if ehrenfest:
        for k in NAMES:
            assert len(getattr(g, k)) == 0, k
    g.propagate(4)
    c.propagate(4)
    assert rel_l2(g.wignerfunction.get(), c.wignerfunction) < TOL
    if ehrenfest:
        for k in NAMES:
            assert obs_close(getattr(g, k), getattr(c, k), TOL), k
    g.close()


@pytest.mark.parametrize("steps", [0, -3])
def test_von_neumann_and_schrodinger_no_steps(steps):
    from accuratewigner_gb300 import RhoVNeumannCUDA1D, SchrodingerWignerCUDA1D
    from oracle.propagators import RhoVNeumannOracle, SchrodingerWignerOracle

    g = RhoVNeumannCUDA1D(**VN)
    c = RhoVNeumannOracle(**VN)
    g.set_rho(VN_INIT)
    c.set_rho(VN_INIT)
    rho0 = g.rho.get()
    g.propagate(steps)
    c.propagate(steps)
    assert g.t == c.t == 0.0
    assert np.array_equal(g.rho.get(), rho0)
    g.propagate(3)
    c.propagate(3)
    assert rel_l2(g.rho.get(), c.rho) < TOL
    g.close()

    init = "exp(-pow(X - 1., 2) + cuda_complex(0., 0.5) * X)"
    g = SchrodingerWignerCUDA1D(**SW)
    c = SchrodingerWignerOracle(**SW)
    g.set_wavefunction(init)
    c.set_wavefunction(init)
    psi0 = g.wavefunction.get()
    g.propagate(steps)
    c.propagate(steps)
    assert g.t == c.t == 0.0
    assert np.array_equal(g.wavefunction.get(), psi0)
    g.propagate(3)
    c.propagate(3)
    assert rel_l2(g.wavefunction.get(), c.wavefunction) < TOL
    for k in NAMES:
        assert obs_close(getattr(g, k), getattr(c, k), TOL), k
    g.close()
