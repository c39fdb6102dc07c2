"""von Neumann, rho-Bloch and Schrodinger-Wigner on the GPU against the oracle (complex128, 1e-10)."""
import numpy as np
import pytest

from conftest import obs_close, rel_l2
from _cases import SW, VN, VN_INIT

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("c128_engine")]

TOL = 1e-10



def test_von_neumann_propagate_ehrenfest():
    from accuratewigner_gb300 import RhoVNeumannCUDA1D
    from oracle.propagators import RhoVNeumannOracle

    g = RhoVNeumannCUDA1D(**VN)
    c = RhoVNeumannOracle(**VN)
    g.set_rho(VN_INIT)
    c.set_rho(VN_INIT)
    assert rel_l2(g.rho.get(), c.rho) < TOL
    g.propagate(20)
    c.propagate(20)
    assert rel_l2(g.rho.get(), c.rho) < TOL
    for name in ("X_average", "X_average_RHS", "P_average", "P_average_RHS", "hamiltonian_average"):
        assert obs_close(getattr(g, name), getattr(c, name), TOL), name
    assert abs(g.get_purity() - c.get_purity()) < 1e-10
    assert abs(g.get_average((None, "P * P", "X")) - c.get_average((None, "P * P", "X"))) < 1e-10
    assert rel_l2(g.get_wignerfunction().get(), c.get_wignerfunction()) < TOL


def test_von_neumann_absorbing_time_dependent():
    from accuratewigner_gb300 import RhoVNeumannCUDA1D
    from oracle.propagators import RhoVNeumannOracle

    p = dict(VN)
    del p["diff_K"], p["diff_V"]
    p.update(F=0.05, functions="__device__ double E(double t) { return F * sin(0.3 * t); }",
             V="0.5 * omega_square * X * X + X * E(t)",
             abs_boundary_x="pow(abs(cos(0.5 * M_PI * X / X_max)), 0.01)",
             abs_boundary_p="exp(-0.0001 * P * P)")
    g = RhoVNeumannCUDA1D(**p)
    c = RhoVNeumannOracle(**p, py_functions={"E": lambda t: 0.05 * np.sin(0.3 * t)})
    g.set_rho(VN_INIT)
    c.set_rho(VN_INIT)
    g.propagate(15)
    c.propagate(15)
    assert rel_l2(g.rho.get(), c.rho) < TOL


def test_rho_bloch_gibbs():
    from accuratewigner_gb300 import RhoBlochCUDA1D
    from oracle.propagators import RhoBlochOracle

    p = dict(t=0.0, dt=0.01, X_gridDIM=128, X_amplitude=20.0, kT=0.3, omega=1.2,
             K="0.5 * P * P", V="0.5 * omega * omega * X * X")
    g = RhoBlochCUDA1D(**p)
    c = RhoBlochOracle(**p)
    assert g.V_min == c.V_min and g.K_min == c.K_min == 0.0
    g.get_gibbs_state()
    c.get_gibbs_state()
    assert g.gibbs_steps_done == c.gibbs_steps_done
    assert rel_l2(g.rho.get(), c.rho) < TOL
    W = g.get_wignerfunction().get().real
    H = 0.5 * (g.P_wigner ** 2 + 1.2 ** 2 * g.X_wigner ** 2)
    exact = np.tanh(0.5 * 1.2 / 0.3) / np.pi * np.exp(-2 * np.tanh(0.5 * 1.2 / 0.3) * H / 1.2)
    assert np.abs(exact - W).max() * g.dXdP_wigner < 1e-6


def test_rho_bloch_ground_state():
    from accuratewigner_gb300 import RhoBlochCUDA1D
    from oracle.propagators import RhoBlochOracle

    p = dict(t=0.0, dt=0.05, X_gridDIM=64, X_amplitude=8.0, dbeta=0.05, K="0.5 * P * P", V="0.5 * X * X")
    g = RhoBlochCUDA1D(**p)
    c = RhoBlochOracle(**p)
    g.get_ground_state(abs_tol_purity=1e-8)
    c.get_ground_state(abs_tol_purity=1e-8)
    assert rel_l2(g.rho.get(), c.rho) < 1e-8




def test_schrodinger_propagate_ehrenfest_and_wigner():
    from accuratewigner_gb300 import SchrodingerWignerCUDA1D
    from oracle.propagators import SchrodingerWignerOracle

    g = SchrodingerWignerCUDA1D(**SW)
    c = SchrodingerWignerOracle(**SW)
    init = "exp(-pow(X - 1., 2) + cuda_complex(0., 0.5) * X)"
    g.set_wavefunction(init)
    c.set_wavefunction(init)
    g.propagate(30)
    c.propagate(30)
    assert rel_l2(g.wavefunction.get(), c.wavefunction) < TOL
    for name in ("X_average", "X_average_RHS", "P_average", "P_average_RHS", "hamiltonian_average"):
        assert obs_close(getattr(g, name), getattr(c, name), TOL), name
    assert rel_l2(g.get_wigner().get(), c.get_wigner()) < TOL
    assert rel_l2(g.get_wigner_blackman().get(), c.get_wigner(blackman=True)) < TOL


def test_schrodinger_without_ehrenfest_and_ground_state():
    from accuratewigner_gb300 import SchrodingerWignerCUDA1D
    from oracle.propagators import SchrodingerWignerOracle

    p = {k: v for k, v in SW.items() if k not in ("diff_K", "diff_V")}
    g = SchrodingerWignerCUDA1D(**p)
    c = SchrodingerWignerOracle(**p)
    g.set_wavefunction("exp(-X * X)")
    c.set_wavefunction("exp(-X * X)")
    g.propagate(20)
    c.propagate(20)
    assert rel_l2(g.wavefunction.get(), c.wavefunction) < TOL
    g.set_ground_state(500)
    c.set_ground_state(500)
    assert rel_l2(g.wavefunction.get(), c.wavefunction) < TOL
    assert abs(g.get_energy() - c.get_energy()) < 1e-10


def test_schrodinger_stationary_states():
    from accuratewigner_gb300 import SchrodingerWignerCUDA1D
    from oracle.propagators import SchrodingerWignerOracle

    p = dict(t=0.0, dt=0.01, X_gridDIM=256, X_amplitude=10.0, K="0.5 * P * P", V="0.5 * X * X")
    g = SchrodingerWignerCUDA1D(**p)
    c = SchrodingerWignerOracle(**p)
    g.get_stationary_states(3, nsteps=300)
    c.get_stationary_states(3, nsteps=300)
    for a, b in zip(g.stationary_states, c.stationary_states):
        assert rel_l2(a, b) < 1e-9


@pytest.mark.parametrize("n", [16384, 32768])
def test_schrodinger_long_wave_function_four_step(n):
    """Wave functions longer than one pass tile (the reference's coherent_strong_field_physics_cuda_1d.py
    uses X_gridDIM = 16 * 2048) go through the four-step transform."""
    from accuratewigner_gb300 import SchrodingerWignerCUDA1D
    from oracle.propagators import SchrodingerWignerOracle

    p = dict(SW, X_gridDIM=n, X_amplitude=40.0)
    g = SchrodingerWignerCUDA1D(**p)
    c = SchrodingerWignerOracle(**p)
    init = "exp(-pow(X - 1., 2) + cuda_complex(0., 0.5) * X)"
    g.set_wavefunction(init)
    c.set_wavefunction(init)
    g.propagate(25)
    c.propagate(25)
    assert rel_l2(g.wavefunction.get(), c.wavefunction) < TOL
    for name in ("X_average", "X_average_RHS", "P_average", "P_average_RHS", "hamiltonian_average"):
        assert obs_close(getattr(g, name), getattr(c, name), TOL), name
    q = {k: v for k, v in p.items() if k not in ("diff_K", "diff_V")}
    g = SchrodingerWignerCUDA1D(**q)
    c = SchrodingerWignerOracle(**q)
    g.set_wavefunction("exp(-X * X)")
    c.set_wavefunction("exp(-X * X)")
    g.propagate(10)
    c.propagate(10)
    assert rel_l2(g.wavefunction.get(), c.wavefunction) < TOL
    g.set_ground_state(200)
    c.set_ground_state(200)
    assert rel_l2(g.wavefunction.get(), c.wavefunction) < TOL
    assert abs(g.get_energy() - c.get_energy()) < 1e-10
