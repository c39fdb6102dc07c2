"""The oracle against the reference's own known answers (CPU only)."""
import numpy as np
import pytest

from oracle.propagators import (RhoBlochOracle, RhoVNeumannOracle, SchrodingerWignerOracle, WignerBlochOracle,
                                WignerMoyalOracle, dbeta_num_beta_steps)

from _cases import WM_ANHARMONIC, WM_INIT


def ho_gibbs(omega, kT, X, P):
    # wigner_bloch_cuda_1d.py:404-409
    return np.tanh(0.5 * omega / kT) / np.pi * np.exp(-2.0 * np.tanh(0.5 * omega / kT) * 0.5 * (P ** 2 + omega ** 2 * X ** 2) / omega)


def test_wigner_bloch_harmonic_gibbs():
    p = dict(t=0.0, dt=0.01, X_gridDIM=128, X_amplitude=10.0, P_gridDIM=128, P_amplitude=10.0, kT=0.5, omega=1.5,
             K="0.5 * P * P", V="0.5 * omega * omega * X * X")
    wb = WignerBlochOracle(**p)
    g = wb.get_gibbs_state()
    err = np.abs(ho_gibbs(1.5, 0.5, wb.X, wb.P) - g.real).max() * wb.dXdP
    assert err < 1e-6
    assert wb.gibbs_steps_done == 200


def test_rho_bloch_harmonic_gibbs():
    p = dict(t=0.0, dt=0.01, X_gridDIM=128, X_amplitude=20.0, kT=0.3, omega=1.2,
             K="0.5 * P * P", V="0.5 * omega * omega * X * X")
    rb = RhoBlochOracle(**p)
    rb.get_gibbs_state()
    W = rb.get_wignerfunction().real
    err = np.abs(ho_gibbs(1.2, 0.3, rb.X_wigner, rb.P_wigner) - W).max() * rb.dXdP_wigner
    assert err < 1e-6
    assert rb.K_min == 0.0  # rho_bloch_cuda_1d.py:370 quirk


def test_wigner_moyal_energy_and_ehrenfest():
    wm = WignerMoyalOracle(**WM_ANHARMONIC)
    wm.set_wignerfunction(WM_INIT)
    wm.propagate(60)
    h = np.array(wm.hamiltonian_average)
    assert (1 - h.min() / h.max()) < 1e-3
    xa = np.array(wm.X_average)
    dxdt = np.gradient(xa, wm.dt)
    assert np.abs(dxdt[2:-2] - np.array(wm.X_average_RHS)[2:-2]).max() < 1e-3
    assert abs(np.sum(wm.wignerfunction).real * wm.dXdP - 1.0) < 1e-12


def test_von_neumann_trace_energy():
    p = dict(t=0.0, dt=0.005, X_gridDIM=128, X_amplitude=10.0, omega_square=0.05, sigma=1.0, p0=0.5, x0=0.5,
             K="0.5 * P * P", V="0.5 * omega_square * X * X", diff_K="P", diff_V="omega_square * X")
    vn = RhoVNeumannOracle(**p)
    vn.set_rho("exp(-sigma * pow(X - x0, 2) + cuda_complex(0., p0) * X) * "
               "exp(-sigma * pow(X_prime - x0, 2) - cuda_complex(0., p0) * X_prime)")
    vn.propagate(40)
    h = np.array(vn.hamiltonian_average)
    assert (1 - h.min() / h.max()) < 1e-6
    assert abs(np.trace(vn.rho).real * vn.dX - 1.0) < 1e-12
    assert abs(vn.get_purity() - 1.0) < 1e-10


def test_schrodinger_ground_state_and_wigner():
    p = dict(t=0.0, dt=0.01, X_gridDIM=256, X_amplitude=10.0, K="0.5 * P * P", V="0.5 * X * X",
             diff_K="P", diff_V="X")
    sw = SchrodingerWignerOracle(**p)
    sw.set_ground_state(2000)
    assert abs(sw.get_energy() - 0.5) < 1e-6
    W = sw.get_wigner()
    assert abs(np.sum(W).real * sw.wigner_dXdP - 1.0) < 1e-12


def test_dbeta_num_beta_steps_rounding():
    # Python 2 round-half-away semantics of the reference
    assert dbeta_num_beta_steps(0.5, 0.01) == (0.01, 200)
    db, n = dbeta_num_beta_steps(0.3, 0.01)
    assert n == 333 and abs(db - 1.0 / (0.3 * 333)) < 1e-18
    assert dbeta_num_beta_steps(0.0, 0.01)[1] == np.inf
