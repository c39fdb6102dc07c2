"""Wigner-Moyal / Wigner-Bloch on the GPU against the oracle (plain complex128, 1e-10 relative L2)."""
import numpy as np
import pytest

from conftest import obs_close, rel_l2
from _cases import WM_ANHARMONIC, WM_INIT, WM_STRONG_FIELD, e_field

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("c128_engine")]

TOL = 1e-10  # plain complex128 form: relative L2 against the FP64 oracle


def _pair(cls_gpu, cls_cpu, params, **extra):
    from oracle.propagators import WignerMoyalOracle  # noqa: F401

    g = cls_gpu(**params, **extra)
    c = cls_cpu(**params)
    return g, c


def test_wigner2rho_rho2wigner_roundtrip():
    from accuratewigner_gb300 import WignerMoyalCUDA1D
    from oracle.propagators import WignerMoyalOracle

    p = dict(WM_ANHARMONIC)
    g = WignerMoyalCUDA1D(**p)
    c = WignerMoyalOracle(**p)
    g.set_wignerfunction(WM_INIT)
    c.set_wignerfunction(WM_INIT)
    assert rel_l2(g.rho.get(), c.rho) < TOL
    g.rho2wigner()
    c.rho2wigner()
    assert rel_l2(g.wignerfunction.get(), c.wignerfunction) < TOL


def test_get_into_a_given_array():
    """get(ary) fills a preallocated host array in place (pycuda's GPUArray.get(ary)) with the bits
    get() returns, and refuses an array of another type or shape."""
    from accuratewigner_gb300 import WignerMoyalCUDA1D

    g = WignerMoyalCUDA1D(**WM_ANHARMONIC)
    g.set_wignerfunction(WM_INIT)
    g.propagate(3)
    host = np.empty(g.wignerfunction.shape, np.complex128)
    assert g.wignerfunction.get(host) is host
    assert np.array_equal(host, g.wignerfunction.get())
    r, c = host.shape
    for bad in (np.empty((r, c), np.complex64), np.empty((3, 3), np.complex128),
                np.empty((r, 2 * c), np.complex128)[:, ::2]):
        with pytest.raises(ValueError):
            g.wignerfunction.get(bad)
    g.close()


def test_propagate_ehrenfest_anharmonic():
    from accuratewigner_gb300 import WignerMoyalCUDA1D
    from oracle.propagators import WignerMoyalOracle

    g = WignerMoyalCUDA1D(**WM_ANHARMONIC)
    c = WignerMoyalOracle(**WM_ANHARMONIC)
    g.set_wignerfunction(WM_INIT)
    c.set_wignerfunction(WM_INIT)
    g.propagate(25)
    c.propagate(25)
    assert g.t == c.t
    assert rel_l2(g.wignerfunction.get(), c.wignerfunction) < TOL
    assert rel_l2(g.rho.get(), c.rho) < TOL
    for name in ("X_average", "X_average_RHS", "P_average", "P_average_RHS", "hamiltonian_average"):
        assert len(getattr(g, name)) == 25
        assert obs_close(getattr(g, name), getattr(c, name), TOL), name
    assert abs(g.get_purity() - c.get_purity()) < 1e-10
    assert abs(g.get_average("X * P") - c.get_average("X * P")) < 1e-10


def test_propagate_without_ehrenfest():
    from accuratewigner_gb300 import WignerMoyalCUDA1D
    from oracle.propagators import WignerMoyalOracle

    p = {k: v for k, v in WM_ANHARMONIC.items() if k not in ("diff_K", "diff_V")}
    g = WignerMoyalCUDA1D(**p)
    c = WignerMoyalOracle(**p)
    g.set_wignerfunction(WM_INIT)
    c.set_wignerfunction(WM_INIT)
    g.propagate(10)
    c.propagate(10)
    g.propagate(7)
    c.propagate(7)
    assert rel_l2(g.wignerfunction.get(), c.wignerfunction) < TOL
    assert rel_l2(g.rho.get(), c.rho) < TOL


def test_strong_field_time_dependent_with_absorber():
    from accuratewigner_gb300 import WignerMoyalCUDA1D
    from oracle.propagators import WignerMoyalOracle

    p = dict(WM_STRONG_FIELD)
    g = WignerMoyalCUDA1D(**p)
    c = WignerMoyalOracle(**p, py_functions={"E": e_field})
    init = "exp(-X * X - P * P) / M_PI"
    g.set_wignerfunction(init)
    c.set_wignerfunction(init)
    g.propagate(30)
    c.propagate(30)
    assert rel_l2(g.wignerfunction.get(), c.wignerfunction) < TOL
    for name in ("X_average", "P_average", "P_average_RHS", "hamiltonian_average"):
        assert obs_close(getattr(g, name), getattr(c, name), TOL), name


def test_time_dependent_absorbers_in_both_frames():
    # abs_boundary_x and abs_boundary_p that change with t: the row pass applies the kicks of t_n and
    # t_n+1 with masks of their own times
    from accuratewigner_gb300 import WignerMoyalCUDA1D
    from oracle.propagators import WignerMoyalOracle

    p = dict(WM_STRONG_FIELD)
    p["abs_boundary_x"] = ("pow(abs(sin(0.5 * M_PI * (XX + XX_max) / XX_max) * sin(0.5 * M_PI * (XX_prime + "
                           "XX_prime_max) / XX_prime_max)), dt * (0.05 + 0.02 * sin(0.1 * t)))")
    p["abs_boundary_p"] = "exp(-dt * 0.001 * (1. + cos(0.2 * t)) * (PP * PP + PP_prime * PP_prime))"
    g = WignerMoyalCUDA1D(**p)
    c = WignerMoyalOracle(**p, py_functions={"E": e_field})
    init = "exp(-pow(X - 2., 2) - P * P) / M_PI"
    g.set_wignerfunction(init)
    c.set_wignerfunction(init)
    for n in (7, 13):  # two calls: the masks carry over between them
        g.propagate(n)
        c.propagate(n)
    assert rel_l2(g.wignerfunction.get(), c.wignerfunction) < TOL
    for name in ("X_average", "P_average", "P_average_RHS", "hamiltonian_average"):
        assert obs_close(getattr(g, name), getattr(c, name), TOL), name
    g.close()


@pytest.mark.parametrize("absorber", [
    # a product f(XX) g(XX'): folded into the kick tables
    "exp(-dt * 0.02 * (pow(XX / XX_max, 8) + pow(XX_prime / XX_prime_max, 8)))",
    # not a product: read per point from the 2-D mask
    "exp(-dt * 0.02 * pow((XX - XX_prime) / XX_max, 2))",
])
def test_time_independent_absorbers_separable_or_not(absorber):
    from accuratewigner_gb300 import WignerMoyalCUDA1D
    from oracle.propagators import WignerMoyalOracle

    p = dict(WM_STRONG_FIELD, abs_boundary_x=absorber)
    g = WignerMoyalCUDA1D(**p)
    c = WignerMoyalOracle(**p, py_functions={"E": e_field})
    init = "exp(-pow(X - 2., 2) - P * P) / M_PI"
    g.set_wignerfunction(init)
    c.set_wignerfunction(init)
    g.propagate(12)
    c.propagate(12)
    assert rel_l2(g.wignerfunction.get(), c.wignerfunction) < TOL
    for name in ("X_average", "P_average", "hamiltonian_average"):
        assert obs_close(getattr(g, name), getattr(c, name), TOL), name
    g.close()


def test_wigner_bloch_gibbs_matches_oracle_and_analytic():
    from accuratewigner_gb300 import WignerBlochCUDA1D
    from oracle.propagators import WignerBlochOracle

    p = dict(t=0.0, dt=0.01, X_gridDIM=128, X_amplitude=10.0, P_gridDIM=128, P_amplitude=10.0, kT=0.5, omega=1.5,
             K="0.5 * P * P", V="0.5 * omega * omega * X * X")
    g = WignerBlochCUDA1D(**p)
    c = WignerBlochOracle(**p)
    assert g.V_min == c.V_min and g.K_min == c.K_min
    Wg = g.get_gibbs_state().get()
    Wc = c.get_gibbs_state()
    assert g.gibbs_steps_done == c.gibbs_steps_done == 200
    assert rel_l2(Wg, Wc) < TOL
    assert rel_l2(g.rho.get(), c.rho) < TOL
    exact = np.tanh(0.5 * 1.5 / 0.5) / np.pi * np.exp(
        -2.0 * np.tanh(0.5 * 1.5 / 0.5) * 0.5 * (g.P ** 2 + 1.5 ** 2 * g.X ** 2) / 1.5)
    assert np.abs(exact - Wg.real).max() * g.dXdP < 1e-6


def test_wigner_bloch_purity_stop():
    from accuratewigner_gb300 import WignerBlochCUDA1D
    from oracle.propagators import WignerBlochOracle

    # very low temperature: purity reaches 1 and the loop stops early (wb:144-153)
    p = dict(t=0.0, dt=0.05, X_gridDIM=64, X_amplitude=6.0, P_gridDIM=64, P_amplitude=6.0, kT=0.005, dbeta=0.05,
             K="0.5 * P * P", V="0.5 * X * X")
    g = WignerBlochCUDA1D(**p)
    c = WignerBlochOracle(**p)
    Wg = g.get_gibbs_state().get()
    Wc = c.get_gibbs_state()
    n = g.get_dbeta_num_beta_steps(0.005, 0.05)[1]
    # both stop once purity reaches one; the exact step depends on the last bits of the purity
    assert g.gibbs_steps_done < n and c.gibbs_steps_done < n
    assert g.get_purity() >= 1.0 - 1e-12
    assert rel_l2(Wg, Wc) < 1e-6


def test_wigner_bloch_ground_state():
    from accuratewigner_gb300 import WignerBlochCUDA1D
    from oracle.propagators import WignerBlochOracle

    p = dict(t=0.0, dt=0.05, X_gridDIM=64, X_amplitude=6.0, P_gridDIM=64, P_amplitude=6.0, dbeta=0.05,
             K="0.5 * P * P", V="0.5 * X * X")
    g = WignerBlochCUDA1D(**p)
    c = WignerBlochOracle(**p)
    Wg = g.get_ground_state(abs_tol_purity=1e-8).get()
    Wc = c.get_ground_state(abs_tol_purity=1e-8)
    assert rel_l2(Wg, Wc) < 1e-8
    assert abs(g.get_average(g.hamiltonian) - 0.5) < 1e-4


def test_large_grid_marginal_pass_1024():
    """1024 x 1024 exercises the clustered marginal column pass (48 KB shared memory per block)."""
    from accuratewigner_gb300 import WignerMoyalCUDA1D
    from oracle.propagators import WignerMoyalOracle

    p = dict(WM_ANHARMONIC, X_gridDIM=1024, P_gridDIM=1024, X_amplitude=12.0, P_amplitude=12.0)
    g = WignerMoyalCUDA1D(**p)
    c = WignerMoyalOracle(**p)
    g.set_wignerfunction(WM_INIT)
    c.set_wignerfunction(WM_INIT)
    g.propagate(3)
    c.propagate(3)
    assert rel_l2(g.wignerfunction.get(), c.wignerfunction) < TOL
    for name in ("X_average", "P_average", "P_average_RHS", "hamiltonian_average"):
        assert obs_close(getattr(g, name), getattr(c, name), TOL), name
