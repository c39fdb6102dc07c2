"""The benchmark configurations at their full sizes, checked through properties that do not need the
oracle: the double-float engine against native FP64 on the same inputs, Hermiticity, trace and
purity of rho.  (The oracle comparisons run at sizes the CPU finishes in seconds.)"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

FIELD_C = """
__device__ double E(double t)
{
    const double T = ncyc * 2. * M_PI / omega;
    return E0 * pow(sin(M_PI * t / T), 2) * sin(omega * t);
}
__device__ double cosmask(double x, double xmax)
{
    const double a = fabs(x) - 0.9 * xmax;
    return a > 0. ? pow(fabs(cos(0.5 * M_PI * fmin(a / (0.1 * xmax), 1.))), 0.125) : 1.;
}
"""

# strong-field Wigner-Moyal, 1024 x 1024 (the headline configuration)
STRONG_FIELD = dict(t=0.0, dt=0.05, X_gridDIM=1024, X_amplitude=60.0, P_gridDIM=1024, P_amplitude=6.0, E0=0.04,
                    omega=0.057, ncyc=5, functions=FIELD_C, K="0.5 * P * P", V="-1. / sqrt(X * X + 2.) + X * E(t)",
                    diff_K="P", diff_V="X / pow(X * X + 2., 1.5) + E(t)",
                    abs_boundary_x="cosmask(XX, XX_max) * cosmask(XX_prime, XX_prime_max)")
NAMES = ("X_average", "P_average", "P_average_RHS", "X_average_RHS", "hamiltonian_average")


def test_strong_field_1024_double_float_against_native_fp64():
    from accuratewigner_gb300 import WignerMoyalCUDA1D

    runs = {}
    for prec in ("c128", "c128-fp64"):
        s = WignerMoyalCUDA1D(precision=prec, **STRONG_FIELD)
        s.set_wignerfunction("exp(-pow(X - 1., 2) - P * P) / M_PI")
        for _ in range(4):
            s.propagate(50)
        runs[prec] = (s.wignerfunction.get(), {k: np.asarray(getattr(s, k)) for k in NAMES}, s.get_purity())
        s.close()
    (w1, o1, p1), (w2, o2, p2) = runs["c128"], runs["c128-fp64"]
    assert rel_l2(w1, w2) < 1e-10
    for k in NAMES:
        assert o1[k].shape == (200,)
        assert np.max(np.abs(o1[k] - o2[k])) < 1e-10 * max(1.0, np.max(np.abs(o2[k]))), k
    assert abs(p1 - p2) < 1e-10


def test_von_neumann_4096_hermitian_normalised_and_engine_independent():
    from accuratewigner_gb300 import RhoVNeumannCUDA1D

    n = 4096
    p = dict(t=0.0, dt=0.02, X_gridDIM=n, X_amplitude=80.0, D=0.18, alpha=1.0, xm=1.4, K="0.5 * P * P",
             V="D * pow(1. - exp(-alpha * (X - xm)), 2) + X * 0.02 * sin(0.01 * t)")
    rng = np.random.default_rng(0)
    centres = rng.uniform(-3.0, 6.0, 8)
    w = rng.uniform(0.2, 1.0, 8)
    w /= w.sum()
    x = np.linspace(-80.0, 80.0 - 160.0 / n, n)
    rho0 = np.zeros((n, n), np.complex128)
    for c, wk in zip(centres, w):
        g = np.exp(-0.5 * (x - c) ** 2 + 0.3j * x)
        rho0 += wk * np.outer(g, g.conj())
    out = {}
    for prec in ("c128", "c128-fp64"):
        s = RhoVNeumannCUDA1D(precision=prec, **p)
        s.set_rho(rho0)
        s.propagate(20)
        r = s.rho.get()
        out[prec] = (r, s.get_purity())
        s.close()
    r, purity = out["c128"]
    dx = 160.0 / n
    assert abs(np.trace(r).real * dx - 1.0) < 1e-12
    assert np.linalg.norm(r - r.conj().T) < 1e-12 * np.linalg.norm(r)
    assert 0.0 < purity <= 1.0
    assert rel_l2(r, out["c128-fp64"][0]) < 1e-10
