"""Shared parameter sets for parity tests (small sizes the oracle finishes in seconds)."""
import numpy as np

# wigner_moyal_cuda_1d.py demo form, anharmonic, non-square grid
WM_ANHARMONIC = dict(
    t=0.0, dt=0.01, X_gridDIM=128, X_amplitude=8.0, P_gridDIM=64, P_amplitude=7.0,
    K="0.5 * P * P", V="0.5 * X * X + 0.05 * X * X * X * X",
    diff_K="P", diff_V="X + 0.2 * X * X * X",
)
WM_INIT = "exp(-pow(X - 1., 2) - P * P) / M_PI"


def e_field(t, E0=0.04, omega=0.057, ncyc=5):
    T = ncyc * 2 * np.pi / omega
    return E0 * np.sin(np.pi * t / T) ** 2 * np.sin(omega * t)


E_FIELD_C = """
__device__ double E(double t)
{
    const double T = ncyc * 2. * M_PI / omega;
    return E0 * pow(sin(M_PI * t / T), 2) * sin(omega * t);
}
"""

# time-dependent strong-field form with an absorbing boundary (the 1024^2 strong-field recipe on a small grid)
WM_STRONG_FIELD = dict(
    t=0.0, dt=0.05, X_gridDIM=128, X_amplitude=30.0, P_gridDIM=128, P_amplitude=4.0,
    E0=0.04, omega=0.057, ncyc=5,
    functions=E_FIELD_C,
    K="0.5 * P * P", V="-1. / sqrt(X * X + 2.) + X * E(t)",
    diff_K="P", diff_V="X / pow(X * X + 2., 1.5) + E(t)",
    abs_boundary_x="pow(abs(sin(0.5 * M_PI * (XX + XX_max) / XX_max) * sin(0.5 * M_PI * (XX_prime + XX_prime_max) / XX_prime_max)), dt * 0.05)",
)

# von Neumann: anharmonic oscillator, a displaced boosted Gaussian pure state
VN = dict(t=0.0, dt=0.005, X_gridDIM=128, X_amplitude=10.0, omega_square=0.05, sigma=1.0, p0=0.5, x0=0.5,
          K="0.5 * P * P", V="0.5 * omega_square * X * X + 0.01 * X * X * X * X",
          diff_K="P", diff_V="omega_square * X + 0.04 * X * X * X")
VN_INIT = ("exp(-sigma * pow(X - x0, 2) + cuda_complex(0., p0) * X) * "
           "exp(-sigma * pow(X_prime - x0, 2) - cuda_complex(0., p0) * X_prime)")

# Schrodinger: anharmonic oscillator
SW = dict(t=0.0, dt=0.01, X_gridDIM=256, X_amplitude=10.0, K="0.5 * P * P", V="0.5 * X * X + 0.05 * X * X * X * X",
          diff_K="P", diff_V="X + 0.2 * X * X * X")
