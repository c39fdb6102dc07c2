"""CPU restatement of the reference's MUB Hamiltonian (band_structure_1d.py:51-80).

TEST INFRASTRUCTURE ONLY: the oracle for ``accuratewigner_gb300.band_structure``,
imported by ``tests/`` alone.  It builds H(k) exactly as the reference does, two
dense transforms of diag K(P + k) between sign flips, where the package gathers
a circulant from one N-point FFT.
"""
import numpy as np


def mub_grids(X_gridDIM, X_amplitude):
    """bs:51-62: X_range, P_range (centred FFT frequencies) and the sign-flip matrix."""
    n = int(X_gridDIM)
    dX = 2.0 * X_amplitude / n
    X = np.linspace(-X_amplitude, X_amplitude - dX, n)
    r = np.arange(n)
    sign = (-1) ** (r[:, None] + r[None, :])
    P = (np.arange(n, dtype=np.float64) - n // 2) * (2.0 * np.pi / (n * dX))
    return X, P, sign


def mub_hamiltonian(X_gridDIM, X_amplitude, V, K, k):
    """bs:64-80 with V(x) and K(p) plain functions; scipy.fftpack's ifft / fft are numpy's."""
    X, P, sign = mub_grids(X_gridDIM, X_amplitude)
    h = np.diag(K(P + k)).astype(np.complex128)
    h *= sign
    h = np.fft.ifft(h, axis=0)
    h = np.fft.fft(h, axis=1)
    h *= sign
    h += np.diag(V(X))
    return h
