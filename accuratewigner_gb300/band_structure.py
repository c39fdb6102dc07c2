"""Band structure and band Gibbs states in mutually unbiased bases (host side).

Counterparts of band_structure_1d.py:7-92 (MUBQBandStructure) and
band_structure_gibbs_state.py:12-116 (MUBGibbsBand).  The reference builds the
dense Hamiltonian H(k) = K(p + k) + V(x) of one cell in the coordinate basis
through two FFTs of diag K (bs:64-80) and diagonalises it with LAPACK; this is
CPU linear algebra in the reference and stays on the host here.  It is the
independent known answer for the rho-Bloch propagator on periodic potentials
(bsg:182-202 compares the two).

Construction used here.  With X_a = dX (a - N/2) and P_m = 2 pi (m - N/2) / (N dX),
the reference's S ifft0 fft1 S of diag K (S = (-1)^(a+b), bs:70-75) is the
circulant matrix

    H_K[a, b] = (1/N) sum_m K(P_m + k) exp(i P_m (X_a - X_b)) = c[(a - b) mod N],

so one N-point FFT of K(P + k) gives its first column and the N x N matrix is a
gather of it, instead of two N x N transforms.  Callables follow the
reference's convention: a function given as a keyword is bound as a method,
V(self, x) and K(self, p).
"""
from types import FunctionType, MethodType

import numpy as np
from scipy import linalg


class MUBQBandStructure:
    """Band structure of H(x, p) = K(p) + V(x) on one lattice cell of length 2 X_amplitude
    (band_structure_1d.py:7-92).  Keywords: X_gridDIM, X_amplitude, V, K (functions of
    (self, x) and (self, p)); any other keyword becomes an attribute."""

    def __init__(self, **kwargs):
        for name, value in kwargs.items():
            setattr(self, name, MethodType(value, self) if isinstance(value, FunctionType) else value)
        for name, what in (("X_gridDIM", "Grid size (X_gridDIM)"), ("X_amplitude", "Coordinate range (X_amplitude)"),
                           ("V", "Potential energy (V)"), ("K", "Momentum dependence (K)")):
            if not hasattr(self, name):
                raise AttributeError("%s was not specified" % what)
        n = int(self.X_gridDIM)
        self.dX = 2.0 * self.X_amplitude / n
        self.X_range = np.linspace(-self.X_amplitude, self.X_amplitude - self.dX, n)
        r = np.arange(n)
        self.sign_flip = (-1) ** (r[:, np.newaxis] + r[np.newaxis, :])
        self.P_range = (np.arange(n, dtype=np.float64) - n // 2) * (2.0 * np.pi / (n * self.dX))
        self._shift = (r[:, np.newaxis] - r[np.newaxis, :]) % n  # circulant index (a - b) mod N

    def _kinetic_column(self, k):
        """c[d] = (1/N) sum_m K(P_m + k) exp(2 pi i (m - N/2) d / N), d = 0 .. N-1."""
        n = int(self.X_gridDIM)
        kp = np.asarray(self.K(self.P_range + k), dtype=np.complex128) * np.broadcast_to(1.0, (n,))
        # exp(2 pi i (m - N/2) d / N) = (-1)^d exp(2 pi i m d / N)
        return np.fft.ifft(kp) * (-1.0) ** np.arange(n)

    def get_hamiltonian(self, k):
        """H(k) in the coordinate representation (bs:64-80)."""
        h = self._kinetic_column(k)[self._shift]
        h[np.diag_indices_from(h)] += self.V(self.X_range)
        return h

    def get_band_structure(self, k, n):
        """The lowest n eigenvalues of H(k) for each Bloch vector of k, shape (n, len(k)) (bs:82-92)."""
        bands = np.array([linalg.eigvalsh(self.get_hamiltonian(q))[:n] for q in np.atleast_1d(k)])
        return bands.T


class MUBGibbsBand(MUBQBandStructure):
    """Gibbs states of one Bloch vector by diagonalisation (band_structure_gibbs_state.py:12-116)."""

    def get_gibbs(self, k_val, kT, n=-1):
        """rho = sum_c |psi_c><psi_c| exp(-E_c / kT) / trace over the bands of H(k_val) (bsg:17-40).

        As in the reference, `n` slices the eigen-pairs with [:n], so the default -1 leaves out
        the highest band (whose Boltzmann weight vanishes at any useful temperature)."""
        vals, vecs = linalg.eigh(self.get_hamiltonian(k_val))
        vecs = vecs[:, :n] * np.exp(1j * k_val * self.X_range[:, np.newaxis])
        vals = vals[:n]
        # weights relative to the lowest band: the same state, without overflow at low kT
        w = np.exp(-(vals - vals[0]) / kT)
        rho = (vecs * w) @ vecs.conj().T
        return rho / rho.trace()

    def get_gibbs_bloch(self, k_val, kT, dbeta=0.005):
        """The reference's own split-operator Bloch loop on the host (bsg:42-89), kept as written
        there: num_beta_steps = ceil(1 / (kT dbeta)), K evaluated at P - k_val, the state
        multiplied by exp(i k_val (X - X')) at the end (its file header marks this propagator as
        incorrect for k_val != 0; at k_val = 0 it is the rho-Bloch propagator)."""
        num_beta_steps = 1.0 / (kT * dbeta)
        if round(num_beta_steps) != num_beta_steps:
            num_beta_steps = np.ceil(num_beta_steps)
            dbeta = 1.0 / (kT * num_beta_steps)
        x = self.X_range[:, np.newaxis]
        xp = self.X_range[np.newaxis, :]
        exp_v = self.sign_flip * np.exp(-0.25 * dbeta * (self.V(x) + self.V(xp)))
        exp_k = np.exp(-0.5 * dbeta * (self.K(self.P_range[:, np.newaxis] - k_val) +
                                       self.K(self.P_range[np.newaxis, :] - k_val)))
        rho = np.eye(int(self.X_gridDIM), dtype=np.complex128)
        for _ in range(int(num_beta_steps)):
            rho *= exp_v
            rho = np.fft.fft(np.fft.ifft(rho, axis=0), axis=1)
            rho *= exp_k
            rho = np.fft.ifft(np.fft.fft(rho, axis=0), axis=1)
            rho *= exp_v
            rho /= rho.trace()
        return rho * np.exp(1j * k_val * (x - xp))

    def get_energy(self, rho):
        """<K + V> of rho (bsg:91-116): V from the diagonal, K from the momentum-basis diagonal."""
        rho = rho / rho.trace()
        average_v = np.dot(rho.diagonal().real, self.V(self.X_range))
        rho_p = np.fft.fft(np.fft.ifft(rho * self.sign_flip, axis=0), axis=1) * self.sign_flip
        rho_p /= rho_p.trace()
        return average_v + np.dot(rho_p.diagonal().real, self.K(self.P_range))
