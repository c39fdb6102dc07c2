"""The identities behind the von Neumann momentum diagonal of the pass kernels (aw_api.cu, vn_run;
aw_util.cu, aw_k_diag_dft), checked in NumPy on random data:

* M_k = (1/N) Sum_i [fft1(T)]_ik exp(+2 pi i k i / N)  (the p branch of get_average,
  rho_vneumann_cuda_1d.py:548-561) equals (1/N) Sum_d G_d exp(-2 pi i k d / N) with the diagonal sums
  G_d = Sum_i T_{i, (i + d) mod N};
* G is what alternating column sums of the rotated, signed branch store give:
  B[i, (j - i) mod N] = (-1)^i T[i, j],  G_m = Sum_i (-1)^i B[i, m];
* the two-launch four-step DFT (d = d1 + n1 d2, k = k2 + n2 k1) equals the direct DFT.
"""
import numpy as np


def _four_step(g, scale):
    n = g.size
    l = int(np.log2(n))
    n1 = 1 << (l // 2)
    n2 = n // n1
    x = np.zeros((n1, n2), complex)
    for d1 in range(n1):
        for k2 in range(n2):
            s = sum(g[d1 + n1 * d2] * np.exp(-2j * np.pi * ((k2 * d2) % n2) / n2) for d2 in range(n2))
            x[d1, k2] = s * np.exp(-2j * np.pi * ((k2 * d1) % n) / n)
    m = np.zeros(n)
    for k2 in range(n2):
        for k1 in range(n1):
            m[k2 + n2 * k1] = scale * sum(x[d1, k2] * np.exp(-2j * np.pi * ((k1 * d1) % n1) / n1)
                                          for d1 in range(n1)).real
    return m


def test_momentum_diagonal_from_diagonal_sums():
    rng = np.random.default_rng(3)
    for n in (8, 32, 64):
        t = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
        i = np.arange(n)[:, None]
        k = np.arange(n)[None, :]
        m_ref = (np.fft.fft(t, axis=1) * np.exp(2j * np.pi * i * k / n)).sum(axis=0) / n
        b = np.zeros_like(t)
        for r in range(n):
            b[r, (np.arange(n) - r) % n] = (-1) ** r * t[r]
        g = ((-1.0) ** np.arange(n)[:, None] * b).sum(axis=0)
        g_direct = np.array([sum(t[r, (r + d) % n] for r in range(n)) for d in range(n)])
        assert np.allclose(g, g_direct, rtol=0, atol=1e-12 * np.abs(g_direct).max())
        m = np.fft.fft(g) / n
        assert np.allclose(m, m_ref, rtol=0, atol=1e-12 * np.abs(m_ref).max())
        assert np.allclose(_four_step(g, 1.0 / n), m_ref.real, rtol=0, atol=1e-12 * np.abs(m_ref).max())
