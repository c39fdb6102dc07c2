"""MUB band structure and band Gibbs states (host side): the package against the restated
reference construction, and both against known answers (Mathieu characteristic values, the
rho-Bloch oracle)."""
import numpy as np
import pytest
from scipy import special

from oracle.band_structure import mub_hamiltonian
from oracle.propagators import RhoBlochOracle

XA, V0 = 4.0, 0.37  # the reference's example lattice (band_structure_gibbs_state.py:130-144)
V_C = "-V0 * (1. + cos(M_PI * (X + X_amplitude) / X_amplitude))"


def v_mathieu(x):
    return -V0 * (1 + np.cos(np.pi * (x + XA) / XA))


def k_free(p):
    return 0.5 * p ** 2


def lattice(n, cls=None):
    from accuratewigner_gb300.band_structure import MUBGibbsBand

    return (cls or MUBGibbsBand)(X_gridDIM=n, X_amplitude=XA, V0=V0, K=lambda self, p: 0.5 * p ** 2,
                                 V=lambda self, x: -self.V0 * (1 + np.cos(np.pi * (x + self.X_amplitude) /
                                                                           self.X_amplitude)))


@pytest.mark.parametrize("n", [64, 256])
@pytest.mark.parametrize("k", [0.0, 0.3, -np.pi / (2 * XA)])
def test_hamiltonian_matches_the_reference_construction(n, k):
    h = lattice(n).get_hamiltonian(k)
    ref = mub_hamiltonian(n, XA, v_mathieu, k_free, k)
    assert np.max(np.abs(h - ref)) < 1e-13 * np.max(np.abs(ref))
    assert np.max(np.abs(h - h.conj().T)) < 1e-14 * np.max(np.abs(ref))


def mathieu_levels(k_edge, count):
    """-1/2 psi'' - V0 (1 + cos(pi (x + Xa) / Xa)) psi = E psi is Mathieu's equation in
    z = pi (x + Xa) / (2 Xa) with q = -(4 Xa^2 / pi^2) V0 and E = pi^2 a / (8 Xa^2) - V0; Bloch vector
    0 takes the pi-periodic solutions (a_2r, b_2r), the zone edge the anti-periodic ones."""
    q = -(4 * XA ** 2 / np.pi ** 2) * V0
    if k_edge:
        a = [special.mathieu_a(2 * r + 1, q) for r in range(count)] + [special.mathieu_b(2 * r + 1, q)
                                                                     for r in range(count)]
    else:
        a = [special.mathieu_a(2 * r, q) for r in range(count)] + [special.mathieu_b(2 * r, q)
                                                                 for r in range(1, count)]
    return np.sort(np.array(a))[:count] * np.pi ** 2 / (8 * XA ** 2) - V0


def test_bands_are_the_mathieu_characteristic_values():
    q = lattice(256)
    bands = q.get_band_structure([0.0, np.pi / (2 * XA)], 6)
    assert bands.shape == (6, 2)
    assert np.max(np.abs(bands[:, 0] - mathieu_levels(False, 6))) < 1e-10
    assert np.max(np.abs(bands[:, 1] - mathieu_levels(True, 6))) < 1e-10


def test_free_particle_bands_are_the_shifted_parabola():
    from accuratewigner_gb300.band_structure import MUBQBandStructure

    q = MUBQBandStructure(X_gridDIM=64, X_amplitude=3.0, K=lambda self, p: 0.5 * p ** 2, V=lambda self, x: 0 * x)
    for k in (0.0, 0.2):
        exact = np.sort(0.5 * (q.P_range + k) ** 2)[:5]
        assert np.allclose(q.get_band_structure([k], 5)[:, 0], exact, rtol=0, atol=1e-12)


def test_missing_keywords_raise_attribute_error():
    from accuratewigner_gb300.band_structure import MUBQBandStructure

    with pytest.raises(AttributeError):
        MUBQBandStructure(X_gridDIM=64, X_amplitude=3.0, K=lambda self, p: p)


def test_band_gibbs_state_energy_and_projector():
    q = lattice(128)
    e = q.get_band_structure([0.0], 3)[:, 0]
    g1 = q.get_gibbs(0.0, 0.5, n=1)  # the lowest band alone: a pure state
    assert abs(np.trace(g1) - 1) < 1e-13
    assert abs(np.sum(np.abs(g1) ** 2) - 1) < 1e-12
    assert abs(q.get_energy(g1) - e[0]) < 1e-11
    g = q.get_gibbs(0.0, 0.5, n=3)
    w = np.exp(-(e - e[0]) / 0.5)
    assert abs(q.get_energy(g) - np.dot(w, e) / w.sum()) < 1e-11


def test_reference_bloch_loop_is_the_rho_bloch_propagator_at_k0():
    q = lattice(64)
    kT, dbeta = 0.5, 0.01  # 200 steps, no re-fit of dbeta
    loop = q.get_gibbs_bloch(0.0, kT, dbeta)
    o = RhoBlochOracle(t=0.0, X_gridDIM=64, X_amplitude=XA, V0=V0, K="0.5 * P * P", V=V_C, dt=0.01, kT=kT, dbeta=dbeta)
    r = o.get_gibbs_state()
    r = r / np.trace(r)
    assert np.linalg.norm(loop - r) / np.linalg.norm(r) < 1e-12


def test_split_operator_gibbs_state_converges_to_the_band_gibbs_state_at_second_order():
    q = lattice(64)
    exact = q.get_gibbs(0.0, 0.5, n=64)
    err = [np.linalg.norm(q.get_gibbs_bloch(0.0, 0.5, db) - exact) / np.linalg.norm(exact) for db in (0.02, 0.01)]
    assert err[0] < 1e-5
    assert 3.6 < err[0] / err[1] < 4.4
