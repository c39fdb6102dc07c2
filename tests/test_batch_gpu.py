"""Batches on the GPU: every instance matches the same propagator run alone (single handle), and
an instance computes bit-identically whatever else is active in its batch."""
import numpy as np
import pytest

from conftest import obs_close, rel_l2

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("c128_engine")]

TOL = 1e-11


def r15(v):
    """The value a #define of the single propagator carries (%.15e)."""
    return float("%.15e" % v)


WB_BASE = dict(t=0.0, X_gridDIM=64, P_gridDIM=64, X_amplitude=6.0, P_amplitude=6.0, K="0.5 * P * P", dt=0.01,
               dbeta=0.01, t_initial=0.0)
WB_V = "a * X * X * X * X - b * X * X + 0.5 * X * X"


def test_wigner_bloch_batch_gibbs_matches_single():
    from accuratewigner_gb300 import WignerBlochCUDA1D
    from accuratewigner_gb300.batch import PropagatorBatch

    vals = [(0.05, 0.5), (0.08, 0.3), (0.03, 0.9)]
    kTs = [2.0, 1.0, 0.5]  # 50, 100, 200 steps: ordered by step count
    b = PropagatorBatch(WignerBlochCUDA1D, 3, params=("a", "b"), init="1.", V=WB_V, kT=1.0, **WB_BASE)
    for k, (a, bb) in enumerate(vals):
        b.set_params(k, [r15(a), r15(bb)])
    done, pur = b.gibbs(kTs)
    for k, (a, bb) in enumerate(vals):
        s = WignerBlochCUDA1D(V=WB_V, a=a, b=bb, kT=kTs[k], **WB_BASE)
        w = s.get_gibbs_state().get()
        assert done[k] == s.gibbs_steps_done
        assert rel_l2(b.wigner(k), w) < TOL, k
        assert abs(b.purity(k) - s.get_purity()) < TOL
    b.close()


WM_BASE = dict(t=0.0, dt=0.01, X_gridDIM=64, X_amplitude=7.0, P_gridDIM=64, P_amplitude=6.0, K="0.5 * P * P",
               diff_K="P")
WM_V = "c2 * X * X + c4 * X * X * X * X"
WM_DV = "2. * c2 * X + 4. * c4 * X * X * X"
WM_INIT = "exp(-pow(X - x0, 2) - pow(P - p0, 2))"
WM_VALS = [(0.5, 0.02, 1.0, 0.0), (0.3, 0.05, -0.5, 0.7), (0.8, 0.0, 0.2, -1.0)]


def _wm_batch():
    from accuratewigner_gb300 import WignerMoyalCUDA1D
    from accuratewigner_gb300.batch import PropagatorBatch

    b = PropagatorBatch(WignerMoyalCUDA1D, len(WM_VALS), params=("c2", "c4", "x0", "p0"), init=WM_INIT, V=WM_V,
                        diff_V=WM_DV, **WM_BASE)
    for k, v in enumerate(WM_VALS):
        b.set_params(k, [r15(x) for x in v])
    return b


def test_wigner_moyal_batch_matches_single():
    from accuratewigner_gb300 import WignerMoyalCUDA1D

    b = _wm_batch()
    b.init_state()
    b.propagate(20)
    for k, (c2, c4, x0, p0) in enumerate(WM_VALS):
        s = WignerMoyalCUDA1D(V=WM_V, diff_V=WM_DV, c2=c2, c4=c4, x0=x0, p0=p0, **WM_BASE)
        s.set_wignerfunction(WM_INIT)
        s.propagate(20)
        assert rel_l2(b.wigner(k), s.wignerfunction.get()) < TOL, k
        assert rel_l2(b.rho(k), s.rho.get()) < TOL, k
        h = b.history(k)
        for name, col in zip(("X_average", "X_average_RHS", "P_average", "P_average_RHS", "hamiltonian_average"),
                             range(5)):
            assert obs_close(h[:, col], getattr(s, name), TOL), (k, name)
    b.close()


def test_instance_is_bit_identical_alone_and_in_the_mix():
    b = _wm_batch()
    b.init_state()
    b.propagate(15)
    mixed = b.wigner(1), b.rho(1), b.history(1)
    # instance 1 again, now the only active one
    b.set_active([False, True, False])
    b.init_state(1, 1)
    b.propagate(15, 0, len(WM_VALS))
    alone = b.wigner(1), b.rho(1), b.history(1)
    for m, a in zip(mixed, alone):
        assert np.array_equal(m, a)
    b.close()


VN_BASE = dict(t=0.0, dt=0.01, X_gridDIM=64, X_amplitude=8.0, K="0.5 * P * P")
VN_V = "c2 * X * X + c4 * X * X * X * X"
VN_INIT = "exp(-pow(X - x0, 2) - pow(X_prime - x0, 2))"


def test_von_neumann_batch_matches_single():
    from accuratewigner_gb300 import RhoVNeumannCUDA1D
    from accuratewigner_gb300.batch import PropagatorBatch

    vals = [(0.2, 0.01, 0.5), (0.1, 0.03, -1.0)]
    b = PropagatorBatch(RhoVNeumannCUDA1D, 2, params=("c2", "c4", "x0"), init=VN_INIT, V=VN_V, **VN_BASE)
    for k, v in enumerate(vals):
        b.set_params(k, [r15(x) for x in v])
    b.init_state()
    b.propagate(25)
    for k, (c2, c4, x0) in enumerate(vals):
        s = RhoVNeumannCUDA1D(V=VN_V, c2=c2, c4=c4, x0=x0, **VN_BASE)
        s.set_rho(VN_INIT)
        s.propagate(25)
        assert rel_l2(b.rho(k), s.rho.get()) < TOL, k
        assert rel_l2(b.wigner(k), s.get_wignerfunction().get()) < TOL, k
    b.close()


def test_rho_bloch_batch_gibbs_matches_single():
    from accuratewigner_gb300 import RhoBlochCUDA1D
    from accuratewigner_gb300.batch import PropagatorBatch

    base = dict(t=0.0, dt=0.01, X_gridDIM=64, X_amplitude=8.0, K="0.5 * P * P", dbeta=0.01)
    vals = [(0.5,), (1.2,)]
    kTs = [1.0, 0.5]
    b = PropagatorBatch(RhoBlochCUDA1D, 2, params=("w",), init="double(i == j)", V="0.5 * w * w * X * X", kT=1.0,
                        **base)
    for k, v in enumerate(vals):
        b.set_params(k, [r15(x) for x in v])
    done, pur = b.gibbs(kTs)
    for k, (w,) in enumerate(vals):
        s = RhoBlochCUDA1D(V="0.5 * w * w * X * X", w=w, kT=kTs[k], **base)
        r = s.get_gibbs_state().get()
        assert done[k] == s.gibbs_steps_done
        assert rel_l2(b.rho(k), r) < TOL, k
    b.close()
