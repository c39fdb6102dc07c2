"""Grouped propagation: von Neumann propagators of different grid sizes, and a batch, advanced together
(aw_group_propagate): members of side up to 128 (complex64: 256) with one persistent launch per pass of a
step, larger ones through their own step loop on their own streams, concurrently.

* A member computes the same bits alone (a group of one) and in a group with others: its tiles run the
  same kernel code whichever other members share the launch.
* The grouped steps agree with the member's ordinary propagate() (rho_vneumann_cuda_1d.py:429-448, held
  to the oracle elsewhere) to rounding: both use radix-8 stages, in separately compiled kernels.  A
  larger member gives propagate()'s bits.
"""
import ctypes

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

INIT = ("exp(-sigma * pow(X - x0, 2) + cuda_complex(0., p0) * X) * "
        "exp(-sigma * pow(X_prime - x0, 2) - cuda_complex(0., p0) * X_prime)")
ROUNDING = {"c128": 1e-12, "c128-fp64": 1e-12, "c64": 1e-5}


def _own(n, precision):
    """True when a member of side n runs its own step loop instead of the grouped launches."""
    return n > (256 if precision == "c64" else 128)


def _params(n, k, precision):
    a = float(np.sqrt(np.pi * n / 2.0))
    return dict(t=0.0, dt=0.01, X_gridDIM=n, X_amplitude=a, sigma=0.5 + 0.1 * k, p0=0.3 * k, x0=0.2 * k,
                K="0.5 * P * P", V="0.5 * X * X + 0.01 * X * X * X * X", precision=precision)


def _radix8(obj, n, precision):
    """Row and column shapes of 8 elements a thread (the double-float 1024-point row defaults to 4)."""
    from accuratewigner_gb300 import _lib

    row = 1 if (precision == "c128" and n == 1024) else 0
    _lib.check(_lib.load().aw_pass_form(obj._h, (ctypes.c_int32 * 4)(-1, -1, 0, row), None))


@pytest.mark.parametrize("precision", ["c128", "c128-fp64", "c64"])
def test_group_of_sizes_alone_in_the_mix_and_against_propagate(precision):
    from accuratewigner_gb300 import RhoVNeumannCUDA1D
    from accuratewigner_gb300.batch import propagate_group

    sizes = [64, 128, 256, 1024]
    steps = 7

    def fresh(k, n):
        g = RhoVNeumannCUDA1D(**_params(n, k, precision))
        g.set_rho(INIT)
        return g

    group = [fresh(k, n) for k, n in enumerate(sizes)]
    propagate_group(group, 3)
    propagate_group(group, steps - 3)
    mixed = [(g.rho.get(), float(g.t)) for g in group]
    for g in group:
        g.close()
    for k, n in enumerate(sizes):
        # a group of one: the same bits as in the mix
        g = fresh(k, n)
        propagate_group([g], 3)
        propagate_group([g], steps - 3)
        assert float(g.t) == mixed[k][1]
        assert np.array_equal(g.rho.get(), mixed[k][0]), n
        g.close()
        if _own(n, precision):
            # a large member runs its own step loop: propagate()'s bits
            g = fresh(k, n)
            g.propagate(3)
            g.propagate(steps - 3)
            assert np.array_equal(g.rho.get(), mixed[k][0]), n
            g.close()
        # the ordinary step loop with the same radix: the same to rounding
        g = fresh(k, n)
        _radix8(g, n, precision)
        g.propagate(steps)
        assert float(g.t) == mixed[k][1]
        assert rel_l2(mixed[k][0], g.rho.get()) < ROUNDING[precision], n
        g.close()


def test_group_with_a_batch_member():
    """A batch of three 128 x 128 instances (their own constants) grouped with a 512 x 512 propagator."""
    from accuratewigner_gb300 import RhoVNeumannCUDA1D
    from accuratewigner_gb300.batch import PropagatorBatch, propagate_group

    def batch():
        p = _params(128, 0, "c128-fp64")
        for k in ("sigma", "p0", "x0"):
            p.pop(k)
        b = PropagatorBatch(RhoVNeumannCUDA1D, 3, params=("sigma", "p0", "x0"), init=INIT, **p)
        for s in range(3):
            b.set_params(s, [0.5 + 0.2 * s, 0.4 * s, -0.3 * s])
        b.init_state()
        return b

    def single():
        g = RhoVNeumannCUDA1D(**_params(512, 1, "c128-fp64"))
        g.set_rho(INIT)
        return g

    b, s1 = batch(), single()
    propagate_group([b, s1], 5)
    got = [b.rho(k) for k in range(3)]
    got_single = s1.rho.get()
    assert np.allclose(b.t, 0.05) and abs(float(s1.t) - 0.05) < 1e-15
    b.close()
    s1.close()
    b0 = batch()  # alone: the batch as a group of one
    propagate_group([b0], 5)
    for k in range(3):
        assert np.array_equal(b0.rho(k), got[k]), k
    b0.close()
    b1 = batch()  # the ordinary batched step loop
    _radix8(b1.prop, 128, "c128-fp64")
    b1.propagate(5)
    for k in range(3):
        assert rel_l2(got[k], b1.rho(k)) < 1e-12, k
    b1.close()
    s2 = single()
    _radix8(s2, 512, "c128-fp64")
    s2.propagate(5)
    assert rel_l2(got_single, s2.rho.get()) < 1e-12
    s2.close()


def test_group_rejects_what_it_does_not_run():
    from accuratewigner_gb300 import RhoVNeumannCUDA1D, WignerMoyalCUDA1D
    from accuratewigner_gb300.batch import propagate_group

    a = RhoVNeumannCUDA1D(**_params(64, 0, "c128"))
    b = RhoVNeumannCUDA1D(**_params(128, 1, "c64"))
    with pytest.raises(Exception, match="form"):
        propagate_group([a, b], 1)
    w = WignerMoyalCUDA1D(t=0.0, dt=0.01, X_gridDIM=64, X_amplitude=8.0, P_gridDIM=64, P_amplitude=7.0,
                          K="0.5 * P * P", V="0.5 * X * X")
    with pytest.raises(Exception, match="von Neumann"):
        propagate_group([a, w], 1)
    e = RhoVNeumannCUDA1D(diff_K="P", diff_V="X", **_params(64, 2, "c128"))
    with pytest.raises(Exception, match="observables"):
        propagate_group([a, e], 1)
    for g in (a, b, w, e):
        g.close()
