"""The Wigner-Moyal step loop replayed from CUDA graphs against the same loop on the streams.

aw_propagate runs windows of steps from captured graphs (the reference's per-step host loop,
wigner_moyal_cuda_1d.py:563-582, launches every kernel from Python).  The graph changes only how the
launches reach the GPU, so W, rho and every recorded observable must be bit-identical with and without
it: for a time-independent and a time-dependent potential (the kick tables are rebuilt between
windows), for odd and even step counts (the two captured branch-buffer patterns) and over several calls
(replays of the same graphs).
"""
import numpy as np
import pytest

from _cases import E_FIELD_C, WM_ANHARMONIC, WM_INIT, WM_STRONG_FIELD

pytestmark = pytest.mark.gpu

NAMES = ("X_average", "X_average_RHS", "P_average", "P_average_RHS", "hamiltonian_average")


def _run(params, precision, graph, calls):
    from accuratewigner_gb300 import WignerMoyalCUDA1D, _lib

    g = WignerMoyalCUDA1D(precision=precision, **params)
    _lib.check(_lib.load().aw_graph(g._h, int(graph)))
    g.set_wignerfunction(WM_INIT)
    for n in calls:
        g.propagate(n)
    out = g.wignerfunction.get(), g.rho.get(), {k: np.array(getattr(g, k)) for k in NAMES}, float(g.t)
    g.close()
    return out


@pytest.mark.parametrize("precision", ["c128", "c128-fp64", "c64"])
@pytest.mark.parametrize("case", ["anharmonic", "strong_field"])
def test_graph_windows_are_bit_identical_to_the_stream_loop(case, precision):
    params = dict(WM_ANHARMONIC) if case == "anharmonic" else dict(WM_STRONG_FIELD)
    calls = (50, 37, 20, 51, 50, 300)  # even and odd counts, remainders, replays, a call of two windows
    W0, r0, o0, t0 = _run(params, precision, False, calls)
    W1, r1, o1, t1 = _run(params, precision, True, calls)
    assert t0 == t1
    assert np.array_equal(W0, W1) and np.array_equal(r0, r1)
    for k in NAMES:
        assert o0[k].shape == (sum(calls),) and np.array_equal(o0[k], o1[k]), k


def test_graph_launch_count_matches_the_stream_loop():
    """The launches a replayed window makes are counted like the stream loop's."""
    from accuratewigner_gb300 import WignerMoyalCUDA1D, _lib

    counts = []
    for graph in (0, 1):
        g = WignerMoyalCUDA1D(**WM_ANHARMONIC)
        _lib.check(_lib.load().aw_graph(g._h, graph))
        g.set_wignerfunction(WM_INIT)
        g.propagate(40)  # captures
        n0 = _lib.launch_count()
        g.propagate(40)  # replays
        counts.append(_lib.launch_count() - n0)
        g.close()
    assert counts[0] == counts[1] > 0
