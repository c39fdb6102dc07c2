"""The continuous-batching request loop: every result is the same alone and in a mix."""
import numpy as np
import pytest

from conftest import obs_close, rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _requests(keep=True):
    from accuratewigner_gb300.serve import Request

    spec = [("wm", 64, 40, (0.5, 0.01, 0.02), 0.5, -0.3), ("vn", 64, 55, (0.3, 0.0, 0.01), -0.7, 0.4),
            ("rb", 64, 70, (0.8, 0.0, 0.0), 0.0, 0.0), ("wm", 128, 65, (0.2, -0.01, 0.03), 1.0, 0.5),
            ("wm", 64, 25, (0.9, 0.0, 0.0), -1.0, 1.0), ("vn", 128, 30, (0.6, 0.02, 0.0), 0.3, -0.8),
            ("rb", 64, 45, (0.4, 0.0, 0.02), 0.0, 0.0)]
    return [Request(i, k, n, s, c, x0, p0, arrival=0.0, keep_state=keep) for i, (k, n, s, c, x0, p0) in enumerate(spec)]


def test_results_are_the_same_alone_and_in_the_mix():
    from accuratewigner_gb300.serve import Engine

    slots = {64: 3, 128: 2}
    mix = _requests()
    eng = Engine(chunk=20, slots=slots)
    eng.run(mix, realtime=False)
    eng.close()
    for r in mix:
        assert r.done is not None and r.steps_done > 0
        alone = _requests()[r.rid]
        e1 = Engine(chunk=20, slots=slots)
        e1.run([alone], realtime=False)
        e1.close()
        assert alone.steps_done == r.steps_done
        assert rel_l2(r.state, alone.state) < TOL, (r.rid, r.kind)
        assert abs(r.purity - alone.purity) < TOL
        if r.kind == "wm":
            hm, ha = np.concatenate(r.history), np.concatenate(alone.history)
            assert hm.shape == ha.shape == (r.steps, hm.shape[1])
            for col in range(5):
                assert obs_close(hm[:, col], ha[:, col], TOL), (r.rid, col)


def test_served_wigner_moyal_matches_the_plain_propagator():
    from accuratewigner_gb300 import WignerMoyalCUDA1D
    from accuratewigner_gb300.serve import DV_EXPR, INIT, V_EXPR, Engine, amplitude

    r = [q for q in _requests() if q.kind == "wm"][0]
    eng = Engine(chunk=20, slots={64: 2, 128: 2})
    eng.run([r], realtime=False)
    eng.close()
    a = amplitude(r.n)
    c2, c3, c4 = r.coeffs
    s = WignerMoyalCUDA1D(t=0.0, dt=0.01, X_gridDIM=r.n, P_gridDIM=r.n, X_amplitude=a, P_amplitude=a,
                          K="0.5 * P * P", V=V_EXPR, diff_K="P", diff_V=DV_EXPR, c2=c2, c3=c3, c4=c4, x0=r.x0,
                          p0=r.p0)
    s.set_wignerfunction(INIT["wm"])
    for _ in range(r.steps // 20):
        s.propagate(20)
    s.propagate(r.steps % 20)
    assert rel_l2(r.state, s.wignerfunction.get()) < 1e-10
    h = np.concatenate(r.history)
    assert obs_close(h[:, 0], s.X_average, 1e-10)


def test_auto_precision_measures_the_complex64_error_and_falls_back():
    """An auto engine runs each request's probe window in complex64 and complex128, keeps complex64
    when the extrapolated measured error is within the request's tolerance, and otherwise falls back
    to complex128 from the complex128 probe's state (then the result is the complex128 one)."""
    from accuratewigner_gb300.serve import C64_MIN_TOL, Engine, Request

    def reqs():
        return [Request(0, "wm", 64, 400, (0.5, 0.01, 0.02), 0.5, -0.3, keep_state=True, tol=1e-3),
                Request(1, "vn", 64, 1000, (0.3, 0.0, 0.01), -0.7, 0.4, keep_state=True, tol=C64_MIN_TOL)]

    auto = reqs()
    eng = Engine(precision="auto", chunk=50, slots={64: 2})
    eng.run(auto, realtime=False)
    eng.close()
    ref = reqs()
    e2 = Engine(precision="c128", chunk=50, slots={64: 2})
    e2.run(ref, realtime=False)
    e2.close()
    loose, tight = auto
    assert loose.precision == "c64" and not loose.fell_back and loose.est_error <= loose.tol
    assert tight.precision == "c128" and tight.fell_back and tight.est_error > tight.tol
    for a, r in zip(auto, ref):
        assert a.steps_done == r.steps_done == a.steps
        assert rel_l2(a.state, r.state) <= a.tol, (a.rid, rel_l2(a.state, r.state))
    # the fallback continued the complex128 trajectory: the same as complex128 throughout
    assert rel_l2(tight.state, ref[1].state) < 1e-10
    hm, hr = np.concatenate(loose.history), np.concatenate(ref[0].history)
    assert hm.shape == hr.shape == (400, hm.shape[1])
