"""Host logic of the request loop (no GPU): the seeded request stream and the pool memory model."""
import numpy as np


def test_stream_is_seeded_and_well_formed():
    from accuratewigner_gb300.serve import make_stream

    a = make_stream(200, rate=50.0, seed=3)
    b = make_stream(200, rate=50.0, seed=3)
    assert [(r.kind, r.n, r.steps, r.coeffs, r.arrival) for r in a] == [(r.kind, r.n, r.steps, r.coeffs, r.arrival)
                                                                        for r in b]
    arr = np.array([r.arrival for r in a])
    assert np.all(np.diff(arr) > 0)
    # mean inter-arrival close to 1 / rate
    assert 0.6 / 50 < np.mean(np.diff(arr)) < 1.6 / 50
    assert {r.kind for r in a} == {"wm", "vn", "rb"}
    assert {r.n for r in a} <= {128, 256, 512, 1024, 2048}
    assert all(100 <= r.steps <= 5000 for r in a)
    assert all(r.coeffs[0] > 0 and r.coeffs[2] >= 0 for r in a)


def test_pool_memory_grows_with_side_and_slots():
    from accuratewigner_gb300.serve import amplitude, pool_bytes

    assert pool_bytes("wm", 2048, 2) > pool_bytes("wm", 1024, 2) > pool_bytes("wm", 1024, 1)
    assert pool_bytes("vn", 512, 4) > pool_bytes("wm", 512, 4)
    # dX dP = 2 pi / n with equal amplitudes
    for n in (128, 2048):
        a = amplitude(n)
        assert abs((2 * a / n) ** 2 - 2 * np.pi / n) < 1e-12


class _FakePool:
    """Runs a request at once on the host: complex128 gives the state `base`, complex64 the same state
    with a relative error `c64_err`; records every request it was given."""

    def __init__(self, engine, precision, base, c64_err, log):
        self.engine, self.precision, self.base, self.c64_err, self.log = engine, precision, base, c64_err, log

    def submit(self, r):
        import numpy as np

        self.log.append(r)
        state = self.base * (1.0 + (self.c64_err if self.precision == "c64" else 0.0))
        r.start = 0.0
        r.steps_done = r.steps
        r.history = [np.full((r.steps, 3), 1.0 if self.precision == "c64" else 2.0)]
        r.state = state
        r.rho = state
        r.purity = 0.5
        r.done = 1.0
        (r.on_done or self.engine._finished)(r)


def _auto_engine(c64_err, fallback="c128"):
    import numpy as np

    from accuratewigner_gb300.serve import Engine

    eng = Engine(precision="auto", fallback=fallback)
    log = []
    base = np.ones((4, 4), np.complex128)
    eng.pool = lambda kind, n, precision=None: _FakePool(eng, precision, base, c64_err, log)
    return eng, log


def test_auto_falls_back_to_complex128_on_the_measured_error():
    """A request whose extrapolated complex64 error exceeds its tolerance continues in complex128
    from the complex128 probe's state; the estimate is recorded."""
    from accuratewigner_gb300.serve import C64_GROWTH, PROBE_STEPS, Request

    eng, log = _auto_engine(c64_err=1e-6)
    tight = Request(0, "wm", 128, 1000, (0.5, 0.0, 0.0), tol=2e-6)
    eng.submit(tight)
    assert [r.precision for r in log] == ["c64", "c128", "c128"]
    assert [r.steps for r in log] == [PROBE_STEPS, PROBE_STEPS, 1000 - PROBE_STEPS]
    assert log[2].init_rho is log[1].rho  # continued from the complex128 probe
    assert tight.fell_back and tight.precision == "c128"
    assert abs(tight.est_error - 1e-6 * (1000 / PROBE_STEPS) ** C64_GROWTH) < 1e-12
    assert tight.steps_done == 1000 and tight.done is not None
    assert eng.finished == [tight]


def test_auto_keeps_complex64_within_tolerance():
    from accuratewigner_gb300.serve import PROBE_STEPS, Request

    eng, log = _auto_engine(c64_err=1e-6)
    loose = Request(1, "vn", 256, 1000, (0.5, 0.0, 0.0), tol=1e-3)
    eng.submit(loose)
    assert [r.precision for r in log] == ["c64", "c128", "c64"]
    assert log[2].init_rho is log[0].rho  # continued from the complex64 probe
    assert not loose.fell_back and loose.precision == "c64" and loose.est_error < 1e-3
    # the probe's observable rows come first, then the continuation's
    assert len(loose.history) == 2 and loose.history[0].shape[0] == PROBE_STEPS
    # a request no longer than the probe window ends with it
    eng2, log2 = _auto_engine(c64_err=1e-6)
    short = Request(2, "wm", 128, 50, (0.5, 0.0, 0.0), tol=1e-5)
    eng2.submit(short)
    assert [r.steps for r in log2] == [50, 50] and short.precision == "c64" and short.steps_done == 50


def test_auto_routes_unreachable_tolerances_to_complex128():
    from accuratewigner_gb300.serve import C64_MIN_TOL, Engine, Request

    eng = Engine(precision="auto")
    assert eng.precision_for(Request(0, "wm", 128, 50, (0.5, 0.0, 0.0), tol=C64_MIN_TOL / 2)) == "c128"
    assert eng.precision_for(Request(0, "wm", 128, 50, (0.5, 0.0, 0.0), tol=1e-5)) == "c64"
    assert Engine(precision="c128").precision_for(Request(0, "wm", 128, 50, (0.5, 0.0, 0.0))) == "c128"


def test_auto_falls_back_to_native_fp64_when_asked():
    """With fallback="c128-fp64" the complex128 probe and the continuation run in native FP64."""
    from accuratewigner_gb300.serve import PROBE_STEPS, Request

    eng, log = _auto_engine(c64_err=1e-6, fallback="c128-fp64")
    tight = Request(0, "vn", 256, 900, (0.5, 0.0, 0.0), tol=2e-6)
    eng.submit(tight)
    assert [r.precision for r in log] == ["c64", "c128-fp64", "c128-fp64"]
    assert [r.steps for r in log] == [PROBE_STEPS, PROBE_STEPS, 900 - PROBE_STEPS]
    assert tight.fell_back and tight.precision == "c128-fp64"
