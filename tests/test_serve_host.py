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


def test_auto_precision_routes_by_the_error_model():
    from accuratewigner_gb300.serve import Engine, Request, c64_error

    eng = Engine(precision="auto")
    short = Request(0, "wm", 128, 50, (0.5, 0.0, 0.0), tol=1e-5)
    long = Request(1, "wm", 2048, 5000, (0.5, 0.0, 0.0), tol=1e-5)
    loose = Request(2, "vn", 2048, 5000, (0.5, 0.0, 0.0), tol=1e-3)
    assert c64_error(128, 50) <= 1e-5 < c64_error(2048, 5000) <= 1e-3
    assert eng.precision_for(short) == "c64"
    assert eng.precision_for(long) == "c128"
    assert eng.precision_for(loose) == "c64"
    assert Engine(precision="c128").precision_for(short) == "c128"
