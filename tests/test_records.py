"""Run records on the host: HHG spectrum, settings filter, record reader, ground-state cache logic."""
import os

import numpy as np
import pytest


def test_hhg_spectrum_is_the_reference_formula():
    signal = pytest.importorskip("scipy.signal")
    from scipy import fftpack

    from accuratewigner_gb300.records import hhg_spectrum

    dt, omega = 0.05, 0.057
    t = dt * np.arange(1, 40001)
    j = np.sin(omega * t) + 1e-3 * np.sin(3 * omega * t) + 1e-6 * np.cos(5.5 * omega * t)
    om, sp = hhg_spectrum(list(j), dt, omega)
    ref = np.abs(fftpack.fftshift(fftpack.fft(signal.windows.blackman(j.size) * j))) ** 2
    ref /= ref.max()
    ref_om = fftpack.fftshift(fftpack.fftfreq(j.size, dt / (2 * np.pi))) / omega
    assert np.allclose(om, ref_om, rtol=0, atol=1e-12)
    assert np.max(np.abs(sp - ref)) < 1e-13
    # the fundamental is the peak (bin width 0.055 omega here)
    assert abs(abs(om[np.argmax(sp)]) - 1.0) < 0.06


def test_settings_keep_numbers_strings_and_arrays_only():
    from accuratewigner_gb300.records import _storable

    assert _storable(1.5) is not None and _storable("0.5 * P * P") is not None
    assert _storable(np.arange(3)) is not None
    assert _storable(lambda self, t: t) is None
    assert _storable({"a": 1}) is None


def test_read_record_returns_the_groups(tmp_path):
    from accuratewigner_gb300.records import read_record

    d = tmp_path / "run"
    os.makedirs(d / "frames")
    np.savez(d / "settings.npz", X_wigner=np.arange(4.0), V=np.array("X * X"))
    for n in range(3):
        np.savez(d / "frames" / ("%d.npz" % n), wigner=np.full((2, 4), n, float), t=np.float64(0.1 * n),
                 prob=np.ones(2, complex))
    np.savez(d / "frames" / "3.tmp.npz", wigner=np.zeros(1))  # a write in progress is not a frame
    np.savez(d / "ehrenfest.npz", X_average=np.arange(5.0))
    r = read_record(str(d))
    assert sorted(r["frames"]) == [0, 1, 2]
    assert r["frames"][2]["wigner"][0, 0] == 2 and float(r["frames"][1]["t"]) == 0.1
    assert str(r["settings"]["V"]) == "X * X"
    assert np.array_equal(r["ehrenfest"]["X_average"], np.arange(5.0))


class _HostArray:
    def __init__(self, a):
        self.a = a

    def get(self):
        return self.a.copy()

    def set(self, v):
        self.a[...] = v


class _FakeBloch:
    """Host stand-in with the attributes and methods the cache uses."""

    def __init__(self, V="-1. / sqrt(X * X + 2.)"):
        self.X_gridDIM = self.P_gridDIM = 8
        self.X_amplitude, self.P_amplitude, self.dt, self.K, self.V = 5.0, 4.0, 0.01, "0.5 * P * P", V
        self.cuda_consts = "#define X_amplitude 5.0\n"
        self.rho = _HostArray(np.zeros((8, 8), complex))
        self.computed = 0
        self.rho2wigner_calls = 0

    def get_ground_state(self, abs_tol_purity=1e-12):
        self.computed += 1
        self.rho.set(np.arange(64.0).reshape(8, 8) + 1j)

    def rho2wigner(self):
        self.rho2wigner_calls += 1


def test_ground_state_cache_is_computed_once_and_keyed_by_the_hamiltonian(tmp_path):
    from accuratewigner_gb300.records import ground_state

    path = str(tmp_path / "ground_state_rho.npz")
    a = _FakeBloch()
    assert ground_state(a, path) == "computed" and a.computed == 1
    b = _FakeBloch()
    assert ground_state(b, path) == "loaded" and b.computed == 0 and b.rho2wigner_calls == 1
    assert np.array_equal(b.rho.get(), a.rho.get())
    c = _FakeBloch(V="-1. / sqrt(X * X + 1.37)")  # another potential: the cache does not apply
    assert ground_state(c, path) == "computed" and c.computed == 1
    with open(path, "wb") as f:  # a damaged file is recomputed
        f.write(b"not an npz")
    assert ground_state(_FakeBloch(), path) == "computed"
