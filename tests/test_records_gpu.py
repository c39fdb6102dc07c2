"""Run records on the GPU: frames written asynchronously equal the synchronous reads, the Ehrenfest
series and settings are stored, and a cached ground state reloads bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PARAMS = dict(t=0.0, dt=0.05, X_gridDIM=128, X_amplitude=20.0, P_gridDIM=64, P_amplitude=4.0, kT=1.0, dbeta=0.05,
              F=0.04, omega=0.057, K="0.5 * P * P", diff_K="P",
              V="-1. / sqrt(X * X + 1.37) + X * F * sin(omega * t)",
              diff_V="X / pow(X * X + 1.37, 1.5) + F * sin(omega * t)")


def test_frames_ehrenfest_and_ground_state_cache(tmp_path):
    from accuratewigner_gb300 import WignerBlochCUDA1D
    from accuratewigner_gb300.records import RunRecord, ground_state, read_record

    cache = str(tmp_path / "ground_state_rho.npz")
    run = str(tmp_path / "run")
    s = WignerBlochCUDA1D(**PARAMS)
    assert ground_state(s, cache, abs_tol_purity=1e-8) == "computed"
    rho0, w0 = s.rho.get(), s.wignerfunction.get()
    sync = []
    with RunRecord(run, s, dict(PARAMS, E=lambda self, t: t)) as rec:
        for _ in range(4):
            s.propagate(15)
            rec.save_frame()
            sync.append((s.wignerfunction.get().real, float(s.t), s.rho.get().diagonal()))
    r = read_record(run)
    assert sorted(r["frames"]) == [0, 1, 2, 3]
    for n, (w, t, prob) in enumerate(sync):
        f = r["frames"][n]
        assert np.array_equal(f["wigner"], w) and float(f["t"]) == t and np.array_equal(f["prob"], prob)
    for name in ("X_average", "P_average", "X_average_RHS", "P_average_RHS", "hamiltonian_average"):
        assert np.array_equal(r["ehrenfest"][name], np.asarray(getattr(s, name)))
        assert r["ehrenfest"][name].size == 60
    assert np.array_equal(r["settings"]["X_wigner"], s.X) and str(r["settings"]["V"]) == PARAMS["V"]
    assert "E" not in r["settings"]
    s.close()

    s2 = WignerBlochCUDA1D(**PARAMS)
    assert ground_state(s2, cache) == "loaded"
    assert np.array_equal(s2.rho.get(), rho0)
    assert np.array_equal(s2.wignerfunction.get(), w0)
    s2.close()
