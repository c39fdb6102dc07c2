"""The TMA-staged column pass against the per-thread-load form.

The column pass that replaces the reference's strided axis-0 cuFFT plan (cufft.py:274-307, used at
wigner_moyal_cuda_1d.py:550,555 and rho_vneumann_cuda_1d.py:457,462) can stage its tile of whole
columns in shared memory by TMA tensor copies.  Only the movement of the tile changes, so both forms
must give bit-identical states and observables; the autotuner's choice between them must never show
in a result.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NAMES = ("X_average", "X_average_RHS", "P_average", "P_average_RHS", "hamiltonian_average")


def _form(obj, lines, tma):
    """Set the column pass's width and TMA staging (shapes as tuned); return them as in force."""
    import ctypes

    from accuratewigner_gb300 import _lib

    put = (ctypes.c_int32 * 4)(lines, tma, -1, -1)
    got = (ctypes.c_int32 * 4)()
    _lib.check(_lib.load().aw_pass_form(obj._h, put, got))
    return got[0], got[1]


def _run_wm(precision, n, lines, tma, steps=6):
    from accuratewigner_gb300 import WignerMoyalCUDA1D

    p = dict(t=0.0, dt=0.01, X_gridDIM=n, X_amplitude=10.0, P_gridDIM=n, P_amplitude=8.0, K="0.5 * P * P",
             V="0.5 * X * X + 0.05 * X * X * X * X", diff_K="P", diff_V="X + 0.2 * X * X * X", precision=precision)
    g = WignerMoyalCUDA1D(**p)
    assert _form(g, lines, tma) == (lines, tma)
    g.set_wignerfunction("exp(-pow(X - 1., 2) - P * P) / M_PI")
    g.propagate(steps)
    out = g.wignerfunction.get(), g.rho.get(), {k: np.array(getattr(g, k)) for k in NAMES}
    g.close()
    return out


@pytest.mark.parametrize("precision", ["c128", "c128-fp64", "c64"])
@pytest.mark.parametrize("n", [256, 1024])
def test_wigner_moyal_tma_column_pass_is_bit_identical(precision, n):
    lines = 2  # a multiple of 16 bytes per tile row for every element size
    W0, r0, o0 = _run_wm(precision, n, lines, 0)
    W1, r1, o1 = _run_wm(precision, n, lines, 1)
    assert np.array_equal(W0, W1) and np.array_equal(r0, r1)
    for k in NAMES:
        assert np.array_equal(o0[k], o1[k]), k


@pytest.mark.parametrize("precision,lines", [("c128", 1), ("c128-fp64", 1), ("c64", 2)])
def test_von_neumann_4096_tma_column_pass_is_bit_identical(precision, lines):
    from test_baseline_configs_gpu import VN4096, vn4096_rho0

    from accuratewigner_gb300 import RhoVNeumannCUDA1D

    out = []
    rho0 = vn4096_rho0()
    for tma in (0, 1):
        g = RhoVNeumannCUDA1D(precision=precision, **VN4096)
        assert _form(g, lines, tma) == (lines, tma)
        g.set_rho(rho0)
        g.propagate(2)
        out.append((g.rho.get(), {k: np.array(getattr(g, k)) for k in NAMES}))
        g.close()
    (r0, o0), (r1, o1) = out
    assert np.array_equal(r0, r1)
    for k in NAMES:
        assert np.array_equal(o0[k], o1[k]), k


def test_col_form_rejects_misaligned_tma_rows():
    """A complex64 tile of one column has 8-byte rows: TMA boxes need 16."""
    import ctypes

    from accuratewigner_gb300 import WignerMoyalCUDA1D, _lib

    g = WignerMoyalCUDA1D(t=0.0, dt=0.01, X_gridDIM=64, X_amplitude=8.0, P_gridDIM=64, P_amplitude=7.0,
                          K="0.5 * P * P", V="0.5 * X * X", precision="c64")
    lib = _lib.load()
    assert lib.aw_pass_form(g._h, (ctypes.c_int32 * 4)(1, 1, -1, -1), None) == _lib.AW_E_ARG
    assert b"16 bytes" in lib.aw_last_error()
    assert lib.aw_pass_form(g._h, (ctypes.c_int32 * 4)(3, -1, -1, -1), None) == _lib.AW_E_ARG
    assert lib.aw_pass_form(g._h, (ctypes.c_int32 * 4)(-1, -1, 2, -1), None) == _lib.AW_E_ARG
    g.close()


@pytest.mark.parametrize("precision", ["c128", "c128-fp64", "c64"])
def test_autotuned_shapes_stay_within_rounding_of_each_other(precision):
    """The row and column shapes (elements a thread, so radix-4 or radix-8 stages) change only the
    FFT's rounding: every combination agrees with every other far inside the parity tolerance, and
    the forms the autotuner chose are reported."""
    import ctypes

    from accuratewigner_gb300 import WignerMoyalCUDA1D, _lib

    lib = _lib.load()
    p = dict(t=0.0, dt=0.01, X_gridDIM=512, X_amplitude=10.0, P_gridDIM=512, P_amplitude=8.0, K="0.5 * P * P",
             V="0.5 * X * X + 0.05 * X * X * X * X", diff_K="P", diff_V="X + 0.2 * X * X * X", precision=precision)
    tol = 1e-5 if precision == "c64" else 1e-12
    runs = []
    for row_shape in (0, 1):
        for col_shape in (0, 1):
            g = WignerMoyalCUDA1D(**p)
            got = (ctypes.c_int32 * 4)()
            _lib.check(lib.aw_pass_form(g._h, None, got))
            assert got[0] >= 1 and got[1] in (0, 1) and got[2] in (0, 1) and got[3] in (0, 1)
            # the column width 2 has a kernel in both shapes at 512 points for every element size
            _lib.check(lib.aw_pass_form(g._h, (ctypes.c_int32 * 4)(2, 0, col_shape, row_shape), None))
            g.set_wignerfunction("exp(-pow(X - 1., 2) - P * P) / M_PI")
            g.propagate(20)
            runs.append((g.wignerfunction.get(), np.array(g.X_average)))
            g.close()
    W0, x0 = runs[0]
    for W, x in runs[1:]:
        assert np.linalg.norm(W - W0) / np.linalg.norm(W0) < tol
        assert np.max(np.abs(x - x0)) < tol
