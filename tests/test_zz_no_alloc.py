"""aw_reduce_noalloc, the one entry point that allocates no device memory.

It serves callers that cannot allocate: an application that owns the whole
device memory budget and passes only pointers into its own pool, or a
latency-critical loop where cudaMalloc / cudaFree would synchronise the
device.  Its results must agree with the allocating entry points (aw_sum,
aw_purity, aw_trace) within the tolerance the parity tests use, on two calls
in a row (the static scratch keeps the previous call's contents).

This file sorts last so that a failure here comes after every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _reduce(lib, ptr, elem_bytes, n, stride, mode, out):
    rc = lib.aw_reduce_noalloc(ctypes.c_void_p(ptr), elem_bytes, n, stride, mode, ctypes.c_void_p(out.data_ptr()), None)
    assert rc == 0, lib.aw_last_error()
    import torch

    torch.cuda.synchronize()
    return complex(out[0].item(), out[1].item())


def test_noalloc_matches_sum_purity_trace_twice():
    import torch

    from accuratewigner_gb300 import RhoVNeumannCUDA1D, WignerMoyalCUDA1D, _lib

    lib = _lib.load()
    out = torch.zeros(2, dtype=torch.float64, device="cuda")  # the caller's output buffer
    rng = np.random.default_rng(7)

    wm = WignerMoyalCUDA1D(X_gridDIM=256, P_gridDIM=128, X_amplitude=8.0, P_amplitude=7.0, t=0.0, dt=0.01,
                           V="0.5 * X * X", K="0.5 * P * P")
    w = rng.standard_normal((128, 256)) + 1j * rng.standard_normal((128, 256))
    wm.wignerfunction.set(w)
    re, im = ctypes.c_double(), ctypes.c_double()
    assert lib.aw_sum(wm._h, _lib.AW_BUF_WIGNER, ctypes.byref(re), ctypes.byref(im)) == 0
    ref_sum = complex(re.value, im.value)
    ref_purity = wm.get_purity()
    for _ in range(2):
        s = _reduce(lib, wm.wignerfunction.ptr, 16, w.size, 0, 0, out)
        assert abs(s - ref_sum) <= TOL * max(1.0, abs(ref_sum))
        q = _reduce(lib, wm.wignerfunction.ptr, 16, w.size, 0, 1, out)
        purity = 2.0 * np.pi * q.real * wm.dXdP
        assert abs(purity - ref_purity) <= TOL * max(1.0, abs(ref_purity))

    vn = RhoVNeumannCUDA1D(X_gridDIM=128, X_amplitude=10.0, t=0.0, dt=0.01, V="0.5 * X * X", K="0.5 * P * P")
    vn.set_rho("exp(-pow(X - 0.5, 2) - pow(X_prime - 0.5, 2))")
    ref_tr = vn._trace()
    for _ in range(2):
        tr = _reduce(lib, vn.rho.ptr, 16, 128, 129, 3, out)
        assert abs(tr - ref_tr) <= TOL * max(1.0, abs(ref_tr))


def test_noalloc_rejects_oversized_input():
    from accuratewigner_gb300 import _lib

    lib = _lib.load()
    import torch

    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    rc = lib.aw_reduce_noalloc(ctypes.c_void_p(out.data_ptr()), 16, 67108864 + 1, 0, 0,
                               ctypes.c_void_p(out.data_ptr()), None)
    assert rc == _lib.AW_E_ARG
    assert b"67108864" in lib.aw_last_error()
