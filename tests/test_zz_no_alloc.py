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


@pytest.mark.parametrize("elem_bytes", [16, 8])
def test_noalloc_several_chunks_all_modes_against_numpy(elem_bytes):
    """Inputs of several 65536-element chunks plus a remainder, so that the per-chunk partials are
    written and then summed in order; every mode, complex128 and complex64, each call twice (a stale
    partial of the first call, or of the larger call before it, would show in the second)."""
    import torch

    from accuratewigner_gb300 import _lib

    lib = _lib.load()
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    rng = np.random.default_rng(11)
    ctype = np.complex128 if elem_bytes == 16 else np.complex64
    tdtype = torch.complex128 if elem_bytes == 16 else torch.complex64
    n_big = 5 * 65536 + 3
    n = 3 * 65536 + 17
    stride = 3
    host = (rng.standard_normal((n - 1) * stride + 1) + 1j * rng.standard_normal((n - 1) * stride + 1)).astype(ctype)
    dev = torch.from_numpy(host).to("cuda")
    big = torch.from_numpy((rng.standard_normal(n_big) + 1j * rng.standard_normal(n_big)).astype(ctype)).to("cuda")
    assert dev.dtype == tdtype
    a = host[:n].astype(np.complex128)
    diag = host[::stride][:n].astype(np.complex128)
    want = {0: (a.sum(), np.abs(a).sum()),
            1: (complex((a.real ** 2 - a.imag ** 2).sum()), (np.abs(a) ** 2).sum()),
            2: (complex((np.abs(a) ** 2).sum()), (np.abs(a) ** 2).sum()),
            3: (diag.sum(), np.abs(diag).sum())}
    for mode in range(4):
        # a larger call first leaves partials in chunks the next call does not use
        _reduce(lib, big.data_ptr(), elem_bytes, n_big, 1, mode, out)
        for _ in range(2):
            got = _reduce(lib, dev.data_ptr(), elem_bytes, n, stride if mode == 3 else 0, mode, out)
            ref, scale = want[mode]
            assert abs(got - ref) <= 1e-12 * scale, (mode, got, ref)


def test_noalloc_rejects_oversized_input():
    from accuratewigner_gb300 import _lib

    lib = _lib.load()
    import torch

    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    rc = lib.aw_reduce_noalloc(ctypes.c_void_p(out.data_ptr()), 16, 67108864 + 1, 0, 0,
                               ctypes.c_void_p(out.data_ptr()), None)
    assert rc == _lib.AW_E_ARG
    assert b"67108864" in lib.aw_last_error()
