import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libawigner.so")


def pytest_collection_modifyitems(config, items):
    # GPU tests need a device; everything else must pass on the CPU-only build host
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(params=["c128", "c128-fp64"])
def c128_engine(request, monkeypatch):
    """Runs a complex128 parity test with both pass engines: double-float and native FP64."""
    import accuratewigner_gb300._common as common

    monkeypatch.setattr(common, "DEFAULT_PRECISION", request.param)
    return request.param


def rel_l2(a, b):
    import numpy as np

    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def obs_close(a, b, tol, scale=1.0):
    """Observable histories agree to `tol` relative to max(|b|, scale).

    Observables that pass through zero (a centred <x>) are compared against
    their natural scale (order one in atomic units) instead of their own size.
    """
    import numpy as np

    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    if a.shape != b.shape:
        return False
    ref = max(float(np.abs(b).max()) if b.size else 0.0, scale)
    return float(np.abs(a - b).max()) <= tol * ref
