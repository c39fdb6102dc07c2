"""Handles give back all their device memory when they are closed."""
import pytest

pytestmark = pytest.mark.gpu


def test_create_and_close_leaves_no_device_memory_behind():
    import torch

    from _cases import WM_STRONG_FIELD
    from accuratewigner_gb300 import WignerBlochCUDA1D, WignerMoyalCUDA1D
    from accuratewigner_gb300.batch import PropagatorBatch

    def cycle():
        p = dict(WM_STRONG_FIELD)
        p["abs_boundary_x"] = "exp(-dt * 0.01 * (1. + sin(t)) * (XX * XX + XX_prime * XX_prime) / (XX_max * XX_max))"
        s = WignerMoyalCUDA1D(**p)
        s.set_wignerfunction("exp(-X * X - P * P) / M_PI")
        s.propagate(3)
        s.close()
        b = PropagatorBatch(WignerBlochCUDA1D, 4, params=("a",), init="1.", X_gridDIM=64, P_gridDIM=64,
                            X_amplitude=6.0, P_amplitude=6.0, V="a * X * X", K="0.5 * P * P", dt=0.01, dbeta=0.01,
                            kT=1.0, t_initial=0.0)
        for k in range(4):
            b.set_params(k, [0.5 + 0.1 * k])
        b.gibbs([1.0, 1.0, 0.5, 0.5])
        b.close()

    cycle()  # first use: modules, the autotuner cache and the context's own allocations
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(10):
        cycle()
    torch.cuda.synchronize()
    assert free0 - torch.cuda.mem_get_info()[0] < 4 << 20
