"""Every configuration the tests, the bench and the request loop build passes the device-free check
(aw_check_config through check_config): keyword validation as in the constructors, and NVRTC
compilation for sm_103a of each module generated from the expression strings (phase tables, masks,
observable finalize and batch initial states; initial-condition and observable modules).  A broken
expression kernel fails here, on a machine without a GPU, instead of at construction on the GPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


@pytest.fixture(scope="module", autouse=True)
def lib():
    from accuratewigner_gb300 import _build, _lib

    if not os.path.exists(_lib.LIB_PATH):
        _build.build()
    return _lib.load()


def _classes():
    from accuratewigner_gb300 import (RhoBlochCUDA1D, RhoVNeumannCUDA1D, SchrodingerWignerCUDA1D, WignerBlochCUDA1D,
                                      WignerMoyalCUDA1D)

    return {"wm": WignerMoyalCUDA1D, "wb": WignerBlochCUDA1D, "vn": RhoVNeumannCUDA1D, "rb": RhoBlochCUDA1D,
            "sw": SchrodingerWignerCUDA1D}


def _golden_names():
    from golden_cases import CASES

    return sorted(CASES)


@pytest.mark.parametrize("name", _golden_names())
def test_golden_configurations(name):
    from accuratewigner_gb300 import check_config
    from golden_cases import CASES

    spec = CASES[name]
    assert check_config(_classes()[spec["kind"]], **dict(spec["params"])) is None


def test_shared_test_cases():
    from accuratewigner_gb300 import check_config
    from _cases import SW, VN, WM_ANHARMONIC, WM_STRONG_FIELD

    c = _classes()
    for cls, p in ((c["wm"], WM_ANHARMONIC), (c["wm"], WM_STRONG_FIELD), (c["vn"], VN), (c["sw"], SW)):
        check_config(cls, **p)
    check_config(c["wm"], extra_observables=("X * X", "P * P"), **WM_ANHARMONIC)


@pytest.mark.parametrize("precision", ["c128", "c64", "c128-fp64"])
def test_headline_configuration(precision):
    import bench
    from accuratewigner_gb300 import check_config

    c = _classes()
    check_config(c["wm"], precision=precision, **bench.PARAMS)
    # the Gibbs state it starts from
    gibbs = {k: v for k, v in bench.PARAMS.items() if k not in ("diff_K", "diff_V", "abs_boundary_x")}
    check_config(c["wb"], kT=1.0, dbeta=0.05, precision="c128", **gibbs)


def test_batch_and_large_configurations():
    from accuratewigner_gb300 import check_config

    c = _classes()
    base = dict(t=0.0, X_gridDIM=512, P_gridDIM=512, X_amplitude=10.0, P_amplitude=8.0, K="0.5 * P * P",
                V="a * X * X * X * X - b * X * X", dt=0.01, dbeta=0.01, kT=1.0, t_initial=0.0)
    check_config(c["wb"], n_inst=64, batch_params=["a", "b"], batch_init="1.", **base)
    vn = dict(t=0.0, dt=0.02, X_gridDIM=4096, X_amplitude=80.0, D=0.18, alpha=1.0, xm=1.4, K="0.5 * P * P",
              V="D * pow(1. - exp(-alpha * (X - xm)), 2) + X * 0.02 * sin(0.01 * t)", diff_K="P",
              diff_V="2. * D * alpha * exp(-alpha * (X - xm)) * (1. - exp(-alpha * (X - xm))) + 0.02 * sin(0.01 * t)")
    check_config(c["vn"], **vn)


@pytest.mark.parametrize("kind", ["wm", "vn", "rb"])
def test_request_loop_pools(kind):
    from accuratewigner_gb300 import check_config, serve

    n = 256
    a = serve.amplitude(n)
    kw = dict(t=0.0, dt=0.01, X_gridDIM=n, X_amplitude=a, K="0.5 * P * P", V=serve.V_EXPR, precision="c128")
    if kind == "wm":
        kw.update(P_gridDIM=n, P_amplitude=a, diff_K="P", diff_V=serve.DV_EXPR)
    elif kind == "rb":
        kw.update(kT=1.0, dbeta=0.01, t_initial=0.0)
    check_config(serve.CLASSES[kind], n_inst=8, batch_params=list(serve.PARAMS), batch_init=serve.INIT[kind], **kw)


def test_errors_surface_as_the_constructor_raises_them():
    from accuratewigner_gb300 import check_config
    from _cases import WM_ANHARMONIC

    wm = _classes()["wm"]
    with pytest.raises(RuntimeError, match="undefined"):
        check_config(wm, **dict(WM_ANHARMONIC, V="0.5 * X * X + undefined_name * X"))
    with pytest.raises(RuntimeError, match="undefined"):
        check_config(wm, **dict(WM_ANHARMONIC, diff_V="X + no_such_function(X)"))
    with pytest.raises(AssertionError, match="power of two"):
        check_config(wm, **dict(WM_ANHARMONIC, X_gridDIM=100))
    with pytest.raises(AttributeError, match="dt"):
        check_config(wm, **{k: v for k, v in WM_ANHARMONIC.items() if k != "dt"})
    # the check leaves construction as it was: a later constructor call makes a real handle again
    from accuratewigner_gb300 import _common

    assert getattr(_common._CHECK, "arch", None) is None


def test_native_validation_without_a_device():
    """The argument checks of aw_create, reached through the device-free check."""
    from accuratewigner_gb300 import check_config
    from _cases import VN, WM_ANHARMONIC

    c = _classes()
    small = dict(WM_ANHARMONIC, X_gridDIM=16)
    with pytest.raises(AssertionError, match="grid sides"):
        check_config(c["wm"], **small)
    with pytest.raises(AssertionError, match="taken by the kernels"):
        check_config(c["wm"], n_inst=4, batch_params=["X"], batch_init="1.", **WM_ANHARMONIC)
    with pytest.raises(AssertionError, match="not an identifier"):
        check_config(c["wm"], n_inst=4, batch_params=["2a"], batch_init="1.", **WM_ANHARMONIC)
    with pytest.raises(AssertionError, match="do not depend on t"):
        check_config(c["wm"], n_inst=4, batch_params=["a"], batch_init="1.",
                     **dict(WM_ANHARMONIC, V="0.5 * X * X + a * X * sin(t)"))
    with pytest.raises(AssertionError, match="trace and purity only"):
        check_config(c["vn"], n_inst=4, batch_params=["a"], batch_init="1.", **VN)
    # a batch whose per-instance constants appear in V, K and the initial state
    check_config(c["wm"], n_inst=4, batch_params=["a"], batch_init="exp(-a * X * X - P * P)",
                 **dict(WM_ANHARMONIC, V="0.5 * a * X * X"))


def test_size_limits():
    """Grid sides from 32 to 8192 (the von Neumann Wigner grid, 2N, up to 8192); wave functions up to 2^25."""
    from accuratewigner_gb300 import check_config
    from _cases import SW, VN, WM_ANHARMONIC

    c = _classes()
    check_config(c["wm"], **dict(WM_ANHARMONIC, X_gridDIM=8192, P_gridDIM=32))
    with pytest.raises(AssertionError, match="grid sides"):
        check_config(c["wm"], **dict(WM_ANHARMONIC, X_gridDIM=16384))
    check_config(c["vn"], **dict(VN, X_gridDIM=4096))
    with pytest.raises(AssertionError, match="grid sides"):
        check_config(c["vn"], **dict(VN, X_gridDIM=8192))
    check_config(c["sw"], **dict(SW, X_gridDIM=2 ** 25))
    with pytest.raises(AssertionError):
        check_config(c["sw"], **dict(SW, X_gridDIM=2 ** 26))


def test_benchmark_configuration_parity_cases():
    """The benchmark-size parity configurations (plain 256^2, strong field 1024^2, capped-Morse von
    Neumann 4096^2) compile for sm_103a."""
    from accuratewigner_gb300 import check_config
    from test_baseline_configs_gpu import FIELD_C, PLAIN, STRONG, VN4096

    c = _classes()
    check_config(c["wm"], **PLAIN)
    check_config(c["wm"], precision="c64", **PLAIN)
    check_config(c["wm"], functions=FIELD_C, **STRONG)
    check_config(c["vn"], **VN4096)
