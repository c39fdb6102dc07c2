"""The GPU library against golden vectors made by the reference's own kernel code."""
import pytest

from golden_cases import CASES, compare, load_golden, run_ops

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("c128_engine")]

TOL = 1e-10  # complex128 state, either pass engine


def _gpu_cls(kind):
    import accuratewigner_gb300 as aw

    return {"wm": aw.WignerMoyalCUDA1D, "wb": aw.WignerBlochCUDA1D, "vn": aw.RhoVNeumannCUDA1D,
            "rb": aw.RhoBlochCUDA1D, "sw": aw.SchrodingerWignerCUDA1D}[kind]


@pytest.mark.parametrize("name", sorted(n for n, spec in CASES.items() if spec.get("gpu", True)))
def test_gpu_matches_reference_kernels(name):
    spec = CASES[name]
    obj = _gpu_cls(spec["kind"])(**spec["params"])
    got = run_ops(obj, spec)
    bad = compare(got, load_golden(name), TOL)
    assert not bad, bad


# The golden cases held on the CPU oracle only: the ordered von Neumann averages at the plain bar, and the
# Wigner-Bloch / rho-Bloch ground states at 1e-8 (their loops end on purity thresholds, wb:178 and rb:184,
# that rounding in the last digits can move by a step; the reference's dbeta-halving rollback is part of
# what is compared).
GROUND_TOL = 1e-8


@pytest.mark.parametrize("name", sorted(n for n, spec in CASES.items() if not spec.get("gpu", True)))
def test_gpu_matches_reference_kernels_cpu_only_cases(name):
    spec = CASES[name]
    obj = _gpu_cls(spec["kind"])(**spec["params"])
    got = run_ops(obj, spec)
    tol = GROUND_TOL if any(op[0] == "ground_state" for op in spec["ops"]) else TOL
    bad = compare(got, load_golden(name), tol)
    assert not bad, bad
