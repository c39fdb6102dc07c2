"""The NumPy oracle against golden vectors made by the reference's own kernel code (CPU)."""
import pytest

from golden_cases import CASES, compare, load_golden, run_ops

ORACLES = None


def _oracle_cls(kind):
    from oracle import propagators as p

    return {"wm": p.WignerMoyalOracle, "wb": p.WignerBlochOracle, "vn": p.RhoVNeumannOracle,
            "rb": p.RhoBlochOracle, "sw": p.SchrodingerWignerOracle}[kind]


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_reference_kernels(name):
    spec = CASES[name]
    obj = _oracle_cls(spec["kind"])(**spec["params"])
    got = run_ops(obj, spec)
    bad = compare(got, load_golden(name), 1e-12)
    assert not bad, bad
