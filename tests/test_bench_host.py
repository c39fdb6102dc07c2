"""Host-side pieces of bench.py: the side sets of the group workload and the configuration of every
member it builds (the device-free check, NVRTC for sm_103a, in each arithmetic form), and the
roofline figures the headline line reads from the committed ncu summary."""
import pytest


def test_group_side_sets():
    import bench

    assert bench._group_sets("128,256,512,1024,2048") == [[128, 256, 512, 1024, 2048]]
    assert bench._group_sets("64x8;128,256x2;2048") == [[64] * 8, [128, 256, 256], [2048]]


@pytest.mark.parametrize("precision", ["c128", "c128-fp64", "c64"])
def test_group_members_compile(precision):
    import bench

    from accuratewigner_gb300 import RhoVNeumannCUDA1D, check_config

    for k, n in enumerate((64, 128, 256, 512, 2048)):
        assert check_config(RhoVNeumannCUDA1D, **bench.group_member_params(n, k, precision)) is None


def test_fp64_roofline_from_the_committed_counts():
    """A step's FP64 instructions are the row, column and marginal passes' (the launches made once a call
    are left out), against 2 FP64 lanes a clock a SM; only the native FP64 form has the figure."""
    import json
    import os

    import bench

    per = json.load(open(os.path.join(bench.ROOT, "profiles", "traffic_per_launch.json")))
    per = per["fp64_pipe"]["fp64_instructions_per_point"]
    inst = per["row_pass"] + per["column_pass"] + per["marginal_pass"]
    r = bench.fp64_roofline("c128-fp64", 2.25e9, {"sm_mhz": 2070.0}, sms=152)
    assert r["fp64_inst_per_point_step"] == pytest.approx(inst)
    assert r["peak_inst_per_s"] == pytest.approx(2.0 * 152 * 2070e6)
    assert r["frac"] == pytest.approx(inst * 2.25e9 / (2.0 * 152 * 2070e6))
    assert 0.5 < r["frac"] < 1.05
    assert bench.fp64_roofline("c128", 7.2e9, {"sm_mhz": 2070.0}, sms=152) is None
    assert bench.fp64_roofline("c128-fp64", 2.25e9, {}, sms=152) is None


@pytest.mark.parametrize("precision", ["c128", "c128-fp64", "c64"])
def test_traffic_per_launch_covers_every_pass(precision):
    import bench

    for kernel in bench.PASS_UNITS:
        t = bench.load_traffic(kernel, precision)
        assert isinstance(t, int) and t > 0, (kernel, precision)
