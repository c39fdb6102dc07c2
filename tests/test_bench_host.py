"""Host-side pieces of bench.py's group workload: the side sets it parses, and the configuration of
every member it builds passes the device-free check (NVRTC for sm_103a) in each arithmetic form."""
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
