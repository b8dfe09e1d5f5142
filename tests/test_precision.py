"""The precision study (tests/precision_study.py) at a small size: the FP32
walk agrees with the FP64 tree to rounding, both agree with the FP64 direct
sum to the tree's approximation error, and the bound verdicts barely move."""
import pytest


@pytest.mark.gpu
def test_precision_study_small(unbinder):
    from precision_study import run
    res = run(unbinder, n_host=200_000, n_sat=20, n_subset=2000, seed=1)
    assert res["phi_rel_gpu_vs_fp64_tree"]["median"] <= 2e-6, res
    assert res["phi_rel_gpu_vs_fp64_tree"]["p99"] <= 1e-4, res
    assert res["phi_rel_gpu_vs_direct"]["median"] <= 3e-3, res
    assert res["phi_rel_fp64_tree_vs_direct"]["median"] <= 3e-3, res
    assert res["bound"]["flipped_mass_fraction"] <= 2e-3, res
