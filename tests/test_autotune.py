"""Launch settings and the autotuner (hbtg_tuning, hbtg_autotune): every
setting gives the same results, bit for bit, and the autotuner keeps the
fastest on the handle and leaves the batch's in/out frames as it found them."""
import numpy as np
import pytest

from hbtg import abi, synthetic

FIELDS = ("order", "nbound", "mbound", "status", "iterations", "energy", "ref_pos", "ref_vel", "tracer_index",
          "most_bound_id", "kinematics", "core")


def _run(u, db, params):
    db.reset_inout()
    u.unbind_device(params, db.c)
    return db.outputs()


@pytest.mark.gpu
def test_every_launch_setting_gives_the_same_results(unbinder):
    from hbtg.gpu import DeviceBatch
    inp = synthetic.batched(total=300_000, seed=41, nmax=60_000)
    params = abi.parity_params(dm_only=1, box_size=500.0)
    db = DeviceBatch(inp)
    default = unbinder.tuning()
    assert (default["block_sort_max"], default["walk_ranged_min"], default["moments_blocks_per_sm"]) == (8192, 0, 8)
    ref = _run(unbinder, db, params)
    try:
        for setting in ((0, 0, 8), (2048, 1 << 30, 4), (8192, 1024, 1), (8192, 0, 32)):
            unbinder.set_tuning(*setting)
            got = _run(unbinder, db, params)
            for k in FIELDS:
                assert np.array_equal(getattr(got, k), getattr(ref, k)), (setting, k)
    finally:
        unbinder.set_tuning(default["block_sort_max"], default["walk_ranged_min"], default["moments_blocks_per_sm"])


@pytest.mark.gpu
def test_autotune_keeps_the_fastest_and_restores_the_frames(unbinder):
    from hbtg.gpu import DeviceBatch
    inp = synthetic.batched(total=300_000, seed=42, nmax=60_000)
    params = abi.parity_params(dm_only=1, box_size=500.0)
    db = DeviceBatch(inp)
    default = unbinder.tuning()
    ref = _run(unbinder, db, params)
    try:
        db.reset_inout()
        frames = {k: getattr(db, k).clone() for k in ("ref_pos", "ref_vel", "mbp", "mbv", "mbid")}
        report = unbinder.autotune(params, db.c)
        assert len(report) == 12 and all(r["ms"] > 0 for r in report)
        best = min(report, key=lambda r: r["ms"])
        chosen = unbinder.tuning()
        assert (chosen["block_sort_max"], chosen["walk_ranged_min"], chosen["moments_blocks_per_sm"]) == (
            best["block_sort_max"], best["walk_ranged_min"], best["moments_blocks_per_sm"])
        for k, v in frames.items():  # the inputs again
            assert bool((getattr(db, k) == v).all()), k
        got = _run(unbinder, db, params)
        for k in FIELDS:
            assert np.array_equal(getattr(got, k), getattr(ref, k)), k
    finally:
        unbinder.set_tuning(default["block_sort_max"], default["walk_ranged_min"], default["moments_blocks_per_sm"])


def test_tuning_struct_layout():
    t = abi.CTuning(2048, 7, 4, 1.5)
    assert abi.C.sizeof(t) == 24 and t.as_dict()["walk_ranged_min"] == 7
