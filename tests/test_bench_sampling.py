"""The benchmark's CPU sample (the subhaloes the CPU baseline, the reference
arm and the parity block run on): particle-weighted by size decade, the
largest decade always represented, shares close to the batch's, and the same
subhaloes for the same seed."""
import sys

import numpy as np

from conftest import ROOT

sys.path.insert(0, ROOT)


def _decade_shares(sizes):
    dec = np.floor(np.log10(np.maximum(sizes, 1))).astype(int)
    return {int(d): sizes[dec == d].sum() / sizes.sum() for d in np.unique(dec)}


def test_cpu_sample_is_particle_weighted_and_keeps_the_largest_decade():
    import bench
    inp, _ = bench.workload(2_000_000, 3, "batched")
    sample, picked = bench.cpu_sample(inp, 200_000, seed=5)
    sizes = np.diff(inp.offsets)
    got = np.diff(sample.offsets)
    assert np.array_equal(got, sizes[picked]) and np.all(np.diff(picked) > 0)
    top = int(np.floor(np.log10(sizes.max())))
    assert np.floor(np.log10(got.max())) == top  # the largest decade is in the sample
    # below the top decade (few, large subhaloes: taken whole), each decade
    # contributes about its share of the target particle count
    full = _decade_shares(sizes)
    dec = np.floor(np.log10(np.maximum(got, 1))).astype(int)
    for d, share in full.items():
        if share > 0.05 and d < top:
            want = 200_000 * share
            have = got[dec == d].sum()
            assert abs(have - want) < 0.5 * want + 10 ** (d + 1), (d, want, have)
    again, picked2 = bench.cpu_sample(inp, 200_000, seed=5)
    assert np.array_equal(picked, picked2)


def test_strict_cpu_sample_stays_within_its_share():
    import bench
    inp, _ = bench.workload(2_000_000, 3, "batched")
    small, picked = bench.cpu_sample(inp, 100_000, seed=1, strict=True)
    assert small.n_particles <= 1.5 * 100_000 * 1.0 + np.diff(inp.offsets).min()
