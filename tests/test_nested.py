"""Nested unbinding (RecursiveUnbind, src/subhalo_unbind.cpp:810-841) as one
batch per depth: the batching reproduces the reference's depth-first
recursion exactly (CPU, with the oracle as the unbinder), and the GPU gives
the oracle's results through it."""
import numpy as np
import pytest

from hbtg import abi, nested, oracle, synthetic


def _params():
    return abi.parity_params(dm_only=1, box_size=100.0)


def test_depths():
    assert list(nested.depths([-1, 0, 0, 1, 3, -1])) == [0, 1, 1, 2, 3, 0]
    with pytest.raises(ValueError):
        nested.depths([1, 0])


def test_depth_batches_match_the_recursion_on_the_oracle():
    parts, members, parent, frames = synthetic.nested_system(seed=2, n_host=6000, n_sat=4, n_subsat=2)
    prm = _params()
    fn = lambda inp, p: oracle.run_port(inp, p, nthreads=1)
    a = nested.unbind_nested(fn, parts, members, parent, frames, prm)
    b = nested.unbind_recursive_reference(fn, parts, members, parent, frames, prm)
    for ra, rb in zip(a, b):
        assert np.array_equal(ra.members, rb.members)
        assert ra.nbound == rb.nbound and ra.status == rb.status and ra.mbound == rb.mbound
    # the host received its satellites' unbound particles
    assert len(a[0].members) > len(members[0])


@pytest.mark.gpu
def test_gpu_nested_matches_oracle(unbinder):
    parts, members, parent, frames = synthetic.nested_system(seed=3, n_host=20_000, n_sat=6, n_subsat=3)
    prm = _params()
    gpu = nested.unbind_nested(lambda inp, p: unbinder.unbind(inp, p), parts, members, parent, frames, prm)
    ref = nested.unbind_nested(lambda inp, p: oracle.run_port(inp, p), parts, members, parent, frames, prm)
    mism = tot = 0
    for g, r in zip(gpu, ref):
        assert g.status == r.status
        bg, br = set(parts.id[g.members[:g.nbound]]), set(parts.id[r.members[:r.nbound]])
        mism += len(bg ^ br)
        tot += len(br)
    # the plain path's bars: membership 1e-4, bound mass 1e-5
    assert mism <= max(1, 1e-4 * tot), (mism, tot)
    m_g = sum(g.mbound for g in gpu)
    m_r = sum(r.mbound for r in ref)
    assert abs(m_g - m_r) <= 1e-5 * m_r
