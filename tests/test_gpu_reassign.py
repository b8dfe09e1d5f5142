"""GPU particle reassignment (hbtg_reassign_particles): the moves of
SubhaloSnapshot_t::ReassignParticles (src/subhalo_reassign_gas.cpp:65-197)
with GeoTree_t::NearestNeighbours (src/geometric_tree.cpp:108-142), through
the C ABI, against the reference's own neighbour search (golden) and the
oracle."""
import importlib.util
import os

import numpy as np
import pytest

from hbtg import abi, oracle, synthetic

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _golden():
    path = os.path.join(HERE, "golden", "reassign_fof.npz")
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "golden", "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.load_reassign(path)


def test_gpu_reassignment_matches_reference_golden(unbinder):
    inp, group_off, prm, ref = _golden()
    for k, dest in ref.items():
        got = unbinder.reassign(inp, group_off, prm, k)
        assert np.array_equal(got, dest), (k, np.nonzero(got != dest)[0][:10], (got != dest).sum())


def test_gpu_reassignment_vs_oracle_wrapped_groups(unbinder):
    """More and larger groups, some straddling the periodic box faces."""
    inp, group_off = synthetic.fof_groups(seed=7, n_groups=12, n_sat=4, box=40.0, swap=0.15)
    prm = abi.parity_params(thermal=1, box_size=40.0)
    for k in (10, 24):
        got = unbinder.reassign(inp, group_off, prm, k)
        ref = oracle.reassign(inp, group_off, prm, k)
        assert (ref >= 0).sum() > 50
        assert np.array_equal(got, ref), (k, (got != ref).sum())


def test_gpu_reassignment_rejects_bad_arguments(unbinder):
    from hbtg.gpu import UnbindError
    inp, group_off, prm, _ = _golden()
    with pytest.raises(UnbindError):
        unbinder.reassign(inp, group_off, prm, 33)  # more neighbours than the search keeps
    with pytest.raises(UnbindError):
        unbinder.reassign(inp, group_off[:-1], prm, 10)  # groups do not cover the subhaloes
