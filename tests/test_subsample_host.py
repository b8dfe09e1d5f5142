"""Host-side potential-subsampling preparation (no GPU needed): the library's
hbtg_prepare_subsampling reorders particles exactly as the reference's
PrepareParticlesForSubsampling, so preparing on the host and running the
oracle on the prepared particles reproduces the reference's own result."""
import glob
import importlib.util
import os

import numpy as np
import pytest

from hbtg import abi, oracle

HERE = os.path.dirname(os.path.abspath(__file__))


def _load(name):
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "golden", "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.load(os.path.join(HERE, "golden", name + ".npz"))


@pytest.mark.parametrize("name", ["subsampled_dmo", "subsampled_hydro"])
def test_host_preparation_reproduces_reference(name):
    from hbtg.build import build_library
    from hbtg import subsample
    build_library()
    inp, prm, ref = _load(name)
    prep, perm = subsample.prepare(inp, prm)
    p2 = abi.Params.from_buffer_copy(prm)
    p2.prepared_subsample = 1
    got = subsample.compose(oracle.run_port(prep, p2, nthreads=1, want_potential=True), inp, perm)
    for k in ("order", "nbound", "mbound", "energy", "ref_pos", "ref_vel", "most_bound_id", "tracer_index"):
        assert np.array_equal(getattr(got, k), getattr(ref, k)), k


def test_preparation_is_identity_without_subsampling():
    from hbtg.build import build_library
    from hbtg import subsample, synthetic
    build_library()
    inp = synthetic.small_cases(seed=0)
    perm = subsample.permutation(inp, abi.parity_params(dm_only=1))
    seg = np.repeat(np.arange(inp.n_sub), np.diff(inp.offsets))
    assert np.array_equal(perm, np.arange(inp.n_particles) - inp.offsets[:-1][seg])
