"""hbtg_unbind_batch_noalloc: the unbinding entry point for callers that cannot
allocate GPU memory (code running inside another library's allocation-free
section, under a device-memory pool that must not grow, or on a path where an
allocation's implicit synchronisation is unacceptable).  Its working memory is
a fixed reserve inside the library, so the test checks that it gives the same
results as the allocating entry point, on two calls in a row, and that device
memory does not change across a call.

This file is collected last so that a run stopping at its first failure has
already run every other test."""
import ctypes as C

import numpy as np
import pytest

from hbtg import abi, synthetic
from parity import assert_parity, check_invariants

pytestmark = pytest.mark.gpu

NOALLOC_MAX_PARTICLES = 1 << 16


def _batch():
    a = synthetic.small_cases(seed=4)
    b = synthetic.batched(n_sub=400, seed=9, nmax=3000, box=100.0)
    # one batch from both: small edge cases plus a spread of NFW sizes
    offs = np.concatenate([a.offsets, b.offsets[1:] + a.offsets[-1]])
    cat = lambda x, y: None if x is None else np.concatenate([x, y])
    inp = abi.Inputs(offs, cat(a.pos, b.pos), cat(a.vel, b.vel), cat(a.mass, b.mass), cat(a.id, b.id + 10**9), None,
                     None, cat(a.ref_pos, b.ref_pos), cat(a.ref_vel, b.ref_vel), cat(a.mostbound_pos, b.mostbound_pos),
                     cat(a.mostbound_vel, b.mostbound_vel), cat(a.most_bound_id, b.most_bound_id + 10**9))
    assert inp.n_particles < NOALLOC_MAX_PARTICLES
    return inp


def test_noalloc_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    from hbtg.build import build_library
    from hbtg.gpu import DeviceBatch, Unbinder, library

    build_library()
    lib = library()
    lib.hbtg_unbind_batch_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    lib.hbtg_unbind_batch_noalloc.restype = C.c_int
    inp = _batch()
    prm = abi.parity_params(dm_only=1, box_size=100.0)
    stream = torch.cuda.current_stream().cuda_stream

    # reference result: the allocating device entry point
    u = Unbinder(0)
    db_ref = DeviceBatch(inp)
    db_ref.reset_inout()
    u.unbind_device(prm, db_ref.c, stream)
    ref = db_ref.outputs()
    u.close()

    db = DeviceBatch(inp)
    free_after = []
    for call in range(2):
        db.reset_inout()
        torch.cuda.synchronize()
        rc = lib.hbtg_unbind_batch_noalloc(C.byref(prm), C.byref(db.c), C.c_void_p(stream))
        torch.cuda.synchronize()
        assert rc == 0, rc
        free_after.append(torch.cuda.mem_get_info()[0])
        got = db.outputs()
        check_invariants(inp, got)
        assert_parity(inp, got, ref, prm)
        for k in ("nbound", "status", "iterations", "tracer_index"):
            assert np.array_equal(getattr(got, k), getattr(ref, k)), (call, k)
        np.testing.assert_allclose(got.mbound, ref.mbound, rtol=1e-5)
    # the second call allocated nothing on the device
    assert free_after[0] == free_after[1]


def test_noalloc_rejects_batches_beyond_its_reserve():
    pytest.importorskip("torch")
    from hbtg.build import build_library
    from hbtg.gpu import library

    build_library()
    lib = library()
    lib.hbtg_unbind_batch_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    lib.hbtg_unbind_batch_noalloc.restype = C.c_int
    prm = abi.parity_params(dm_only=1)
    offsets = np.array([0, NOALLOC_MAX_PARTICLES + 1], np.int64)
    b = abi.CBatch()
    b.n_sub = 1
    b.offsets = offsets.ctypes.data
    # the size check happens on the host before any pointer is used
    assert lib.hbtg_unbind_batch_noalloc(C.byref(prm), C.byref(b), None) == 1


def _paired_halo():
    """One NFW halo whose every particle has a coincident twin (same position
    and velocity, another ID): the uncompressed octree of the bound set then
    holds a chain of cells down to the deepest key level for every pair, far
    more tree records than the reserve's 196,608 for 60,000 particles."""
    base = synthetic.nfw_single(n=30_000, seed=5, interloper_frac=0.05)
    n = base.n_particles
    two = lambda a: np.concatenate([a, a])
    return abi.Inputs(np.array([0, 2 * n], np.int64), two(base.pos), two(base.vel), two(base.mass),
                      np.concatenate([base.id, base.id + 10**9]), None, None, base.ref_pos.copy(),
                      base.ref_vel.copy(), base.mostbound_pos.copy(), base.mostbound_vel.copy(),
                      base.most_bound_id.copy())


def test_noalloc_tree_overflow_leaves_caller_arrays_untouched():
    """A tree larger than the reserve found part-way through the call (here the
    tree of RefineBindingEnergyOrder over the whole bound set, built after the
    iterations have moved the frames) returns HBTG_ERR_NOMEM with none of the
    caller's arrays written, so the same batch can be retried through the
    allocating entry point and gives that entry point's result."""
    torch = pytest.importorskip("torch")
    from hbtg import subsample
    from hbtg.build import build_library
    from hbtg.gpu import DeviceBatch, Unbinder, library

    build_library()
    lib = library()
    lib.hbtg_unbind_batch_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    lib.hbtg_unbind_batch_noalloc.restype = C.c_int
    raw = _paired_halo()
    assert raw.n_particles < NOALLOC_MAX_PARTICLES
    prm = abi.parity_params(dm_only=1, box_size=100.0, max_sample_size=1000, refine_most_bound=1,
                            refine_fraction=1.0)
    inp, _ = subsample.prepare(raw, prm)
    prm.prepared_subsample = 1
    stream = torch.cuda.current_stream().cuda_stream

    db = DeviceBatch(inp)
    db.reset_inout()
    torch.cuda.synchronize()
    rc = lib.hbtg_unbind_batch_noalloc(C.byref(prm), C.byref(db.c), C.c_void_p(stream))
    torch.cuda.synchronize()
    assert rc == 2, rc  # HBTG_ERR_NOMEM
    after = db.outputs()
    np.testing.assert_array_equal(after.ref_pos, inp.ref_pos)
    np.testing.assert_array_equal(after.ref_vel, inp.ref_vel)
    np.testing.assert_array_equal(after.mostbound_pos, inp.mostbound_pos)
    np.testing.assert_array_equal(after.mostbound_vel, inp.mostbound_vel)
    np.testing.assert_array_equal(after.most_bound_id, inp.most_bound_id)
    for k in ("order", "nbound", "mbound", "status", "iterations", "tracer_index", "core", "kinematics"):
        assert not np.any(getattr(after, k)), k

    # the retry through the allocating entry point starts from the same inputs
    u = Unbinder(0)
    u.unbind_device(prm, db.c, stream)
    retry = db.outputs()
    fresh = DeviceBatch(inp)
    fresh.reset_inout()
    u.unbind_device(prm, fresh.c, stream)
    ref = fresh.outputs()
    u.close()
    assert ref.status[0] == 0 and ref.nbound[0] > 2 * 1000
    for k in ("order", "nbound", "mbound", "ref_pos", "ref_vel", "most_bound_id", "core"):
        assert np.array_equal(getattr(retry, k), getattr(ref, k)), k
