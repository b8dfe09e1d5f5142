"""GPU parity: libhbtg.so (through its C ABI) against the CPU oracle and the
reference golden fixtures, at sizes the oracle finishes in seconds, plus
size-independent invariants at larger sizes."""
import ctypes as C
import glob
import os

import numpy as np
import pytest

from hbtg import abi, oracle, synthetic
from parity import assert_full_parity, assert_parity, check_invariants, compare

pytestmark = pytest.mark.gpu

GOLDEN = sorted(p for p in glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "*.npz"))
                if not os.path.basename(p).startswith(("nested", "reassign")))


def _load_golden(path):
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(os.path.dirname(path), "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.load(path)


def unbind_any(unbinder, inp, prm, **kw):
    """GPU call; with subsampling on, the particles are first prepared on the host
    (the reference's PrepareParticlesForSubsampling) and the order composed back."""
    if prm.max_sample_size > 0 and not prm.prepared_subsample:
        from hbtg import subsample
        prep, perm = subsample.prepare(inp, prm)
        p2 = abi.Params.from_buffer_copy(prm)
        p2.prepared_subsample = 1
        return subsample.compose(unbinder.unbind(prep, p2, **kw), inp, perm)
    return unbinder.unbind(inp, prm, **kw)


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_gpu_matches_reference_golden(unbinder, path):
    inp, prm, ref = _load_golden(path)
    got = unbind_any(unbinder, inp, prm, want_potential=True)
    check_invariants(inp, got, sorted_energies=not (prm.max_sample_size > 0 and prm.refine_most_bound))
    m = assert_full_parity(inp, got, ref, prm)
    assert m["energy_rel_median"] < 1e-5, m
    assert m["matched"] >= inp.n_sub - 1, m


def test_gpu_small_dmo_vs_oracle(unbinder):
    inp = synthetic.small_cases(seed=7)
    prm = abi.parity_params(dm_only=1, box_size=100.0)
    got = unbinder.unbind(inp, prm, want_potential=True)
    ref = oracle.run_port(inp, prm, want_potential=True)
    check_invariants(inp, got)
    assert_full_parity(inp, got, ref, prm)
    # empty subhalo conventions
    empty = np.nonzero(ref.status == abi.SUB_EMPTY)[0]
    assert np.array_equal(got.tracer_index[empty], ref.tracer_index[empty])


def test_gpu_hydro_thermal_vs_oracle(unbinder):
    inp = synthetic.hydro(seed=5, n_sub=40, nmin=100, nmax=20_000, box=300.0)
    prm = abi.parity_params(thermal=1, box_size=300.0)
    got = unbinder.unbind(inp, prm, want_potential=True)
    ref = oracle.run_port(inp, prm, want_potential=True)
    check_invariants(inp, got)
    m = assert_full_parity(inp, got, ref, prm)
    # non-tracer gas can lead the bound order: the tracer index and most-bound ID
    assert np.any(ref.tracer_index > 0)
    # per-type bound counts and masses
    assert np.abs(got.nbound_type - ref.nbound_type).sum() <= max(2, 1e-4 * ref.nbound.sum())
    rel = np.abs(got.mbound_type.sum(0) - ref.mbound_type.sum(0)) / np.maximum(ref.mbound_type.sum(0), 1e-30)
    assert np.all(rel < 1e-6), rel  # the same float sums in the same order (CountParticleTypes)


def test_gpu_mass_dynamic_range_vs_oracle(unbinder):
    """One particle 1e10 times heavier than the rest in the first subhalo: the
    fixed-point multipole sums of the other subhaloes are scaled by their own
    largest mass, so their energies keep the precision of an ordinary batch."""
    inp = synthetic.hydro(seed=5, n_sub=40, nmin=100, nmax=20_000, box=300.0)
    inp.mass[int(inp.offsets[0])] = 1e10
    prm = abi.parity_params(thermal=1, box_size=300.0)
    got = unbinder.unbind(inp, prm)
    ref = oracle.run_port(inp, prm)
    check_invariants(inp, got)
    m = assert_parity(inp, got, ref, prm)
    assert m["energy_rel_median"] < 1e-5, m


def test_gpu_nfw_single_1e5(unbinder):
    inp = synthetic.nfw_single(n=100_000, seed=0)
    prm = abi.parity_params(dm_only=1, box_size=100.0)
    got = unbinder.unbind(inp, prm, want_potential=True)
    ref = oracle.run_port(inp, prm, inner_parallel=True, want_potential=True)
    check_invariants(inp, got)
    m = assert_full_parity(inp, got, ref, prm)
    assert got.iterations[0] == ref.iterations[0] or abs(int(got.nbound[0]) - int(ref.nbound[0])) <= 10
    np.testing.assert_allclose(got.ref_pos, ref.ref_pos, rtol=0, atol=1e-4)
    np.testing.assert_allclose(got.ref_vel, ref.ref_vel, rtol=1e-4, atol=1e-3)
    np.testing.assert_allclose(got.kinematics, ref.kinematics, rtol=1e-3, atol=1e-3)


def test_gpu_batched_vs_oracle(unbinder):
    inp = synthetic.batched(n_sub=3000, seed=11, nmax=100_000)
    prm = abi.parity_params(dm_only=1, box_size=500.0)
    got = unbinder.unbind(inp, prm, want_potential=True)
    ref = oracle.run_port(inp, prm, want_potential=True)
    check_invariants(inp, got)
    assert_full_parity(inp, got, ref, prm)


def test_gpu_device_entry_matches_host_entry(unbinder):
    torch = pytest.importorskip("torch")
    from hbtg.gpu import DeviceBatch
    inp = synthetic.small_cases(seed=2)
    prm = abi.parity_params(dm_only=1, box_size=100.0)
    host = unbinder.unbind(inp, prm)
    db = DeviceBatch(inp)
    db.reset_inout()
    unbinder.unbind_device(prm, db.c, torch.cuda.current_stream().cuda_stream)
    dev = db.outputs()
    for k in ("order", "nbound", "status", "mbound", "tracer_index", "iterations", "most_bound_id"):
        assert np.array_equal(getattr(host, k), getattr(dev, k)), k


def test_gpu_deterministic(unbinder):
    inp = synthetic.batched(n_sub=500, seed=3, nmax=20_000)
    prm = abi.parity_params(dm_only=1, box_size=500.0)
    a = unbinder.unbind(inp, prm)
    b = unbinder.unbind(inp, prm)
    assert np.array_equal(a.order, b.order)
    assert np.array_equal(a.energy, b.energy)


def test_gpu_max_iterations_status(unbinder):
    inp = synthetic.small_cases(seed=0)
    prm = abi.parity_params(dm_only=1, box_size=100.0, max_iterations=1)
    got = unbinder.unbind(inp, prm, allow_max_iter=True)
    ref = oracle.run_port(inp, prm)
    assert np.array_equal(got.status, ref.status)
    assert np.all(got.iterations <= 1)


def test_gpu_invalid_arguments(unbinder):
    from hbtg.gpu import UnbindError
    inp = synthetic.small_cases(seed=0)
    prm = abi.parity_params(dm_only=1, box_size=100.0, softening=-1.0)
    with pytest.raises(UnbindError) as e:
        unbinder.unbind(inp, prm)
    assert e.value.code == 1
    prm = abi.parity_params(dm_only=1, box_size=100.0, max_sample_size=1000)
    with pytest.raises(UnbindError) as e:
        unbinder.unbind(inp, prm)
    assert e.value.code == 5


def test_gpu_invariants_large_batch(unbinder):
    inp = synthetic.batched(total=3_000_000, seed=21)
    prm = abi.parity_params(dm_only=1, box_size=500.0)
    got = unbinder.unbind(inp, prm)
    big = np.argsort(np.diff(inp.offsets))[-50:]
    check_invariants(inp.subset(big), _subset_out(got, inp, big))
    st = unbinder.stats()
    assert st["total_bound"] == int(got.nbound.sum())


def _subset_out(out, inp, subs):
    rows = np.concatenate([np.arange(inp.offsets[s], inp.offsets[s + 1]) for s in subs])
    d = {}
    for k, v in out.__dict__.items():
        if v is None:
            d[k] = None
        elif k in ("order", "energy", "potential"):
            d[k] = v[rows]
        else:
            d[k] = v[subs]
    return abi.Outputs(**d)


def test_gpu_subsampled_batched_vs_oracle(unbinder):
    """Potential subsampling (the reference default, MaxSampleSizeOfPotentialEstimate =
    1000) with RefineMostBoundParticle on a batch that mixes small and large subhaloes."""
    inp = synthetic.batched(n_sub=400, seed=13, nmax=60_000)
    prm = abi.parity_params(dm_only=1, box_size=500.0, max_sample_size=1000)
    got = unbind_any(unbinder, inp, prm, want_potential=True)
    ref = oracle.run_port(inp, prm, nthreads=1, want_potential=True)
    check_invariants(inp, got, sorted_energies=False)
    assert_full_parity(inp, got, ref, prm)


def test_gpu_subsampled_hydro_per_type_and_total(unbinder):
    inp = synthetic.hydro(seed=12, n_sub=20, nmin=1500, nmax=20_000, box=300.0)
    for per_type in (1, 0):
        prm = abi.parity_params(thermal=1, box_size=300.0, max_sample_size=1000, upscale_per_type=per_type)
        got = unbind_any(unbinder, inp, prm, want_potential=True)
        ref = oracle.run_port(inp, prm, nthreads=1, want_potential=True)
        check_invariants(inp, got, sorted_energies=False)
        assert_full_parity(inp, got, ref, prm)


def test_gpu_subsampling_requires_prepared_particles(unbinder):
    from hbtg.gpu import UnbindError
    inp = synthetic.batched(n_sub=20, seed=1, nmax=5000)
    prm = abi.parity_params(dm_only=1, box_size=500.0, max_sample_size=1000)
    with pytest.raises(UnbindError) as e:
        unbinder.unbind(inp, prm)
    assert e.value.code == 5


def _sphere(rng, n, radius):
    """n points uniform in a sphere (rejection sampling, as make_test_subhalo)."""
    out = []
    while len(out) < n:
        x = rng.uniform(-radius, radius, 3)
        if x @ x <= radius * radius:
            out.append(x)
    return np.array(out)


def test_gpu_core_phase_space_known_answer(unbinder):
    """The reference's known-answer test of GetCorePhaseSpaceProperties
    (unit_tests/test_build_pos_vel.cpp:76-164): 100-particle spheres of radius
    2 around (10, 10, 10) with one coordinate moved to each of -3, -0.1, 0.1,
    50, 99.9, 100.1, 103 in a periodic box of 100, velocities within 30 of
    (20, 20, 20).  The masses are heavy enough that every particle stays
    bound; the core (the first 20 bound particles, wrapped about the first)
    must match the test's own mass-weighted formula to 1e-5, and its
    dispersions to 1e-5 fractionally."""
    rng = np.random.default_rng(0)
    xs = [-3.0, -0.1, 0.1, 50.0, 99.9, 100.1, 103.0]
    pos, vel, counts = [], [], []
    for rep in range(5):
        for x in xs:
            for dim in range(3):
                c = np.array([10.0, 10.0, 10.0])
                c[dim] = x
                p = _sphere(rng, 100, 2.0)
                p = p[np.argsort((p * p).sum(1), kind="stable")] + c  # sorted by radius, as the fixture
                pos.append(p)
                vel.append(_sphere(rng, 100, 30.0) + 20.0)
                counts.append(100)
    pos = np.concatenate(pos).astype(np.float32)
    vel = np.concatenate(vel).astype(np.float32)
    n = len(pos)
    offsets = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    S = len(counts)
    first = offsets[:-1]
    ref_pos = pos[first].copy()
    ref_vel = np.array([vel[o:o + 100].mean(0) for o in first], np.float32)
    inp = abi.Inputs(offsets, pos, vel, np.full(n, 1000.0, np.float32), np.arange(n, dtype=np.int64) * 3 + 1, None,
                     None, ref_pos, ref_vel, pos[first].copy(), vel[first].copy(), (first * 3 + 1).astype(np.int64))
    prm = abi.parity_params(dm_only=1, box_size=100.0)
    got = unbinder.unbind(inp, prm)
    assert np.all(got.nbound == 100)
    box, half = 100.0, 50.0
    for s in range(S):
        o = offsets[s]
        idx = o + got.order[o:o + 100]
        x = pos[idx].astype(np.float64)
        v = vel[idx].astype(np.float64)
        core = idx[:20]  # DM only: every particle is a tracer; CoreSize = SubCoreSizeMin = 20
        ref = x[0]
        d = pos[core].astype(np.float64) - ref
        d = np.where(d > half, d - box, np.where(d < -half, d + box, d))
        w = ref + d  # wrap_position about the first bound particle
        m = 1000.0
        msum = m * len(core)
        cp = (m * w).sum(0) / msum
        cv = (m * vel[core].astype(np.float64)).sum(0) / msum
        sr = np.sqrt(((m * w * w).sum(0) / msum - cp * cp).sum())
        sv = np.sqrt(((m * vel[core].astype(np.float64) ** 2).sum(0) / msum - cv * cv).sum())
        gc = got.core[s].astype(np.float64)
        dpos = gc[:3] - cp
        dpos = np.where(dpos > half, dpos - box, np.where(dpos < -half, dpos + box, dpos))
        assert np.sqrt((dpos ** 2).sum()) < 1e-5, (s, gc[:3], cp)
        assert np.all(np.abs(gc[3:6] - cv) < 1e-5), (s, gc[3:6], cv)
        assert abs(gc[6] - sr) / sr < 1e-5 and abs(gc[7] - sv) / sv < 1e-5, (s, gc[6:], sr, sv)
        # the sanity checks of the reference test
        centre = pos[o:o + 100].mean(0)
        dc = gc[:3] - centre
        dc = np.where(dc > half, dc - box, np.where(dc < -half, dc + box, dc))
        assert np.sqrt((dc ** 2).sum()) < 2.0 and gc[6] <= 2.0 and gc[7] <= 30.0
