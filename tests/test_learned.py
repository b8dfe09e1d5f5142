"""Learned warm start: the proposer network's kernels against the CPU oracle
(oracle/mlp_ref.py), the warm-started iteration against the plain cold start
(the judge of its bound mass and membership), and what a network trained on
the GPU gains over the method without it."""
import os
import sys

import numpy as np
import pytest

from conftest import ROOT

sys.path.insert(0, os.path.join(ROOT, "oracle"))
import mlp_ref  # noqa: E402  (the checker)

from hbtg import abi, learned, synthetic  # noqa: E402
from parity import check_invariants, compare  # noqa: E402


# ---------------------------------------------------------------------------
# CPU
# ---------------------------------------------------------------------------
def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    w = mlp_ref.init_weights(3).astype(np.float64)
    x = rng.standard_normal((37, 6))
    y = (rng.random(37) < 0.5).astype(float)
    sw = rng.random(37) + 0.5
    _, g, _ = mlp_ref.loss_and_grad(w, x, y, sw, rounding=False)
    idx = rng.choice(mlp_ref.N_PARAMS, 60, replace=False)
    num = []
    for i in idx:
        e = np.zeros_like(w)
        e[i] = 1e-6
        num.append((mlp_ref.loss_and_grad(w + e, x, y, sw, False)[0] -
                    mlp_ref.loss_and_grad(w - e, x, y, sw, False)[0]) / 2e-6)
    assert np.max(np.abs(np.array(num) - g[idx])) <= 1e-6 * np.max(np.abs(g[idx]))


def test_bf16_rounding_is_nearest_even():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, -2.5, 0.0], np.float32)
    r = mlp_ref.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6 and r[3] == 1.0
    assert r[4] == -2.5 and r[5] == 0.0


def test_weight_layout_agrees_with_the_library():
    w = learned.initial_weights(0)
    assert w.shape == (abi.MLP_PARAMS,) == (mlp_ref.N_PARAMS,)
    d = mlp_ref.unpack(w)
    assert d["W1"].shape == (6, 64) and d["W2"].shape == (64, 64) and np.all(d["b1"] == 0)


def test_stripped_workload_lists_previous_members_first():
    inp = synthetic.stripped(n_sub=30, seed=3, nmax=5000)
    assert inp.prior_nbound.shape == (30,) and inp.prior_energy.shape == (inp.n_particles,)
    counts = np.diff(inp.offsets)
    assert np.all(inp.prior_nbound <= counts) and inp.prior_nbound.sum() > 0.5 * counts.sum()
    sub = inp.subset([3, 1])
    assert np.array_equal(sub.prior_nbound, inp.prior_nbound[[3, 1]])


def test_model_file_round_trip(tmp_path):
    m = learned.Model(learned.initial_weights(2), 0.4, 50, dict(note="x"))
    p = str(tmp_path / "m.npz")
    m.save(p)
    m2 = learned.Model.load(p)
    assert np.array_equal(m.weights, m2.weights) and m2.threshold == pytest.approx(0.4)
    assert m2.min_particles == 50 and m2.meta["note"] == "x"


def test_shipped_model_is_well_formed():
    if not os.path.exists(learned.MODEL_FILE):
        pytest.skip("no trained model shipped")
    m = learned.Model.load()
    assert m.weights.shape == (abi.MLP_PARAMS,) and np.all(np.isfinite(m.weights))
    assert 0.0 < m.threshold < 1.0 and m.min_particles >= 0


# ---------------------------------------------------------------------------
# GPU: the network's kernels
# ---------------------------------------------------------------------------
def _rows(n, seed):
    rng = np.random.default_rng(seed)
    x = np.stack([rng.random(n) * 4, rng.random(n) * 3, rng.standard_normal(n) * 2, rng.standard_normal(n),
                  rng.choice([-1.0, 0.0, 1.0], n), rng.choice([0.0, 1.0, -0.5], n)], 1).astype(np.float32)
    y = (rng.random(n) < 0.7).astype(np.float32)
    sw = (rng.random(n) + 0.5).astype(np.float32)
    return x, y, sw


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 17, 5003])
def test_mlp_forward_matches_oracle(unbinder, n):
    import torch
    x, _, _ = _rows(n, n)
    w = learned.initial_weights(5)
    w[mlp_ref.N_PARAMS - 1] = 0.3
    prob = learned.mlp_forward(torch.from_numpy(w).cuda(), torch.from_numpy(x).cuda()).cpu().numpy()
    ref, _ = mlp_ref.forward(w, x)
    # an intermediate sitting on a BF16 rounding boundary can round the other
    # way under another FP32 summation order: rare rows move by about one
    # BF16 step of one activation
    close = np.isclose(prob, ref, rtol=2e-4, atol=2e-6)
    assert close.mean() >= 0.998, close.mean()
    np.testing.assert_allclose(prob, ref, rtol=3e-3, atol=1e-4)


@pytest.mark.gpu
@pytest.mark.parametrize("n,weighted", [(5003, True), (64, False), (200_000, True)])
def test_mlp_gradient_matches_oracle(unbinder, n, weighted):
    import torch
    x, y, sw = _rows(n, 7 + n)
    w = learned.initial_weights(6)
    swt = torch.from_numpy(sw).cuda() if weighted else None
    grad, loss = learned.mlp_backward(torch.from_numpy(w).cuda(), torch.from_numpy(x).cuda(),
                                      torch.from_numpy(y).cuda(), swt)
    l_ref, g_ref, _ = mlp_ref.loss_and_grad(w, x, y, sw if weighted else None)
    g = grad.cpu().numpy().astype(np.float64)
    # FP32 accumulation in another order: the gradient as a whole within 1e-3
    assert np.linalg.norm(g - g_ref) <= 1e-3 * np.linalg.norm(g_ref)
    np.testing.assert_allclose(g, g_ref, rtol=2e-2, atol=2e-3 * np.max(np.abs(g_ref)))
    assert float(loss.item()) == pytest.approx(l_ref, rel=1e-4)


@pytest.mark.gpu
def test_adam_step_matches_formula(unbinder):
    import torch
    rng = np.random.default_rng(4)
    n = abi.MLP_PARAMS
    w0 = rng.standard_normal(n).astype(np.float32)
    g = (rng.standard_normal(n) * 10).astype(np.float32)
    m0 = (rng.standard_normal(n) * 0.1).astype(np.float32)
    v0 = (rng.random(n) * 0.1).astype(np.float32)
    t = lambda a: torch.from_numpy(a.copy()).cuda()
    w, gr, m, v = t(w0), t(g), t(m0), t(v0)
    rc = learned._lib().hbtg_adam_step(w.data_ptr(), gr.data_ptr(), m.data_ptr(), v.data_ptr(), n, 1e-2, 0.9, 0.999,
                                       1e-8, 0.5, 3, 0)
    assert rc == 0
    b1, b2, lr = (float(np.float32(q)) for q in (0.9, 0.999, 1e-2))  # the kernel's FP32 constants
    gs = g.astype(np.float64) * 0.5
    m1 = b1 * m0 + (1 - b1) * gs
    v1 = b2 * v0 + (1 - b2) * gs * gs
    w1 = w0 - lr * (m1 / (1 - b1 ** 3)) / (np.sqrt(v1 / (1 - b2 ** 3)) + 1e-8)
    np.testing.assert_allclose(m.cpu().numpy(), m1, rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(v.cpu().numpy(), v1, rtol=1e-5, atol=1e-9)
    np.testing.assert_allclose(w.cpu().numpy(), w1, rtol=1e-5, atol=1e-6)


# ---------------------------------------------------------------------------
# GPU: the warm-started iteration
# ---------------------------------------------------------------------------
def _params():
    return abi.parity_params(dm_only=1, box_size=500.0)


def _plain_and_trace(u, inp, params):
    from hbtg.gpu import DeviceBatch
    db = DeviceBatch(inp)
    db.reset_inout()
    u.unbind_device(params, db.c)
    plain = db.outputs()
    return db, plain, u.trace_labels_device(inp.n_particles, which=1)


# The warm path computes the second iteration from a new tree of the set the
# plain method reaches by correcting its first-iteration energies; the two
# differ by the tree's approximation error (opening angle 0.45), which moves
# particles with |E| that small across E = 0.  On these small, marginal test
# batches that is a few 1e-4 of the bound mass, of either sign.
PATH_NOISE = 6e-4


def _statuses_agree(inp, got, ref, params):
    from parity import near_disruption
    bad = [s for s in np.nonzero(got.status != ref.status)[0]
           if not (near_disruption(inp, got, s, params) or near_disruption(inp, ref, s, params))]
    assert not bad, bad


@pytest.mark.gpu
def test_warm_start_from_first_iteration_trace_keeps_the_plain_fixed_point(unbinder):
    """The ideal proposal (the plain run's own first-iteration survivors): the
    warm start follows the plain path from its second iteration, with less
    tree work."""
    inp = synthetic.stripped(n_sub=300, seed=11, nmax=30_000)
    params = _params()
    unbinder.count_interactions(True)
    try:
        db, plain, labels = _plain_and_trace(unbinder, inp, params)
        work_plain = unbinder.stats()["interactions"]
        db.reset_inout()
        unbinder.unbind_warm_device(params, db, labels, min_particles=0)
        warm = db.outputs()
        st = unbinder.stats()
    finally:
        unbinder.count_interactions(False)
    check_invariants(inp, plain)
    check_invariants(inp, warm)
    _statuses_agree(inp, warm, plain, params)
    m = compare(inp, warm, plain)
    assert m["mass_rel"] <= PATH_NOISE and m["membership"] <= 2 * PATH_NOISE, m
    assert st["warm_subhaloes"] > 0 and st["readmitted"] == 0
    assert st["interactions"] < work_plain, (st["interactions"], work_plain)


@pytest.mark.gpu
def test_three_state_trace_proposal_skips_the_first_test(unbinder):
    """Trusting the survivors and leaving the rest out untested: no first test
    at all, and the plain path from its second iteration."""
    import torch
    inp = synthetic.stripped(n_sub=300, seed=17, nmax=30_000)
    params = _params()
    db, plain, labels = _plain_and_trace(unbinder, inp, params)
    prop = torch.where(labels.bool(), torch.ones_like(labels), torch.full_like(labels, 2))
    db.reset_inout()
    unbinder.unbind_warm_device(params, db, prop, min_particles=100)
    warm = db.outputs()
    st = unbinder.stats()
    check_invariants(inp, warm)
    _statuses_agree(inp, warm, plain, params)
    assert st["warm_subhaloes"] > 0 and st["readmitted"] == 0
    m = compare(inp, warm, plain)
    assert m["mass_rel"] <= PATH_NOISE and m["membership"] <= 2 * PATH_NOISE, m


@pytest.mark.gpu
def test_first_test_keeps_wrongly_excluded_particles(unbinder):
    """A proposal that misses a tenth of the survivors: the first test finds
    every one of them, and the result stays at the plain fixed point."""
    import torch
    inp = synthetic.stripped(n_sub=120, seed=12, nmax=20_000)
    params = _params()
    db, plain, labels = _plain_and_trace(unbinder, inp, params)
    g = torch.Generator(device="cuda")
    g.manual_seed(0)
    drop = torch.rand(labels.shape, device="cuda", generator=g) < 0.1
    prop = (labels.bool() & ~drop).to(torch.uint8)
    db.reset_inout()
    unbinder.unbind_warm_device(params, db, prop, min_particles=0)
    warm = db.outputs()
    st = unbinder.stats()
    check_invariants(inp, warm)
    dropped = int((labels.bool() & drop).sum().item())
    assert st["readmitted"] >= 0.9 * dropped, (st["readmitted"], dropped)
    _statuses_agree(inp, warm, plain, params)
    m = compare(inp, warm, plain)
    assert m["mass_rel"] <= PATH_NOISE and m["membership"] <= 2 * PATH_NOISE, m


@pytest.mark.gpu
def test_empty_proposal_is_the_plain_method(unbinder):
    """Trusting nothing, the first test is the plain first iteration itself;
    subhaloes whose first iteration converges restart cold."""
    import torch
    inp = synthetic.batched(total=300_000, seed=16, nmax=50_000)
    params = _params()
    db, plain, _ = _plain_and_trace(unbinder, inp, params)
    db.reset_inout()
    unbinder.unbind_warm_device(params, db, torch.zeros(inp.n_particles, dtype=torch.uint8, device="cuda"))
    warm = db.outputs()
    st = unbinder.stats()
    check_invariants(inp, warm)
    _statuses_agree(inp, warm, plain, params)
    m = compare(inp, warm, plain)
    assert m["mass_rel"] <= PATH_NOISE and m["membership"] <= 2 * PATH_NOISE, m
    one = int(np.sum((plain.iterations == 1) & (np.diff(inp.offsets) > 0)))
    assert st["cold_restarts"] >= (1 if one else 0)


@pytest.mark.gpu
def test_warm_start_without_exclusions_is_the_plain_path(unbinder):
    import torch
    inp = synthetic.batched(total=200_000, seed=14, nmax=50_000)
    params = _params()
    db, plain, _ = _plain_and_trace(unbinder, inp, params)
    db.reset_inout()
    unbinder.unbind_warm_device(params, db, torch.ones(inp.n_particles, dtype=torch.uint8, device="cuda"))
    warm = db.outputs()
    assert unbinder.stats()["warm_subhaloes"] == 0
    for k in ("order", "nbound", "mbound", "status", "iterations", "energy"):
        assert np.array_equal(getattr(warm, k), getattr(plain, k)), k


@pytest.mark.gpu
def test_features_are_deterministic_and_finite(unbinder):
    from hbtg.gpu import DeviceBatch
    inp = synthetic.stripped(n_sub=200, seed=15, nmax=50_000)
    params = _params()
    db = DeviceBatch(inp)
    db.reset_inout()
    f1 = unbinder.features_device(params, db).cpu().numpy()
    f2 = unbinder.features_device(params, db).cpu().numpy()
    assert np.array_equal(f1, f2) and np.all(np.isfinite(f1))
    assert set(np.unique(f1[:, 4])) <= {-1.0, 1.0}
    f3 = unbinder.features_device(params, db, use_prior=False).cpu().numpy()
    assert np.all(f3[:, 3] == 0) and np.all(f3[:, 4] == 0)
    assert np.array_equal(f1[:, [0, 1, 2, 5]], f3[:, [0, 1, 2, 5]])
    # the previously bound particles mostly have negative monopole energies
    prev = f1[:, 4] > 0
    assert np.mean(f1[prev, 2] < 0) > 0.8


@pytest.mark.gpu
def test_trained_network_gains_over_the_plain_method(unbinder):
    """Train on the GPU from scratch on a small trace set; on held-out
    subhaloes the learned warm start does less tree work than the cold start
    and stays at its fixed point (bound mass within 2e-4 on this batch of
    1500; the benchmark reports the full-size figure)."""
    from hbtg.gpu import DeviceBatch
    params = _params()
    train_set = [(synthetic.stripped(n_sub=3000, seed=21, nmax=100_000), True)]
    model = learned.train(unbinder, train_set, params, steps=1500, batch=32768, min_particles=100)
    assert model.meta["train_error"] < 0.02
    assert 0.0 < model.threshold < 1.0
    test = synthetic.stripped(n_sub=1500, seed=22, nmax=100_000)
    db = DeviceBatch(test)
    unbinder.count_interactions(True)
    try:
        db.reset_inout()
        unbinder.unbind_device(params, db.c)
        plain = db.outputs()
        work_plain = unbinder.stats()["interactions"]
        model.install(unbinder)
        db.reset_inout()
        unbinder.unbind_learned_device(params, db)
        warm = db.outputs()
        st = unbinder.stats()
    finally:
        unbinder.count_interactions(False)
    check_invariants(test, warm)
    m = compare(test, warm, plain)
    assert m["mass_rel"] <= 2e-4 and m["membership"] <= 2 * PATH_NOISE, m
    assert st["warm_subhaloes"] > 0
    assert st["interactions"] < 0.85 * work_plain, (st["interactions"], work_plain)


@pytest.mark.gpu
def test_uncertain_particles_join_untested(unbinder):
    """first_test = 0: the particles between the two thresholds join the set
    without the first test (no tree of every particle), the first frame is the
    trusted particles' own, and the exact iteration still ends at the plain
    fixed point with every kept particle bound."""
    from hbtg.gpu import DeviceBatch
    if not os.path.exists(learned.MODEL_FILE):
        pytest.skip("no trained model shipped")
    params = _params()
    inp = synthetic.stripped(n_sub=1500, seed=23, nmax=100_000)
    db = DeviceBatch(inp)
    db.reset_inout()
    unbinder.unbind_device(params, db.c)
    plain = db.outputs()
    m = learned.Model.load()
    got = {}
    for ft in (1, 0):
        unbinder.set_model(m.weights, m.threshold, m.min_particles, m.exclude_below, ft)
        db.reset_inout()
        unbinder.unbind_learned_device(params, db)
        got[ft] = (db.outputs(), unbinder.stats())
    m.install(unbinder)
    warm, st = got[0]
    check_invariants(inp, warm)
    assert st["warm_subhaloes"] > 0 and st["readmitted"] == 0 and st["readmit_rounds"] == 0
    assert got[1][1]["readmit_rounds"] == 1
    r = compare(inp, warm, plain)
    assert r["mass_rel"] <= 2e-4 and r["membership"] <= 2 * PATH_NOISE, r
    # the tree of every particle is not built: fewer tree cells than with the test
    assert st["tree_nodes"] < got[1][1]["tree_nodes"], (st["tree_nodes"], got[1][1]["tree_nodes"])


def test_model_file_keeps_first_test(tmp_path):
    m = learned.Model(learned.initial_weights(2), 0.9, 50, {}, 1e-3, 0)
    p = str(tmp_path / "m.npz")
    m.save(p)
    m2 = learned.Model.load(p)
    assert m2.first_test == 0 and m2.exclude_below == pytest.approx(1e-3)


@pytest.mark.gpu
def test_learned_proposal_matches_network_thresholds(unbinder):
    """The learned call takes its proposal straight from the tensor-core
    inference (proposal bytes, no probability array): the particles it leaves
    out are exactly those to which hbtg_mlp_forward gives a probability below
    exclude_below, in exactly the subhaloes that start warm (large enough, and
    their kept set below BoundMassPrecision of their particles)."""
    import torch
    from hbtg.gpu import DeviceBatch
    if not os.path.exists(learned.MODEL_FILE):
        pytest.skip("no trained model shipped")
    params = _params()
    inp = synthetic.stripped(n_sub=400, seed=31, nmax=50_000)
    m = learned.Model.load()
    assert m.first_test == 0
    db = DeviceBatch(inp)
    db.reset_inout()
    feats = unbinder.features_device(params, db)  # the learned call's own features, in the input frame
    prob = learned.mlp_forward(torch.from_numpy(m.weights).cuda(), feats).cpu().numpy()
    m.install(unbinder)
    db.reset_inout()
    unbinder.unbind_learned_device(params, db)
    st = unbinder.stats()
    sizes = np.diff(inp.offsets)
    seg = np.repeat(np.arange(inp.n_sub), sizes)
    kept = np.bincount(seg, weights=~(prob < np.float32(m.exclude_below)), minlength=inp.n_sub).astype(np.int64)
    warm = (sizes >= m.min_particles) & (kept.astype(np.float32) < sizes.astype(np.float32) * np.float32(0.995))
    assert st["warm_subhaloes"] == int(warm.sum()) > 0
    assert st["excluded"] == int(np.sum((sizes - kept)[warm]))
