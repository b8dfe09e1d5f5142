"""Learned warm start of the unbinding iteration.

The proposer is a 6-64-64-1 network (include/hbt_unbind_gpu.h,
hbtg_mlp_forward) that reads six per-particle features (hbtg_features_device)
and proposes the set the iteration starts from.  It is trained here, on the
GPU, by the library's own tensor-core kernels (hbtg_mlp_backward,
hbtg_adam_step), on traces the plain method generates: the label of a
particle is 1 when it survived its subhalo's first exact iteration
(hbtg_trace_labels_device, which=1).  Particles the network trusts skip that
iteration, the most expensive one of the method (every particle against the
tree of every particle); the library gives every other particle the
iteration's own test, so nothing it would have kept is lost, and then takes
the plain method's own path from its second iteration.

Model files (.npz): weights (float32 [4673]), threshold (trusted at or
above), exclude_below (left out untested below), min_particles and a JSON
description of the training run.
"""
from __future__ import annotations

import json
import math
import os
from dataclasses import dataclass, field

import numpy as np

from . import abi, synthetic
from .abi import MLP_PARAMS, NUM_FEATURES

MODEL_FILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "warm_start_model.npz")
LAYERS = [("W1", NUM_FEATURES * 64), ("b1", 64), ("W2", 64 * 64), ("b2", 64), ("w3", 64), ("b3", 1)]


@dataclass
class Model:
    weights: np.ndarray
    threshold: float = 0.5      # trusted at or above
    min_particles: int = 100    # smaller subhaloes start cold
    meta: dict = field(default_factory=dict)
    exclude_below: float = 0.0  # left out without the first test below
    first_test: int = 1         # 1: uncertain particles get the first test; 0: they join the set untested

    def save(self, path):
        np.savez(path, weights=np.asarray(self.weights, np.float32), threshold=np.float32(self.threshold),
                 min_particles=np.int64(self.min_particles), exclude_below=np.float32(self.exclude_below),
                 first_test=np.int32(self.first_test), meta=np.array(json.dumps(self.meta)))

    @staticmethod
    def load(path=MODEL_FILE):
        z = np.load(path)
        lo = float(z["exclude_below"]) if "exclude_below" in z else 0.0
        ft = int(z["first_test"]) if "first_test" in z else 1
        return Model(z["weights"].astype(np.float32), float(z["threshold"]), int(z["min_particles"]),
                     json.loads(str(z["meta"])), lo, ft)

    def install(self, unbinder):
        unbinder.set_model(self.weights, self.threshold, self.min_particles, self.exclude_below, self.first_test)


def initial_weights(seed=0):
    """He-normal weights, zero biases, in the library's flat layout."""
    rng = np.random.default_rng(seed)
    parts = []
    for name, n in LAYERS:
        if name.startswith("b"):
            parts.append(np.zeros(n))
        else:
            fan_in = NUM_FEATURES if name == "W1" else 64
            gain = 1.0 if name == "w3" else 2.0
            parts.append(rng.standard_normal(n) * math.sqrt(gain / fan_in))
    w = np.concatenate(parts).astype(np.float32)
    assert w.shape == (MLP_PARAMS,)
    return w


def _lib():
    from .gpu import library
    return library()


def _check(rc, what):
    if rc != 0:
        from .gpu import UnbindError
        raise UnbindError(rc, what)


def mlp_forward(weights, features, stream_ptr=0):
    """sigmoid(net(features)) on the device (torch tensors in, torch tensor out)."""
    import torch
    n = features.shape[0]
    prob = torch.empty(max(n, 1), dtype=torch.float32, device=features.device)
    _check(_lib().hbtg_mlp_forward(weights.data_ptr(), features.data_ptr(), prob.data_ptr(), n, stream_ptr),
           "hbtg_mlp_forward")
    return prob[:n]


def mlp_backward(weights, features, labels, sample_weights=None, stream_ptr=0):
    """(grad [4673], loss [1]) of the summed weighted BCE, on the device."""
    import torch
    grad = torch.empty(MLP_PARAMS, dtype=torch.float32, device=features.device)
    loss = torch.empty(1, dtype=torch.float32, device=features.device)
    _check(_lib().hbtg_mlp_backward(weights.data_ptr(), features.data_ptr(), labels.data_ptr(),
                                    None if sample_weights is None else sample_weights.data_ptr(),
                                    features.shape[0], grad.data_ptr(), loss.data_ptr(), stream_ptr),
           "hbtg_mlp_backward")
    return grad, loss


class Trainer:
    """Adam on the device with the library's kernels; torch only holds memory."""

    def __init__(self, weights=None, device="cuda:0", seed=0):
        import torch
        w = initial_weights(seed) if weights is None else np.asarray(weights, np.float32)
        self.w = torch.from_numpy(w.copy()).to(device)
        self.m = torch.zeros_like(self.w)
        self.v = torch.zeros_like(self.w)
        self.step_no = 0

    def step(self, feats, labels, lr, sample_weights=None):
        grad, loss = mlp_backward(self.w, feats, labels, sample_weights)
        self.step_no += 1
        _check(_lib().hbtg_adam_step(self.w.data_ptr(), grad.data_ptr(), self.m.data_ptr(), self.v.data_ptr(),
                                     MLP_PARAMS, float(lr), 0.9, 0.999, 1e-8, 1.0 / max(feats.shape[0], 1),
                                     self.step_no, 0), "hbtg_adam_step")
        return loss

    def fit(self, feats, labels, steps=3000, batch=65536, lr=3e-3, lr_min=1e-4, seed=0, log_every=0):
        """Mini-batches of rows drawn uniformly; cosine learning-rate decay."""
        import torch
        g = torch.Generator(device=feats.device)
        g.manual_seed(seed)
        n = feats.shape[0]
        history = []
        for k in range(steps):
            idx = torch.randint(0, n, (min(batch, n),), device=feats.device, generator=g)
            rate = lr_min + 0.5 * (lr - lr_min) * (1 + math.cos(math.pi * k / max(steps - 1, 1)))
            loss = self.step(feats[idx].contiguous(), labels[idx].contiguous(), rate)
            if log_every and (k % log_every == 0 or k == steps - 1):
                history.append((k, float(loss.item()) / min(batch, n)))
        return history

    def weights(self):
        return self.w.cpu().numpy()


def traces(unbinder, inp, params, use_prior=True, device="cuda:0"):
    """Features and labels of one batch: the features the learned call would
    compute, then the plain method's first-iteration survivors (torch tensors
    on the device)."""
    from .gpu import DeviceBatch
    db = DeviceBatch(inp, device=device, want_energy=False)
    db.reset_inout()
    feats = unbinder.features_device(params, db, use_prior=use_prior).clone()
    db.reset_inout()
    unbinder.unbind_device(params, db.c)
    labels = unbinder.trace_labels_device(inp.n_particles, which=1, device=device).float()
    return feats, labels


def choose_threshold(prob, labels, fp_weight=50.0):
    """The probability cut minimising fp_weight * false positives + false
    negatives.  A survivor the network does not trust only costs one more
    target in the first test; a trusted particle that the first iteration
    would have removed moves the warm path off the plain one."""
    pos = labels > 0.5
    best, best_t, best_err = None, 0.5, 0.0
    for t in np.linspace(0.02, 0.98, 49):
        pred = prob >= float(t)
        fn = int((~pred & pos).sum().item())
        fp = int((pred & ~pos).sum().item())
        cost = fp_weight * fp + fn
        if best is None or cost < best:
            best, best_t, best_err = cost, float(t), (fn + fp) / max(len(labels), 1)
    return best_t, best_err


def choose_exclusion(prob, labels, max_missed=2e-5):
    """The largest probability below which leaving particles out untested
    loses at most max_missed of the survivors (each such survivor moves the
    warm path off the plain one by about its own mass; the benchmark's bound
    mass error against the plain path measures the effect)."""
    pos = labels > 0.5
    npos = max(int(pos.sum().item()), 1)
    best = 0.0
    for t in np.concatenate([[1e-7, 3e-7], np.logspace(-6, np.log10(0.5), 40)]):
        missed = int(((prob < float(t)) & pos).sum().item())
        if missed <= max_missed * npos:
            best = float(t)
        else:
            break
    return best


def training_batches(n_sub_stripped=100_000, n_batched=2_000_000, seed=1000, nmax=1_000_000):
    """The inputs of the training traces: tidally stripped subhaloes with a
    previous bound set, and (without a prior) subhaloes of the batched workload."""
    out = [(synthetic.stripped(n_sub=n_sub_stripped, seed=seed, nmax=nmax), True)]
    if n_batched:
        out.append((synthetic.batched(total=n_batched, seed=seed + 1, nmax=nmax), False))
    return out


def train(unbinder, batches, params, steps=3000, batch=65536, seed=0, min_particles=100, log_every=0):
    """Trains a model on the traces of `batches` [(Inputs, use_prior)]."""
    import torch
    feats, labels = [], []
    for inp, use_prior in batches:
        f, l = traces(unbinder, inp, params, use_prior=use_prior)
        counts = np.diff(inp.offsets)
        seg = np.repeat(np.arange(inp.n_sub), counts)
        survivors = np.bincount(seg, weights=l.cpu().numpy(), minlength=inp.n_sub)
        # subhaloes the first iteration disrupts have no second iteration to start
        keep_sub = (counts >= min_particles) & (survivors >= params.min_num_part)
        keep = torch.from_numpy(np.repeat(keep_sub, counts)).to(f.device)
        feats.append(f[keep])
        labels.append(l[keep])
    feats = torch.cat(feats)
    labels = torch.cat(labels)
    tr = Trainer(seed=seed)
    history = tr.fit(feats, labels, steps=steps, batch=batch, seed=seed, log_every=log_every)
    prob = mlp_forward(tr.w, feats)
    thr, err = choose_threshold(prob, labels)
    lo = min(choose_exclusion(prob, labels), thr)
    pos = labels > 0.5
    missed = {"%.0e" % t: int(((prob < t) & pos).sum().item()) for t in (1e-6, 1e-5, 1e-4, 1e-3, 1e-2, 0.1)}
    meta = dict(rows=int(feats.shape[0]), positive=float(labels.mean().item()), steps=steps, batch=batch,
                train_error=err, history=history,
                left_out=float((prob < lo).float().mean().item()),
                left_out_survivors=int(((prob < lo) & pos).sum().item()),
                tested=float(((prob >= lo) & (prob < thr)).float().mean().item()),
                survivors_below=missed, positives=int(pos.sum().item()))
    return Model(tr.weights(), thr, min_particles, meta, lo)


def main(argv=None):
    """Trains the shipped model: python -m hbtg.learned OUT.npz [n_sub_stripped] [n_batched] [steps]."""
    import sys
    import time

    from .gpu import Unbinder
    args = sys.argv[1:] if argv is None else argv
    out = args[0] if args else MODEL_FILE
    n_str = int(args[1]) if len(args) > 1 else 100_000
    n_bat = int(args[2]) if len(args) > 2 else 2_000_000
    steps = int(args[3]) if len(args) > 3 else 3000
    params = abi.parity_params(dm_only=1, box_size=500.0)
    t0 = time.time()
    batches = training_batches(n_str, n_bat)
    t1 = time.time()
    u = Unbinder(0)
    model = train(u, batches, params, steps=steps, log_every=250)
    t2 = time.time()
    model.meta.update(dict(n_sub_stripped=n_str, n_batched=n_bat, generate_s=t1 - t0, train_s=t2 - t1,
                           params=dict(softening=float(params.softening), box_size=500.0, G=1.0)))
    model.save(out)
    print(json.dumps(dict(out=out, threshold=model.threshold, exclude_below=model.exclude_below,
                          **{k: v for k, v in model.meta.items() if k != "history"})))
    for k, l in model.meta["history"]:
        print("step %5d loss %.5f" % (k, l))


if __name__ == "__main__":
    main()
