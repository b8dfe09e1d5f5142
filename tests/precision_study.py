"""Precision study: the FP32 tree walk against FP64.

One host halo (NFW, c=5) with satellites on bound orbits, straddling a box
face (synthetic.precision_host), ε = 0.005 r_200.  For a seeded random subset
of particles:

  1. potential of every particle (the first iteration's potential) at the
     subset: the GPU walk (FP32, compensated sums), the oracle's FP64 tree
     (same geometry and opening criterion) and the FP64 direct sum (no tree);
     relative errors separate FP32 rounding (GPU vs FP64 tree) from the tree
     approximation (FP64 tree vs direct);
  2. the GPU unbinding of the whole system; then, in its final frame and with
     its final bound set as the sources, each subset particle's binding
     energy from the GPU walk and from the FP64 direct sum: the mass fraction
     whose bound / unbound verdict differs is the bound-mass error of the
     walk against the exact potential.

Usage (on a GPU): python tests/precision_study.py [n_host] [n_sat] [n_subset] [out.json]
The full configuration is 1e7 / 200 / 1e5; tests/test_precision.py runs a
small one.  Test infrastructure: it uses the CPU oracle.
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "hbt-herons_gb300"))

from hbtg import abi, oracle, synthetic  # noqa: E402


def _stats(a):
    a = np.asarray(a, np.float64)
    return dict(median=float(np.median(a)), p99=float(np.percentile(a, 99)), max=float(a.max()))


def run(unbinder, n_host=10_000_000, n_sat=200, n_subset=100_000, seed=0, n_subset_energy=None):
    t0 = time.time()
    inp = synthetic.precision_host(n_host=n_host, n_sat=n_sat, seed=seed)
    r200 = inp.meta["r200"]
    prm = abi.parity_params(dm_only=1, box_size=inp.meta["box"], softening=0.005 * r200)
    n = inp.n_particles
    rng = np.random.default_rng(seed + 1)
    sub = np.sort(rng.choice(n, min(n_subset, n), replace=False))
    timing = {"generate_s": time.time() - t0}

    # 1. potential of every particle at the subset
    t = time.time()
    gpu = unbinder.tree_potential(prm, inp.pos, inp.mass, sub).astype(np.float64)
    timing["gpu_tree_s"] = time.time() - t
    t = time.time()
    tree64 = oracle.tree_potential(prm, inp.pos, inp.mass, inp.pos[sub], inp.mass[sub])
    timing["fp64_tree_s"] = time.time() - t
    t = time.time()
    direct = oracle.tree_potential(prm, inp.pos, inp.mass, inp.pos[sub], inp.mass[sub], direct=True)
    timing["fp64_direct_s"] = time.time() - t
    rel = lambda a, b: np.abs(a - b) / np.abs(b)

    # 2. bound verdicts in the GPU's final frame and bound set
    t = time.time()
    out = unbinder.unbind(inp, prm, want_energy=False)
    timing["gpu_unbind_s"] = time.time() - t
    nb = int(out.nbound[0])
    bound_idx = out.order[:nb]
    esub = sub if n_subset_energy is None else sub[:n_subset_energy]
    bpos, bmass = inp.pos[bound_idx], inp.mass[bound_idx]
    # a subset particle outside the bound set is a target that is not a source
    in_b = np.zeros(n, bool)
    in_b[bound_idx] = True
    src_index = np.full(n, -1, np.int64)
    src_index[bound_idx] = np.arange(nb)
    pot_gpu = np.zeros(len(esub))
    pot_dir = np.zeros(len(esub))
    inside = in_b[esub]
    if inside.any():
        pot_gpu[inside] = unbinder.tree_potential(prm, bpos, bmass, src_index[esub[inside]])
        pot_dir[inside] = oracle.tree_potential(prm, bpos, bmass, inp.pos[esub[inside]], inp.mass[esub[inside]],
                                                direct=True)
    if (~inside).any():  # copies of negligible mass appended as extra sources stand for outside particles
        outs = esub[~inside]
        pos2 = np.vstack([bpos, inp.pos[outs]])
        mass2 = np.concatenate([bmass, np.full(len(outs), 1e-30, np.float32)])
        pot_gpu[~inside] = unbinder.tree_potential(prm, pos2, mass2, nb + np.arange(len(outs)))
        pot_dir[~inside] = oracle.tree_potential(prm, bpos, bmass, inp.pos[outs], None, direct=True)
    dv = inp.vel[esub].astype(np.float64) - out.ref_vel[0].astype(np.float64)
    kin = 0.5 * np.sum(dv * dv, axis=1)
    flip = (kin + pot_gpu < 0) != (kin + pot_dir < 0)
    m = inp.mass[esub].astype(np.float64)
    timing["energy_s"] = time.time() - t
    return dict(
        config=dict(n_host=n_host, n_sat=n_sat, particles=n, subset=len(sub), subset_energy=len(esub),
                    softening=float(prm.softening), open_angle=float(prm.open_angle), box=inp.meta["box"],
                    seed=seed),
        phi_rel_gpu_vs_direct=_stats(rel(gpu, direct)),
        phi_rel_gpu_vs_fp64_tree=_stats(rel(gpu, tree64)),
        phi_rel_fp64_tree_vs_direct=_stats(rel(tree64, direct)),
        bound=dict(nbound=nb, mbound=float(out.mbound[0]), iterations=int(out.iterations[0]),
                   verdict_flips=int(flip.sum()), flipped_mass_fraction=float(m[flip].sum() / m.sum())),
        timing_s=timing,
    )


def main():
    from hbtg.gpu import Unbinder
    a = sys.argv[1:]
    n_host = int(float(a[0])) if a else 10_000_000
    n_sat = int(a[1]) if len(a) > 1 else 200
    n_sub = int(float(a[2])) if len(a) > 2 else 100_000
    u = Unbinder(0)
    res = run(u, n_host, n_sat, n_sub, n_subset_energy=min(n_sub, 20_000))
    text = json.dumps(res, indent=1)
    print(text)
    if len(a) > 3:
        with open(a[3], "w") as f:
            f.write(text)


if __name__ == "__main__":
    main()
