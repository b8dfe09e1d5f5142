"""Nested unbinding by depth: SubhaloSnapshot_t::RefineParticles'
RecursiveUnbind (src/subhalo_unbind.cpp:810-841) as one batch per depth.

The reference unbinds a FoF host's subhalo tree depth-first: each child is
unbound first, then its unbound particles (Particles[Nbound:], in the order
Unbind left them) are appended to its parent's source, then the parent is
unbound.  Subhaloes at the same depth never feed one another, so all of them
are one batch: the deepest level first, then, after appending every child's
unbound tail to its parent (children in ascending subhalo index, the order of
NestedSubhalos here), the next level up.  MergeTrappedSubhalos (the merger
pass and second Unbind of a host) is not part of this path.

`unbind_fn(inputs, params) -> Outputs` is any batch unbinder with the
hbtg_unbind_batch contract (the GPU library, or the CPU oracle in tests).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .abi import Inputs, Outputs


@dataclass
class Particles:
    """Global particle table; subhalo sources are index lists into it."""
    pos: np.ndarray               # float32 [P, 3]
    vel: np.ndarray               # float32 [P, 3]
    mass: np.ndarray              # float32 [P]
    id: np.ndarray                # int64 [P]
    type: np.ndarray | None = None
    u: np.ndarray | None = None


@dataclass
class SubhaloResult:
    members: np.ndarray  # global particle indices, in the order Unbind left them (bound first)
    nbound: int
    mbound: float
    status: int
    iterations: int
    ref_pos: np.ndarray
    ref_vel: np.ndarray
    most_bound_id: int
    energy: np.ndarray | None  # binding energies of the bound particles


def depths(parent):
    """Depth of every subhalo in the nesting forest (roots 0); raises on a cycle."""
    parent = np.asarray(parent, np.int64)
    n = len(parent)
    depth = np.full(n, -1, np.int64)
    for s in range(n):
        chain = []
        t = s
        while t >= 0 and depth[t] < 0:
            chain.append(t)
            if len(chain) > n:
                raise ValueError("nesting has a cycle")
            t = int(parent[t])
        d = 0 if t < 0 else depth[t] + 1
        for u in reversed(chain):
            depth[u] = d
            d += 1
    return depth


def _batch(parts: Particles, members, subs, frames):
    counts = np.array([len(members[s]) for s in subs], np.int64)
    offsets = np.zeros(len(subs) + 1, np.int64)
    np.cumsum(counts, out=offsets[1:])
    idx = np.concatenate([members[s] for s in subs]) if len(subs) else np.zeros(0, np.int64)
    pick = lambda a: None if a is None else np.ascontiguousarray(a[idx])
    f = lambda k: np.ascontiguousarray(np.asarray(frames[k])[subs])
    return idx, offsets, Inputs(offsets, pick(parts.pos), pick(parts.vel), pick(parts.mass), pick(parts.id),
                                pick(parts.type), pick(parts.u), f("ref_pos"), f("ref_vel"), f("mostbound_pos"),
                                f("mostbound_vel"), f("most_bound_id"))


def unbind_nested(unbind_fn, parts: Particles, members, parent, frames, params):
    """Unbinds every subhalo of a nesting forest; returns [SubhaloResult] by subhalo.

    members[s]: int64 indices of subhalo s's source particles (its own, in order);
    parent[s]: the subhalo it is nested in, or -1; frames: per-subhalo arrays
    ref_pos, ref_vel, mostbound_pos, mostbound_vel, most_bound_id (as in Inputs)."""
    parent = np.asarray(parent, np.int64)
    depth = depths(parent)
    members = [np.asarray(m, np.int64) for m in members]
    results = [None] * len(members)
    for d in range(int(depth.max(initial=-1)), -1, -1):
        subs = np.nonzero(depth == d)[0]
        if not len(subs):
            continue
        idx, offsets, inp = _batch(parts, members, subs, frames)
        out: Outputs = unbind_fn(inp, params)
        for k, s in enumerate(subs):
            off, end = offsets[k], offsets[k + 1]
            order = idx[off + out.order[off:end]]
            nb = int(out.nbound[k])
            results[s] = SubhaloResult(order, nb, float(out.mbound[k]), int(out.status[k]), int(out.iterations[k]),
                                       out.ref_pos[k].copy(), out.ref_vel[k].copy(), int(out.most_bound_id[k]),
                                       None if out.energy is None else out.energy[off:off + nb].copy())
        # children, in ascending subhalo index, hand their unbound tails to their parents
        for s in subs:
            p = int(parent[s])
            if p >= 0:
                r = results[s]
                members[p] = np.concatenate([members[p], r.members[r.nbound:]])
    return results


def unbind_recursive_reference(unbind_fn, parts: Particles, members, parent, frames, params):
    """The reference's recursion, one subhalo per call (test helper: the depth
    batching must give the same results)."""
    parent = np.asarray(parent, np.int64)
    children = [[] for _ in members]
    for s, p in enumerate(parent):
        if p >= 0:
            children[p].append(s)
    members = [np.asarray(m, np.int64) for m in members]
    results = [None] * len(members)

    def recurse(s):
        for c in children[s]:
            recurse(c)
            r = results[c]
            members[s] = np.concatenate([members[s], r.members[r.nbound:]])
        idx, offsets, inp = _batch(parts, members, [s], frames)
        out = unbind_fn(inp, params)
        nb = int(out.nbound[0])
        results[s] = SubhaloResult(idx[out.order], nb, float(out.mbound[0]), int(out.status[0]),
                                   int(out.iterations[0]), out.ref_pos[0].copy(), out.ref_vel[0].copy(),
                                   int(out.most_bound_id[0]), None if out.energy is None else out.energy[:nb].copy())

    for s in range(len(members)):
        if parent[s] < 0:
            recurse(s)
    return results
