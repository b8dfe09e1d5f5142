"""Potential subsampling support (MaxSampleSizeOfPotentialEstimate > 0).

The reference draws each large subhalo's potential subsample by reordering
its particles with std::partition + std::random_shuffle inside Unbind
(PrepareParticlesForSubsampling, src/subhalo_unbind.cpp:430-443).  The GPU
path takes that reordering as an input: `prepare` applies it on the host
(hbtg_prepare_subsampling, same algorithm and random sequence), and `compose`
maps the returned order back to the caller's particle order.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .abi import CBatch, Inputs, Outputs, Params, _ptr


def permutation(inp: Inputs, params: Params) -> np.ndarray:
    """perm[offsets[s]+k] = input local index placed at position k."""
    from .gpu import library
    lib = library()
    lib.hbtg_prepare_subsampling.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    lib.hbtg_prepare_subsampling.restype = C.c_int
    offsets = np.ascontiguousarray(inp.offsets, np.int64)
    typ = None if inp.type is None else np.ascontiguousarray(inp.type, np.uint8)
    b = CBatch()
    b.n_sub = inp.n_sub
    b.offsets = _ptr(offsets)
    b.type = _ptr(typ)
    perm = np.zeros(max(inp.n_particles, 1), np.int64)
    rc = lib.hbtg_prepare_subsampling(C.byref(params), C.byref(b), perm.ctypes.data)
    if rc != 0:
        raise RuntimeError("hbtg_prepare_subsampling returned %d" % rc)
    return perm[:inp.n_particles]


def prepare(inp: Inputs, params: Params):
    """Returns (inputs reordered for subsampling, perm)."""
    perm = permutation(inp, params)
    seg = np.repeat(np.arange(inp.n_sub), np.diff(inp.offsets))
    rows = inp.offsets[:-1][seg] + perm
    pick = lambda a: None if a is None else np.ascontiguousarray(a[rows])
    out = Inputs(inp.offsets.copy(), pick(inp.pos), pick(inp.vel), pick(inp.mass), pick(inp.id), pick(inp.type),
                 pick(inp.u), inp.ref_pos.copy(), inp.ref_vel.copy(), inp.mostbound_pos.copy(),
                 inp.mostbound_vel.copy(), inp.most_bound_id.copy(), dict(inp.meta))
    return out, perm


def compose(out: Outputs, inp: Inputs, perm: np.ndarray) -> Outputs:
    """Maps `order` of a call on prepared inputs back to the original particle order."""
    seg = np.repeat(np.arange(inp.n_sub), np.diff(inp.offsets))
    base = inp.offsets[:-1][seg]
    out.order = perm[base + out.order]
    return out
