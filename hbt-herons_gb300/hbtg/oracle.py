"""Loaders for the ORACLE libraries (test and measurement infrastructure).

Only tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline /
reference legs use this module: it runs the CPU restatement in
``oracle/unbind_port.cpp`` (liboracle.so) or the reference's own Unbind
compiled into ``oracle/_ref/``.  The product path (``hbtg.gpu``) never
imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

from .abi import CallBuffers, Inputs, Params

REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
ORACLE_DIR = os.path.join(REPO, "oracle")

_libs = {}


def _build_module():
    if ORACLE_DIR not in sys.path:
        sys.path.insert(0, ORACLE_DIR)
    import build_oracle  # noqa: E402
    return build_oracle


def port_lib():
    if "port" not in _libs:
        path = _build_module().build_port()
        lib = C.CDLL(path)
        lib.oracle_unbind_batch.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int]
        lib.oracle_unbind_batch.restype = C.c_int
        lib.oracle_last_interactions.restype = C.c_int64
        lib.oracle_last_cells.restype = C.c_int64
        lib.oracle_subhalo_properties.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_void_p]
        lib.oracle_subhalo_properties.restype = C.c_int
        lib.oracle_reassign.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        lib.oracle_reassign.restype = C.c_int
        for fn in (lib.oracle_tree_potential, lib.oracle_direct_potential):
            fn.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                           C.c_void_p]
            fn.restype = C.c_int
        _libs["port"] = lib
    return _libs["port"]


def reference_lib(variant):
    """The reference's own Unbind ('dmo' or 'hydro'); None when it was not built."""
    key = "ref_" + variant
    if key not in _libs:
        path = os.path.join(ORACLE_DIR, "_ref", "libref_%s.so" % variant)
        if not os.path.exists(path):
            mod = _build_module()
            if mod.reference_available():
                mod.build_reference()
        if not os.path.exists(path):
            return None
        lib = C.CDLL(path)
        lib.ref_unbind_batch.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int]
        lib.ref_unbind_batch.restype = C.c_int
        lib.ref_subhalo_properties.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_void_p]
        lib.ref_subhalo_properties.restype = C.c_int
        lib.ref_recursive_unbind.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int64] + \
            [C.c_void_p] * 6
        lib.ref_recursive_unbind.restype = C.c_int
        lib.ref_reassign.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        lib.ref_reassign.restype = C.c_int
        _libs[key] = lib
    return _libs[key]


def run_port(inp: Inputs, params: Params, nthreads=0, inner_parallel=False, want_potential=False):
    buf = CallBuffers(inp, want_energy=True, want_potential=want_potential)
    rc = port_lib().oracle_unbind_batch(C.byref(params), C.byref(buf.c), nthreads, int(inner_parallel))
    if rc != 0:
        raise RuntimeError("oracle_unbind_batch returned %d" % rc)
    return buf.out


def run_reference(inp: Inputs, params: Params, nthreads=0, inner_parallel=False, want_potential=False):
    variant = "dmo" if params.dm_only else "hydro"
    if not params.dm_only and not params.thermal:
        raise ValueError("the reference oracle is built with UNBIND_WITH_THERMAL_ENERGY for hydro inputs")
    lib = reference_lib(variant)
    if lib is None:
        raise FileNotFoundError("reference oracle not built (reference sources absent)")
    buf = CallBuffers(inp, want_energy=True, want_potential=want_potential)
    rc = lib.ref_unbind_batch(C.byref(params), C.byref(buf.c), nthreads, int(inner_parallel))
    if rc != 0:
        raise RuntimeError("ref_unbind_batch returned %d" % rc)
    return buf.out


def tree_potential(params, src_pos, src_mass, tgt_pos, tgt_mass=None, direct=False):
    lib = port_lib()
    src_pos = np.ascontiguousarray(src_pos, np.float32)
    src_mass = np.ascontiguousarray(src_mass, np.float32)
    tgt_pos = np.ascontiguousarray(tgt_pos, np.float32)
    tm = None if tgt_mass is None else np.ascontiguousarray(tgt_mass, np.float32)
    out = np.zeros(len(tgt_pos), np.float64)
    fn = lib.oracle_direct_potential if direct else lib.oracle_tree_potential
    rc = fn(C.byref(params), len(src_pos), src_pos.ctypes.data, src_mass.ctypes.data, len(tgt_pos),
            tgt_pos.ctypes.data, None if tm is None else tm.ctypes.data, out.ctypes.data)
    if rc != 0:
        raise RuntimeError("oracle potential returned %d" % rc)
    return out


def _props_batch(inp: Inputs, out):
    """A CBatch over the inputs and an unbinding call's outputs."""
    from .abi import _ptr
    buf = CallBuffers(inp, want_energy=False)
    for k in ("order", "nbound", "mbound", "mostbound_pos"):
        setattr(buf.out, k, np.ascontiguousarray(getattr(out, k)))
    buf.c.order, buf.c.nbound = _ptr(buf.out.order), _ptr(buf.out.nbound)
    buf.c.mbound, buf.c.mostbound_pos = _ptr(buf.out.mbound), _ptr(buf.out.mostbound_pos)
    return buf


def subhalo_properties(inp: Inputs, out, params: Params, snapshot_id=1, source_relax=3.0, init=None,
                       reference=False):
    """CalculateProfileProperties / CalculateShape / TruncateSource of every
    subhalo from an unbinding call's outputs: the restatement, or with
    `reference` the reference's own functions (oracle/_ref)."""
    from .abi import Props
    buf = _props_batch(inp, out)
    props = Props(inp.n_sub, init)
    if reference:
        lib = reference_lib("dmo" if params.dm_only else "hydro")
        if lib is None:
            raise FileNotFoundError("reference oracle not built (reference sources absent)")
        fn = lib.ref_subhalo_properties
    else:
        fn = port_lib().oracle_subhalo_properties
    rc = fn(C.byref(params), C.byref(buf.c), int(snapshot_id), float(source_relax), C.byref(props.c))
    if rc != 0:
        raise RuntimeError("subhalo properties returned %d" % rc)
    return props


def reference_recursive_unbind(parts, members, parent, frames, params: Params, merge_trapped=True, snapshot_id=1):
    """The reference's own Subhalo_t::RecursiveUnbind (with MergeRecursively)
    from every root of a nesting forest (oracle/_ref).  Returns a dict of
    per-subhalo arrays: nbound, mbound, most_bound_id, sink_track, snap_sink,
    snap_death, and ids (list of the final Particles' IDs)."""
    from .abi import _ptr
    lib = reference_lib("dmo" if params.dm_only else "hydro")
    if lib is None:
        raise FileNotFoundError("reference oracle not built (reference sources absent)")
    S = len(members)
    idx = np.concatenate(members) if S else np.zeros(0, np.int64)
    offsets = np.zeros(S + 1, np.int64)
    np.cumsum([len(m) for m in members], out=offsets[1:])
    pick = lambda a: None if a is None else np.ascontiguousarray(a[idx])
    f = lambda k: np.ascontiguousarray(np.asarray(frames[k]))
    inp = Inputs(offsets, pick(parts.pos), pick(parts.vel), pick(parts.mass), pick(parts.id), pick(parts.type),
                 pick(parts.u), f("ref_pos"), f("ref_vel"), f("mostbound_pos"), f("mostbound_vel"), f("most_bound_id"))
    buf = CallBuffers(inp, want_energy=False)
    cap = int(offsets[-1]) * 8 + 16
    out_off, out_count = np.zeros(S, np.int64), np.zeros(S, np.int64)
    out_ids = np.zeros(cap, np.int64)
    sink = np.zeros(S, np.int64)
    ssink, sdeath = np.zeros(S, np.int32), np.zeros(S, np.int32)
    par = np.ascontiguousarray(parent, np.int64)
    rc = lib.ref_recursive_unbind(C.byref(params), C.byref(buf.c), _ptr(par), int(merge_trapped), int(snapshot_id),
                                  cap, _ptr(out_off), _ptr(out_count), _ptr(out_ids), _ptr(sink), _ptr(ssink),
                                  _ptr(sdeath))
    if rc != 0:
        raise RuntimeError("ref_recursive_unbind returned %d" % rc)
    return dict(nbound=buf.out.nbound.copy(), mbound=buf.out.mbound.copy(), most_bound_id=buf.out.most_bound_id.copy(),
                sink_track=sink, snap_sink=ssink, snap_death=sdeath,
                ids=[out_ids[out_off[s]:out_off[s] + out_count[s]].copy() for s in range(S)])


def reassign(inp: Inputs, group_off, params: Params, num_neighbours=10, reference=False):
    """The moves of ReassignParticles for FoF groups given as ranges of
    subhaloes (group_off): dest[i] = the subhalo particle i moves to, or -1.
    The restatement, or with `reference` the reference's own neighbour search
    (oracle/_ref, hydro build)."""
    from .abi import CReassign
    dest = np.full(inp.n_particles, -1, np.int64)
    go = np.ascontiguousarray(group_off, np.int64)
    offs = np.ascontiguousarray(inp.offsets, np.int64)
    pos = np.ascontiguousarray(inp.pos, np.float32)
    typ = np.ascontiguousarray(inp.type, np.uint8)
    r = CReassign(len(go) - 1, go.ctypes.data, inp.n_sub, offs.ctypes.data, pos.ctypes.data, typ.ctypes.data,
                  dest.ctypes.data)
    if reference:
        lib = reference_lib("hydro")
        if lib is None:
            raise FileNotFoundError("reference oracle not built (reference sources absent)")
        fn = lib.ref_reassign
    else:
        fn = port_lib().oracle_reassign
    rc = fn(C.byref(params), C.byref(r), int(num_neighbours))
    if rc != 0:
        raise RuntimeError("reassign returned %d" % rc)
    return dest
