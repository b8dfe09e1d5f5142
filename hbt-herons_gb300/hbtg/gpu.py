"""Python binding of the GB300 unbinding library (libhbtg.so) through its C ABI.

This is the product path: every call goes to the CUDA library.  There is no
CPU fallback; if the library is missing or no sm_103 device is present the
calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .abi import (CallBuffers, CBatch, CModel, CPrior, CStats, Inputs, MLP_PARAMS, NUM_FEATURES, Outputs, Params,
                  STATUS_NAMES, _ptr)
from .build import LIB

_lib = None


class UnbindError(RuntimeError):
    def __init__(self, code, what):
        super().__init__("%s failed: %s (%d)" % (what, STATUS_NAMES.get(code, "?"), code))
        self.code = code


def library(path=LIB):
    """Loads libhbtg.so (built in-tree by hbtg.build.build_library)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise FileNotFoundError("libhbtg.so not built: run hbtg.build.build_library() (%s)" % path)
        lib = C.CDLL(path)
        lib.hbtg_create.argtypes = [C.POINTER(C.c_void_p), C.c_int]
        lib.hbtg_destroy.argtypes = [C.c_void_p]
        lib.hbtg_unbind_batch.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        lib.hbtg_unbind_batch_device.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.hbtg_get_stats.argtypes = [C.c_void_p, C.c_void_p]
        lib.hbtg_set_count_interactions.argtypes = [C.c_void_p, C.c_int]
        lib.hbtg_status_string.argtypes = [C.c_int]
        lib.hbtg_status_string.restype = C.c_char_p
        lib.hbtg_default_params.argtypes = [C.c_void_p]
        lib.hbtg_default_params.restype = None
        lib.hbtg_measure_fp32_peak.argtypes = [C.c_int, C.POINTER(C.c_double)]
        lib.hbtg_measure_fp32_peak.restype = C.c_int
        P = C.c_void_p
        lib.hbtg_set_model.argtypes = [P, P]
        lib.hbtg_unbind_batch_learned.argtypes = [P, P, P, P]
        lib.hbtg_unbind_batch_learned_device.argtypes = [P, P, P, P, P]
        lib.hbtg_unbind_batch_warm_device.argtypes = [P, P, P, P, C.c_int64, P]
        lib.hbtg_features_device.argtypes = [P, P, P, P, P, P]
        lib.hbtg_trace_labels_device.argtypes = [P, P, C.c_int, P]
        lib.hbtg_tree_potential_device.argtypes = [P, P, C.c_int64, P, P, C.c_int64, P, P, P]
        lib.hbtg_mlp_forward.argtypes = [P, P, P, C.c_int64, P]
        lib.hbtg_mlp_backward.argtypes = [P, P, P, P, C.c_int64, P, P, P]
        lib.hbtg_adam_step.argtypes = [P, P, P, P, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float,
                                       C.c_int, P]
        lib.hbtg_get_tuning.argtypes = [P, P]
        lib.hbtg_set_tuning.argtypes = [P, P]
        for fn in ("hbtg_create", "hbtg_destroy", "hbtg_unbind_batch", "hbtg_unbind_batch_device", "hbtg_get_stats",
                   "hbtg_set_count_interactions", "hbtg_set_model", "hbtg_unbind_batch_learned",
                   "hbtg_unbind_batch_learned_device", "hbtg_unbind_batch_warm_device", "hbtg_features_device",
                   "hbtg_trace_labels_device", "hbtg_mlp_forward", "hbtg_mlp_backward", "hbtg_adam_step",
                   "hbtg_tree_potential_device", "hbtg_get_tuning", "hbtg_set_tuning"):
            getattr(lib, fn).restype = C.c_int
        _lib = lib
    return _lib


def measure_fp32_peak(device=0):
    """FP32 FMA throughput of the device (TFLOP/s), measured by a kernel of the library."""
    v = C.c_double()
    rc = library().hbtg_measure_fp32_peak(device, C.byref(v))
    if rc != 0:
        raise UnbindError(rc, "hbtg_measure_fp32_peak")
    return v.value


class Unbinder:
    """One device handle (hbtg_create/hbtg_destroy)."""

    def __init__(self, device=0):
        self.lib = library()
        self.h = C.c_void_p()
        rc = self.lib.hbtg_create(C.byref(self.h), device)
        if rc != 0:
            raise UnbindError(rc, "hbtg_create")

    def close(self):
        if self.h:
            self.lib.hbtg_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def count_interactions(self, enable=True):
        self.lib.hbtg_set_count_interactions(self.h, int(enable))

    # -- launch settings ------------------------------------------------------
    def tuning(self):
        """The handle's launch settings (hbtg_get_tuning), as a dict."""
        from .abi import CTuning
        t = CTuning()
        rc = self.lib.hbtg_get_tuning(self.h, C.byref(t))
        if rc != 0:
            raise UnbindError(rc, "hbtg_get_tuning")
        return t.as_dict()

    def set_tuning(self, block_sort_max, walk_ranged_min, moments_blocks_per_sm):
        from .abi import CTuning
        t = CTuning(int(block_sort_max), int(walk_ranged_min), int(moments_blocks_per_sm), 0.0)
        rc = self.lib.hbtg_set_tuning(self.h, C.byref(t))
        if rc != 0:
            raise UnbindError(rc, "hbtg_set_tuning")

    def autotune(self, params: Params, cbatch: CBatch, stream_ptr=0):
        """hbtg_autotune on a device batch: the candidates with their times;
        the fastest becomes the handle's setting."""
        from .abi import CTuning
        rep = (CTuning * 64)()
        n = C.c_int(0)
        fn = self.lib.hbtg_autotune
        fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
        fn.restype = C.c_int
        rc = fn(self.h, C.byref(params), C.byref(cbatch), C.c_void_p(stream_ptr), rep, 64, C.byref(n))
        if rc != 0:
            raise UnbindError(rc, "hbtg_autotune")
        return [rep[i].as_dict() for i in range(min(n.value, 64))]

    def unbind(self, inp: Inputs, params: Params, want_energy=True, want_potential=False, allow_max_iter=False):
        """Host-pointer call (hbtg_unbind_batch)."""
        buf = CallBuffers(inp, want_energy=want_energy, want_potential=want_potential)
        rc = self.lib.hbtg_unbind_batch(self.h, C.byref(params), C.byref(buf.c))
        if rc != 0 and not (rc == 4 and allow_max_iter):
            raise UnbindError(rc, "hbtg_unbind_batch")
        return buf.out

    def unbind_raw(self, params: Params, cbatch: CBatch):
        rc = self.lib.hbtg_unbind_batch(self.h, C.byref(params), C.byref(cbatch))
        if rc != 0 and rc != 4:
            raise UnbindError(rc, "hbtg_unbind_batch")
        return rc

    def unbind_device(self, params: Params, cbatch: CBatch, stream_ptr=0):
        """Device-pointer call (hbtg_unbind_batch_device); cbatch holds device pointers
        except `offsets` (host)."""
        rc = self.lib.hbtg_unbind_batch_device(self.h, C.byref(params), C.byref(cbatch), C.c_void_p(stream_ptr))
        if rc != 0 and rc != 4:
            raise UnbindError(rc, "hbtg_unbind_batch_device")
        return rc

    def stats(self):
        s = CStats()
        self.lib.hbtg_get_stats(self.h, C.byref(s))
        return s.as_dict()

    # -- warm start ---------------------------------------------------------
    def set_model(self, weights, threshold, min_particles=0, exclude_below=0.0, first_test=1):
        """Loads the proposer network (hbtg_set_model)."""
        w = np.ascontiguousarray(weights, dtype=np.float32)
        if w.shape != (MLP_PARAMS,):
            raise ValueError("expected %d weights" % MLP_PARAMS)
        m = CModel(w.ctypes.data, float(threshold), int(min_particles), float(exclude_below), int(first_test))
        rc = self.lib.hbtg_set_model(self.h, C.byref(m))
        if rc != 0:
            raise UnbindError(rc, "hbtg_set_model")

    def unbind_learned(self, inp: Inputs, params: Params, want_energy=True, allow_max_iter=False):
        """Host-pointer learned warm start (hbtg_unbind_batch_learned); the
        prior comes from inp.prior_nbound / inp.prior_energy when present."""
        buf = CallBuffers(inp, want_energy=want_energy)
        nb = None if inp.prior_nbound is None else np.ascontiguousarray(inp.prior_nbound, dtype=np.int64)
        en = None if inp.prior_energy is None else np.ascontiguousarray(inp.prior_energy, dtype=np.float32)
        prior = CPrior(None if nb is None else nb.ctypes.data, None if en is None else en.ctypes.data)
        rc = self.lib.hbtg_unbind_batch_learned(self.h, C.byref(params), C.byref(buf.c), C.byref(prior))
        if rc != 0 and not (rc == 4 and allow_max_iter):
            raise UnbindError(rc, "hbtg_unbind_batch_learned")
        return buf.out

    def unbind_learned_device(self, params: Params, db, stream_ptr=0, use_prior=True):
        """Device-pointer learned warm start on a DeviceBatch."""
        prior = db.cprior() if use_prior else CPrior(None, None)
        rc = self.lib.hbtg_unbind_batch_learned_device(self.h, C.byref(params), C.byref(db.c), C.byref(prior),
                                                       C.c_void_p(stream_ptr))
        if rc != 0 and rc != 4:
            raise UnbindError(rc, "hbtg_unbind_batch_learned_device")
        return rc

    def unbind_warm_device(self, params: Params, db, proposal, min_particles=0, stream_ptr=0):
        """Warm start from an explicit proposal (torch uint8 tensor [N] on the
        device: 1 trusted, 0 to test, 2 left out without the test)."""
        ptr = proposal.data_ptr() if proposal is not None and proposal.numel() else None
        rc = self.lib.hbtg_unbind_batch_warm_device(self.h, C.byref(params), C.byref(db.c), ptr,
                                                    int(min_particles), C.c_void_p(stream_ptr))
        if rc != 0 and rc != 4:
            raise UnbindError(rc, "hbtg_unbind_batch_warm_device")
        return rc

    def features_device(self, params: Params, db, use_prior=True, stream_ptr=0):
        """The proposer's inputs for a DeviceBatch (in its current frame arrays):
        a torch float32 tensor [N, 6]."""
        import torch
        n = db.inp.n_particles
        f = torch.empty((max(n, 1), NUM_FEATURES), dtype=torch.float32, device=db.pos.device)
        prior = db.cprior() if use_prior else CPrior(None, None)
        rc = self.lib.hbtg_features_device(self.h, C.byref(params), C.byref(db.c), C.byref(prior), f.data_ptr(),
                                           C.c_void_p(stream_ptr))
        if rc != 0:
            raise UnbindError(rc, "hbtg_features_device")
        return f[:n]

    def subhalo_properties(self, inp: Inputs, out, params: Params, snapshot_id=1, source_relax=3.0, init=None):
        """CalculateProfileProperties / CalculateShape / TruncateSource of
        every subhalo from an unbinding call's outputs (host arrays, through
        hbtg_subhalo_properties).  Returns an abi.Props."""
        from .abi import Props
        buf = CallBuffers(inp, want_energy=False)
        for k in ("order", "nbound", "mbound", "mostbound_pos"):
            setattr(buf.out, k, np.ascontiguousarray(getattr(out, k)))
        buf.c.order, buf.c.nbound = _ptr(buf.out.order), _ptr(buf.out.nbound)
        buf.c.mbound, buf.c.mostbound_pos = _ptr(buf.out.mbound), _ptr(buf.out.mostbound_pos)
        props = Props(inp.n_sub, init)
        fn = self.lib.hbtg_subhalo_properties
        fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_double, C.c_void_p]
        fn.restype = C.c_int
        rc = fn(self.h, C.byref(params), C.byref(buf.c), int(snapshot_id), float(source_relax), C.byref(props.c))
        if rc != 0:
            raise UnbindError(rc, "hbtg_subhalo_properties")
        return props

    def reassign(self, inp: Inputs, group_off, params: Params, num_neighbours=10):
        """ReassignParticles' moves for FoF groups given as ranges of subhaloes
        (through hbtg_reassign_particles): dest[i] = the subhalo particle i
        moves to, or -1."""
        from .abi import CReassign
        dest = np.full(inp.n_particles, -1, np.int64)
        go = np.ascontiguousarray(group_off, np.int64)
        offs = np.ascontiguousarray(inp.offsets, np.int64)
        pos = np.ascontiguousarray(inp.pos, np.float32)
        typ = np.ascontiguousarray(inp.type, np.uint8)
        r = CReassign(len(go) - 1, go.ctypes.data, inp.n_sub, offs.ctypes.data, pos.ctypes.data, typ.ctypes.data,
                      dest.ctypes.data)
        fn = self.lib.hbtg_reassign_particles
        fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        fn.restype = C.c_int
        rc = fn(self.h, C.byref(params), C.byref(r), int(num_neighbours))
        if rc != 0:
            raise UnbindError(rc, "hbtg_reassign_particles")
        return dest

    def tree_potential(self, params: Params, pos, mass, targets, device="cuda:0"):
        """G/a * tree potential at the listed particles of one set
        (hbtg_tree_potential_device); numpy in, numpy float32 out."""
        import torch
        t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a, dtype=dt)).to(device)
        dpos, dmass = t(pos, np.float32), t(mass, np.float32)
        dtgt = t(targets, np.int64)
        out = torch.empty(max(len(targets), 1), dtype=torch.float32, device=device)
        rc = self.lib.hbtg_tree_potential_device(self.h, C.byref(params), len(mass), dpos.data_ptr(),
                                                 dmass.data_ptr(), len(targets), dtgt.data_ptr(), out.data_ptr(),
                                                 None)
        if rc != 0:
            raise UnbindError(rc, "hbtg_tree_potential_device")
        torch.cuda.synchronize()
        return out[:len(targets)].cpu().numpy()

    def trace_labels_device(self, n, which=1, device="cuda:0", stream_ptr=0):
        """Labels of the last call (hbtg_trace_labels_device): torch uint8 [n];
        which=1 first-iteration survivors, which=0 the last evaluated set."""
        import torch
        lab = torch.zeros(max(n, 1), dtype=torch.uint8, device=device)
        rc = self.lib.hbtg_trace_labels_device(self.h, lab.data_ptr(), int(which), C.c_void_p(stream_ptr))
        if rc != 0:
            raise UnbindError(rc, "hbtg_trace_labels_device")
        return lab[:n]


class DeviceBatch:
    """Device-resident copy of a batch (torch tensors) and the CBatch pointing at it."""

    def __init__(self, inp: Inputs, device="cuda:0", want_energy=True):
        import torch
        t = lambda a, dt=None: torch.from_numpy(np.ascontiguousarray(a)).to(device) if a is not None else None
        self.offsets = np.ascontiguousarray(inp.offsets, dtype=np.int64)
        n, ns = inp.n_particles, inp.n_sub
        self.inp = inp
        self.pos = t(inp.pos.astype(np.float32))
        self.vel = t(inp.vel.astype(np.float32))
        self.mass = t(inp.mass.astype(np.float32))
        self.u = t(inp.u.astype(np.float32)) if inp.u is not None else None
        self.id = t(inp.id.astype(np.int64))
        self.type = t(inp.type.astype(np.uint8)) if inp.type is not None else None
        self.ref_pos0 = t(inp.ref_pos.astype(np.float32))
        self.ref_vel0 = t(inp.ref_vel.astype(np.float32))
        self.mbp0 = t(inp.mostbound_pos.astype(np.float32))
        self.mbv0 = t(inp.mostbound_vel.astype(np.float32))
        self.mbid0 = t(inp.most_bound_id.astype(np.int64))
        z = lambda shape, dt: torch.zeros(shape, dtype=dt, device=device)
        self.ref_pos, self.ref_vel = z((ns, 3), torch.float32), z((ns, 3), torch.float32)
        self.mbp, self.mbv = z((ns, 3), torch.float32), z((ns, 3), torch.float32)
        self.mbid = z(ns, torch.int64)
        self.order = z(max(n, 1), torch.int64)
        self.nbound = z(ns, torch.int64)
        self.mbound = z(ns, torch.float32)
        self.nbound_type = z((ns, 6), torch.int64)
        self.mbound_type = z((ns, 6), torch.float32)
        self.tracer_index = z(ns, torch.int64)
        self.kin = z((ns, 5), torch.float32)
        self.core = z((ns, 8), torch.float32)
        self.energy = z(max(n, 1), torch.float32) if want_energy else None
        self.iterations = z(ns, torch.int32)
        self.status = z(ns, torch.int32)
        self.prior_nbound = t(inp.prior_nbound.astype(np.int64)) if inp.prior_nbound is not None else None
        self.prior_energy = t(inp.prior_energy.astype(np.float32)) if inp.prior_energy is not None else None
        p = lambda x: None if x is None else x.data_ptr()
        self.c = CBatch(ns, self.offsets.ctypes.data, p(self.pos), p(self.vel), p(self.mass), p(self.u), p(self.id),
                        p(self.type), p(self.ref_pos), p(self.ref_vel), p(self.mbp), p(self.mbv), p(self.mbid),
                        p(self.order), p(self.nbound), p(self.mbound), p(self.nbound_type), p(self.mbound_type),
                        p(self.tracer_index), p(self.kin), p(self.core), p(self.energy), None, p(self.iterations),
                        p(self.status))

    def cprior(self):
        p = lambda x: None if x is None else x.data_ptr()
        return CPrior(p(self.prior_nbound), p(self.prior_energy))

    def reset_inout(self):
        """Restores the in/out frame arrays to the inputs (before each call)."""
        self.ref_pos.copy_(self.ref_pos0)
        self.ref_vel.copy_(self.ref_vel0)
        self.mbp.copy_(self.mbp0)
        self.mbv.copy_(self.mbv0)
        self.mbid.copy_(self.mbid0)

    def outputs(self) -> Outputs:
        c = lambda x: None if x is None else x.cpu().numpy()
        n = self.inp.n_particles
        return Outputs(order=c(self.order)[:n], nbound=c(self.nbound), mbound=c(self.mbound),
                       nbound_type=c(self.nbound_type), mbound_type=c(self.mbound_type),
                       tracer_index=c(self.tracer_index), kinematics=c(self.kin), core=c(self.core),
                       energy=None if self.energy is None else c(self.energy)[:n], potential=None,
                       iterations=c(self.iterations), status=c(self.status), ref_pos=c(self.ref_pos),
                       ref_vel=c(self.ref_vel), mostbound_pos=c(self.mbp), mostbound_vel=c(self.mbv),
                       most_bound_id=c(self.mbid))
