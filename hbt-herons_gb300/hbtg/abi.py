"""ctypes mirror of include/hbt_unbind_gpu.h and helpers to call it.

Three libraries export the same batch contract:
  * libhbtg.so           the GB300 product (hbtg_unbind_batch, hbtg_unbind_batch_device)
  * oracle liboracle.so  the CPU restatement (oracle_unbind_batch) - tests/bench only
  * oracle libref_*.so   the reference Subhalo_t::Unbind (ref_unbind_batch) - tests only
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

TYPE_MAX = 6
KIN_STRIDE = 5
CORE_STRIDE = 8

SUB_CONVERGED, SUB_DISRUPTED, SUB_EMPTY, SUB_MAX_ITER = 0, 1, 2, 3

STATUS_NAMES = {0: "HBTG_OK", 1: "HBTG_ERR_INVALID", 2: "HBTG_ERR_NOMEM", 3: "HBTG_ERR_CUDA",
                4: "HBTG_ERR_MAX_ITER", 5: "HBTG_ERR_UNSUPPORTED", 6: "HBTG_ERR_NO_DEVICE"}


class Params(C.Structure):
    """hbtg_params: the HBTConfig values Subhalo_t::Unbind reads (src/config_parser.h:22-201)."""
    _fields_ = [
        ("box_size", C.c_double),
        ("periodic", C.c_int32),
        ("softening", C.c_double),
        ("tree_node_resolution", C.c_double),
        ("open_angle", C.c_double),
        ("bound_mass_precision", C.c_double),
        ("min_num_part", C.c_int64),
        ("min_num_tracer", C.c_int64),
        ("tracer_type_mask", C.c_int32),
        ("no_subsample_mask", C.c_int32),
        ("max_sample_size", C.c_int64),
        ("refine_most_bound", C.c_int32),
        ("refine_fraction", C.c_double),
        ("upscale_per_type", C.c_int32),
        ("sub_core_size_min", C.c_int64),
        ("sub_core_size_factor", C.c_double),
        ("dm_only", C.c_int32),
        ("thermal", C.c_int32),
        ("G", C.c_double),
        ("scale_factor", C.c_double),
        ("hubble", C.c_double),
        ("max_iterations", C.c_int32),
        ("mode", C.c_int32),
        ("seed", C.c_int64),
        ("prepared_subsample", C.c_int32),
    ]

    def as_dict(self):
        return {k: (list(v) if hasattr(v, "__len__") else v) for k, v in ((k, getattr(self, k)) for k, _ in self._fields_)}


def default_params(**overrides) -> Params:
    """Reference defaults (src/config_parser.h:98-172), G from default units
    (src/config_parser.cpp:200), a=1, Hz=0.  Softening must be set by the caller."""
    p = Params()
    p.box_size = 100.0
    p.periodic = 1
    p.softening = 0.005
    p.tree_node_resolution = 0.1 * 0.005
    p.open_angle = 0.45
    p.bound_mass_precision = 0.995
    p.min_num_part = 20
    p.min_num_tracer = 10
    p.tracer_type_mask = (1 << 1) | (1 << 4)
    p.no_subsample_mask = 1 << 5
    p.max_sample_size = 1000
    p.refine_most_bound = 1
    p.refine_fraction = 0.1
    p.upscale_per_type = 1
    p.sub_core_size_min = 20
    p.sub_core_size_factor = 0.0
    p.dm_only = 0
    p.thermal = 0
    p.G = 43.0071
    p.scale_factor = 1.0
    p.hubble = 0.0
    p.max_iterations = 1000
    p.mode = 0
    p.seed = 0
    p.prepared_subsample = 0
    for k, v in overrides.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    if "softening" in overrides and "tree_node_resolution" not in overrides:
        p.tree_node_resolution = 0.1 * p.softening
    return p


def parity_params(**overrides) -> Params:
    """The deterministic configuration used for parity: no potential
    subsampling (testing/config_test.txt:32-34 in the reference), G=1."""
    base = dict(max_sample_size=0, G=1.0)
    base.update(overrides)
    return default_params(**base)


_P = C.c_void_p


class CBatch(C.Structure):
    _fields_ = [
        ("n_sub", C.c_int64),
        ("offsets", _P), ("pos", _P), ("vel", _P), ("mass", _P), ("u", _P), ("id", _P), ("type", _P),
        ("ref_pos", _P), ("ref_vel", _P), ("mostbound_pos", _P), ("mostbound_vel", _P), ("most_bound_id", _P),
        ("order", _P), ("nbound", _P), ("mbound", _P), ("nbound_type", _P), ("mbound_type", _P),
        ("tracer_index", _P), ("kinematics", _P), ("core", _P), ("energy", _P), ("potential", _P),
        ("iterations", _P), ("status", _P),
    ]


class CStats(C.Structure):
    _fields_ = [
        ("n_sub", C.c_int64), ("n_particles", C.c_int64), ("total_bound", C.c_int64),
        ("global_iterations", C.c_int64), ("interactions", C.c_int64), ("tree_nodes", C.c_int64),
        ("ms_total", C.c_double), ("ms_walk", C.c_double), ("ms_plan", C.c_double), ("ms_tree", C.c_double),
        ("ms_part", C.c_double), ("ms_frame", C.c_double), ("ms_final", C.c_double), ("walk_launches", C.c_int64),
        ("kernel_launches", C.c_int64), ("h2d_bytes", C.c_int64), ("d2h_bytes", C.c_int64),
        ("ms_propose", C.c_double), ("warm_subhaloes", C.c_int64), ("excluded", C.c_int64),
        ("readmitted", C.c_int64), ("cold_restarts", C.c_int64), ("readmit_rounds", C.c_int64),
        ("walk_blocks_per_sm", C.c_int64), ("ms_h2d", C.c_double), ("ms_d2h", C.c_double),
        ("walk_steps", C.c_int64), ("walk_nodes", C.c_int64), ("walk_pending_batches", C.c_int64),
        ("walk_entries_full", C.c_int64), ("walk_entries_part", C.c_int64), ("walk_entries_near", C.c_int64),
        ("walk_drained", C.c_int64), ("walk_cycles", C.c_int64 * 8), ("host_syncs", C.c_int64),
    ]

    def as_dict(self):
        return {k: (list(v) if hasattr(v, "__len__") else v) for k, v in ((k, getattr(self, k)) for k, _ in self._fields_)}


class CProps(C.Structure):
    """hbtg_props."""
    _fields_ = [(k, C.c_void_p) for k in ("rmax", "vmax", "rhalf", "renclose", "r200", "m200", "last_vmax",
                                          "rmax_last", "snap_last", "inertia", "inertia_w", "nsource")]


PROPS_FLOAT = ("rmax", "vmax", "rhalf", "renclose", "r200", "m200", "last_vmax", "rmax_last")


class Props:
    """Host arrays of hbtg_props for `n_sub` subhaloes; in/out fields start
    from `init` (a dict of arrays) or zero."""

    def __init__(self, n_sub, init=None, want_nsource=True):
        init = init or {}
        for k in PROPS_FLOAT:
            setattr(self, k, np.array(init.get(k, np.zeros(n_sub)), np.float32))
        self.snap_last = np.array(init.get("snap_last", np.full(n_sub, -1)), np.int32)
        self.inertia = np.zeros((n_sub, 6), np.float32)
        self.inertia_w = np.zeros((n_sub, 6), np.float32)
        self.nsource = np.zeros(n_sub, np.int64) if want_nsource else None
        self.c = CProps(*[_ptr(getattr(self, k)) for k, _ in CProps._fields_])

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in CProps._fields_ if getattr(self, k) is not None}


class CReassign(C.Structure):
    """hbtg_reassign."""
    _fields_ = [("n_groups", C.c_int64), ("group_off", C.c_void_p), ("n_sub", C.c_int64), ("offsets", C.c_void_p),
                ("pos", C.c_void_p), ("type", C.c_void_p), ("dest", C.c_void_p)]


class CPrior(C.Structure):
    """hbtg_prior."""
    _fields_ = [("nbound_prev", _P), ("energy_prev", _P)]


class CTuning(C.Structure):
    """hbtg_tuning: launch settings that leave every result unchanged."""
    _fields_ = [("block_sort_max", C.c_int32), ("walk_ranged_min", C.c_int32), ("moments_blocks_per_sm", C.c_int32),
                ("ms", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class CModel(C.Structure):
    """hbtg_model."""
    _fields_ = [("weights", _P), ("threshold", C.c_float), ("min_particles", C.c_int64),
                ("exclude_below", C.c_float), ("first_test", C.c_int32)]


MLP_PARAMS = 4673
NUM_FEATURES = 6


def _ptr(a):
    return None if a is None else a.ctypes.data


@dataclass
class Inputs:
    """One batch of subhaloes in CSR layout (host numpy arrays)."""
    offsets: np.ndarray          # int64 [n_sub+1]
    pos: np.ndarray              # float32 [N,3]
    vel: np.ndarray              # float32 [N,3]
    mass: np.ndarray             # float32 [N]
    id: np.ndarray               # int64 [N]
    type: np.ndarray | None      # uint8 [N] or None
    u: np.ndarray | None         # float32 [N] or None
    ref_pos: np.ndarray          # float32 [n_sub,3]
    ref_vel: np.ndarray          # float32 [n_sub,3]
    mostbound_pos: np.ndarray    # float32 [n_sub,3]
    mostbound_vel: np.ndarray    # float32 [n_sub,3]
    most_bound_id: np.ndarray    # int64 [n_sub]
    meta: dict = field(default_factory=dict)
    # previous-output knowledge for the warm start (hbtg_prior): particles
    # [0, prior_nbound[s]) of each subhalo were bound, with energies prior_energy
    prior_nbound: np.ndarray | None = None   # int64 [n_sub]
    prior_energy: np.ndarray | None = None   # float32 [N]

    @property
    def n_sub(self):
        return len(self.offsets) - 1

    @property
    def n_particles(self):
        return int(self.offsets[-1])

    def subset(self, subs):
        """A new batch holding only the listed subhaloes (in that order)."""
        subs = np.asarray(subs, dtype=np.int64)
        counts = self.offsets[subs + 1] - self.offsets[subs]
        offs = np.zeros(len(subs) + 1, np.int64)
        np.cumsum(counts, out=offs[1:])
        rows = np.concatenate([np.arange(self.offsets[s], self.offsets[s + 1]) for s in subs]) if len(subs) else \
            np.zeros(0, np.int64)
        pick = lambda a: None if a is None else np.ascontiguousarray(a[rows])
        return Inputs(offs, pick(self.pos), pick(self.vel), pick(self.mass), pick(self.id), pick(self.type),
                      pick(self.u), self.ref_pos[subs].copy(), self.ref_vel[subs].copy(),
                      self.mostbound_pos[subs].copy(), self.mostbound_vel[subs].copy(),
                      self.most_bound_id[subs].copy(), dict(self.meta),
                      None if self.prior_nbound is None else self.prior_nbound[subs].copy(), pick(self.prior_energy))

    def save(self, path):
        d = {k: getattr(self, k) for k in ("offsets", "pos", "vel", "mass", "id", "ref_pos", "ref_vel",
                                           "mostbound_pos", "mostbound_vel", "most_bound_id")}
        if self.type is not None:
            d["type"] = self.type
        if self.u is not None:
            d["u"] = self.u
        if self.prior_nbound is not None:
            d["prior_nbound"] = self.prior_nbound
        if self.prior_energy is not None:
            d["prior_energy"] = self.prior_energy
        np.savez_compressed(path, **d)

    @staticmethod
    def load(path_or_npz, prefix=""):
        z = np.load(path_or_npz) if isinstance(path_or_npz, str) else path_or_npz
        g = lambda k: z[prefix + k] if (prefix + k) in z else None
        return Inputs(g("offsets"), g("pos"), g("vel"), g("mass"), g("id"), g("type"), g("u"), g("ref_pos"),
                      g("ref_vel"), g("mostbound_pos"), g("mostbound_vel"), g("most_bound_id"), {},
                      g("prior_nbound"), g("prior_energy"))


@dataclass
class Outputs:
    order: np.ndarray
    nbound: np.ndarray
    mbound: np.ndarray
    nbound_type: np.ndarray
    mbound_type: np.ndarray
    tracer_index: np.ndarray
    kinematics: np.ndarray
    core: np.ndarray
    energy: np.ndarray | None
    potential: np.ndarray | None
    iterations: np.ndarray
    status: np.ndarray
    ref_pos: np.ndarray
    ref_vel: np.ndarray
    mostbound_pos: np.ndarray
    mostbound_vel: np.ndarray
    most_bound_id: np.ndarray

    def save(self, path, prefix=""):
        d = {prefix + k: v for k, v in self.__dict__.items() if v is not None}
        np.savez_compressed(path, **d)

    @staticmethod
    def load(npz, prefix="out_"):
        keys = Outputs.__dataclass_fields__.keys()
        return Outputs(**{k: (npz[prefix + k] if (prefix + k) in npz else None) for k in keys})


class CallBuffers:
    """Owns the output arrays of one call and the CBatch pointing at them."""

    def __init__(self, inp: Inputs, want_energy=True, want_potential=False):
        n, ns = inp.n_particles, inp.n_sub
        self.inp = inp
        self.offsets = np.ascontiguousarray(inp.offsets, dtype=np.int64)
        self.pos = np.ascontiguousarray(inp.pos, dtype=np.float32)
        self.vel = np.ascontiguousarray(inp.vel, dtype=np.float32)
        self.mass = np.ascontiguousarray(inp.mass, dtype=np.float32)
        self.id = np.ascontiguousarray(inp.id, dtype=np.int64)
        self.type = None if inp.type is None else np.ascontiguousarray(inp.type, dtype=np.uint8)
        self.u = None if inp.u is None else np.ascontiguousarray(inp.u, dtype=np.float32)
        self.out = Outputs(
            order=np.full(n, -1, np.int64), nbound=np.zeros(ns, np.int64), mbound=np.zeros(ns, np.float32),
            nbound_type=np.zeros((ns, TYPE_MAX), np.int64), mbound_type=np.zeros((ns, TYPE_MAX), np.float32),
            tracer_index=np.zeros(ns, np.int64), kinematics=np.zeros((ns, KIN_STRIDE), np.float32),
            core=np.zeros((ns, CORE_STRIDE), np.float32),
            energy=np.zeros(n, np.float32) if want_energy else None,
            potential=np.zeros(n, np.float32) if want_potential else None,
            iterations=np.zeros(ns, np.int32), status=np.full(ns, -1, np.int32),
            ref_pos=np.array(inp.ref_pos, dtype=np.float32, copy=True, order="C"),
            ref_vel=np.array(inp.ref_vel, dtype=np.float32, copy=True, order="C"),
            mostbound_pos=np.array(inp.mostbound_pos, dtype=np.float32, copy=True, order="C"),
            mostbound_vel=np.array(inp.mostbound_vel, dtype=np.float32, copy=True, order="C"),
            most_bound_id=np.array(inp.most_bound_id, dtype=np.int64, copy=True, order="C"),
        )
        o = self.out
        self.c = CBatch(ns, _ptr(self.offsets), _ptr(self.pos), _ptr(self.vel), _ptr(self.mass), _ptr(self.u),
                        _ptr(self.id), _ptr(self.type), _ptr(o.ref_pos), _ptr(o.ref_vel), _ptr(o.mostbound_pos),
                        _ptr(o.mostbound_vel), _ptr(o.most_bound_id), _ptr(o.order), _ptr(o.nbound),
                        _ptr(o.mbound), _ptr(o.nbound_type), _ptr(o.mbound_type), _ptr(o.tracer_index),
                        _ptr(o.kinematics), _ptr(o.core), _ptr(o.energy), _ptr(o.potential), _ptr(o.iterations),
                        _ptr(o.status))
