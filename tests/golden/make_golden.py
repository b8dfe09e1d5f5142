"""Generates the golden fixtures of tests/golden/ by running the REFERENCE's
own Subhalo_t::Unbind (compiled from the reference sources by
oracle/build_oracle.py into oracle/_ref/) on seeded synthetic inputs.

Run from the repository root where the reference sources are present:
    python tests/golden/make_golden.py
Each fixture holds the inputs (prefix in_), the parameters (prefix prm_) and
the reference outputs (prefix out_).
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "hbt-herons_gb300"))

from hbtg import abi, oracle, synthetic  # noqa: E402

CASES = {
    "small_dmo": (lambda: synthetic.small_cases(seed=0), dict(dm_only=1, box_size=100.0)),
    "small_dmo_seed1": (lambda: synthetic.small_cases(seed=1), dict(dm_only=1, box_size=100.0)),
    "small_hydro": (lambda: synthetic.small_hydro(seed=0), dict(thermal=1, box_size=200.0)),
    "nfw_10k": (lambda: synthetic.nfw_single(n=10_000, seed=3), dict(dm_only=1, box_size=100.0)),
    "batched_200": (lambda: synthetic.batched(n_sub=200, seed=4, nmax=4000), dict(dm_only=1, box_size=500.0)),
    # potential subsampling on (the reference default MaxSampleSizeOfPotentialEstimate = 1000)
    "subsampled_dmo": (lambda: synthetic.batched(n_sub=12, seed=8, nmin=1200, nmax=8000, box=500.0),
                       dict(dm_only=1, box_size=500.0, max_sample_size=1000)),
    "subsampled_hydro": (lambda: synthetic.hydro(seed=9, n_sub=8, nmin=1500, nmax=8000, box=300.0),
                         dict(thermal=1, box_size=300.0, max_sample_size=1000)),
    # with the Hubble flow on (Hz such that 200 times the critical density is
    # the synthetic haloes' mean density within r_200): also the post-unbind
    # properties (prop_*) of the reference's CalculateProfileProperties,
    # CalculateShape and TruncateSource
    "properties_dmo": (lambda: synthetic.batched(n_sub=150, seed=5, nmax=20_000, box=500.0),
                       dict(dm_only=1, box_size=500.0, hubble=31.6)),
    "properties_hydro": (lambda: synthetic.hydro(seed=3, n_sub=20, nmin=100, nmax=8000, box=300.0),
                         dict(thermal=1, box_size=300.0, hubble=31.6)),
}

PROPS_SNAPSHOT = 7
PROPS_RELAX = 3.0


def props_init(n_sub):
    """In/out property values before the call (a previous snapshot's Vmax and
    SO values, as the reference keeps them in Subhalo_t)."""
    rng = np.random.default_rng(n_sub)
    return {"last_vmax": rng.uniform(0.0, 80.0, n_sub).astype(np.float32),
            "rmax_last": np.full(n_sub, 0.5, np.float32), "snap_last": np.full(n_sub, 3, np.int32),
            "r200": np.full(n_sub, -1.0, np.float32), "m200": np.full(n_sub, -1.0, np.float32)}


def make(name):
    gen, kw = CASES[name]
    inp = gen()
    prm = abi.parity_params(**kw)
    out = oracle.run_reference(inp, prm, nthreads=1, want_potential=True)
    d = {}
    for k in ("offsets", "pos", "vel", "mass", "id", "type", "u", "ref_pos", "ref_vel", "mostbound_pos",
              "mostbound_vel", "most_bound_id"):
        v = getattr(inp, k)
        if v is not None:
            d["in_" + k] = v
    for k, v in prm.as_dict().items():
        d["prm_" + k] = np.array(v)
    for k, v in out.__dict__.items():
        if v is not None:
            d["out_" + k] = v
    if name.startswith("properties"):
        init = props_init(inp.n_sub)
        props = oracle.subhalo_properties(inp, out, prm, snapshot_id=PROPS_SNAPSHOT, source_relax=PROPS_RELAX,
                                          init=init, reference=True)
        for k, v in init.items():
            d["init_" + k] = v
        for k, v in props.as_dict().items():
            d["prop_" + k] = v
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), name + ".npz")
    np.savez_compressed(path, **d)
    return path


NESTED_SNAPSHOT = 9


def make_nested():
    """A nesting forest with subhaloes that overlap in phase space, through the
    reference's own RecursiveUnbind with MergeRecursively, with
    MergeTrappedSubhalos on (ref1_*) and off (ref0_*)."""
    parts, members, parent, frames = synthetic.nested_system(seed=3, n_host=20_000, n_sat=6, n_subsat=3, n_merge=2)
    prm = abi.parity_params(dm_only=1, box_size=100.0)
    d = {"pos": parts.pos, "vel": parts.vel, "mass": parts.mass, "id": parts.id, "parent": parent,
         "member_off": np.concatenate([[0], np.cumsum([len(m) for m in members])]).astype(np.int64),
         "member_idx": np.concatenate(members).astype(np.int64)}
    for k, v in frames.items():
        d["frame_" + k] = np.asarray(v)
    for k, v in prm.as_dict().items():
        d["prm_" + k] = np.array(v)
    for mt in (1, 0):
        r = oracle.reference_recursive_unbind(parts, members, parent, frames, prm, merge_trapped=mt,
                                              snapshot_id=NESTED_SNAPSHOT)
        for k in ("nbound", "mbound", "most_bound_id", "sink_track", "snap_sink", "snap_death"):
            d["ref%d_%s" % (mt, k)] = r[k]
        d["ref%d_ids_off" % mt] = np.concatenate([[0], np.cumsum([len(x) for x in r["ids"]])]).astype(np.int64)
        d["ref%d_ids" % mt] = np.concatenate(r["ids"]).astype(np.int64)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "nested_merge.npz")
    np.savez_compressed(path, **d)
    return path


REASSIGN_K = (1, 10, 32)


def make_reassign():
    """FoF groups with gas listed in the wrong subhalo, and the moves of the
    reference's ReassignParticles logic over its own GeoTree_t neighbour
    search for NumNeighboursForReassignment in REASSIGN_K."""
    inp, group_off = synthetic.fof_groups(seed=1)
    prm = abi.parity_params(thermal=1, box_size=300.0)
    d = {"group_off": group_off}
    for k in ("offsets", "pos", "type"):
        d["in_" + k] = getattr(inp, k)
    for k, v in prm.as_dict().items():
        d["prm_" + k] = np.array(v)
    for k in REASSIGN_K:
        d["dest_%d" % k] = oracle.reassign(inp, group_off, prm, k, reference=True)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reassign_fof.npz")
    np.savez_compressed(path, **d)
    return path


def load_reassign(path):
    """(Inputs with offsets, pos and type; group_off; params; {k: reference dest})."""
    z = np.load(path)
    n = int(z["in_offsets"][-1])
    S = len(z["in_offsets"]) - 1
    zero3 = np.zeros((S, 3), np.float32)
    inp = abi.Inputs(z["in_offsets"], z["in_pos"], np.zeros((n, 3), np.float32), np.ones(n, np.float32),
                     np.arange(n, dtype=np.int64), z["in_type"], None, zero3, zero3, zero3, zero3,
                     np.zeros(S, np.int64))
    prm = abi.Params()
    for k, _ in abi.Params._fields_:
        setattr(prm, k, z["prm_" + k].item())
    return inp, z["group_off"], prm, {k: z["dest_%d" % k] for k in REASSIGN_K}


def load_props(path):
    """(initial in/out property values, reference properties, snapshot id,
    SourceSubRelaxFactor) of a properties fixture."""
    z = np.load(path)
    init = {k[5:]: z[k] for k in z.files if k.startswith("init_")}
    props = {k[5:]: z[k] for k in z.files if k.startswith("prop_")}
    return init, props, PROPS_SNAPSHOT, PROPS_RELAX


def load(path):
    """Returns (inputs, params, reference outputs) of one fixture."""
    z = np.load(path)
    inp = abi.Inputs.load(z, prefix="in_")
    prm = abi.Params()
    for k, _ in abi.Params._fields_:
        setattr(prm, k, z["prm_" + k].item())
    out = abi.Outputs.load(z, prefix="out_")
    return inp, prm, out


if __name__ == "__main__":
    only = sys.argv[1:]
    if not only or "nested_merge" in only:
        print(make_nested())
    if not only or "reassign_fof" in only:
        print(make_reassign())
    for name in CASES:
        if only and name not in only:
            continue
        print(make(name), os.path.getsize(os.path.join(os.path.dirname(os.path.abspath(__file__)), name + ".npz")))
