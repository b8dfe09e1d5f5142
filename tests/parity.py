"""Parity metrics between two unbinding results on the same inputs.

Tolerances (stated by the project's correctness contract for the plain GPU
path against the reference CPU Unbind):
  * bound-membership mismatch  sum_s |B_s xor B'_s| / sum_s |B'_s| <= 1e-4
  * total bound mass           relative difference <= 1e-5 once the masses of the
                               particles whose membership differs are accounted for
                               (those flips are bounded by the membership bar; a single
                               flip in a small batch alone exceeds 1e-5)
  * per-subhalo status         identical, except where one of the two sits
                               within one particle of the disruption limit
  * most-bound particle        identical ID, or a tie: the two candidates'
                               oracle energies differ by <= ENERGY_TIE_REL*|E|
  * binding energies           FP32 walk vs FP64 walk: median relative
                               difference <= 1e-5 on particles bound in both
"""
from __future__ import annotations

import numpy as np

MEMBERSHIP_TOL = 1e-4
MASS_TOL = 1e-5
ENERGY_TIE_REL = 2e-5


def bound_ids(inp, out, s):
    off = inp.offsets[s]
    nb = int(out.nbound[s])
    return inp.id[off + out.order[off:off + nb]]


def compare(inp, got, ref):
    """Returns a dict of parity metrics of `got` against `ref`."""
    ns = inp.n_sub
    mism = 0
    tot_ref = 0
    flip_mass = 0.0  # mass bound only in got minus mass bound only in ref
    worst_sub_rel = 0.0
    status_diff = []
    mb_diff = []
    e_rel = []
    for s in range(ns):
        a, b = bound_ids(inp, got, s), bound_ids(inp, ref, s)
        tot_ref += len(b)
        if got.status[s] != ref.status[s]:
            status_diff.append(s)
        d = len(np.setxor1d(a, b, assume_unique=True))
        mism += d
        if d:
            off, end = inp.offsets[s], inp.offsets[s + 1]
            ids, ms = inp.id[off:end], inp.mass[off:end].astype(np.float64)
            flip_mass += ms[np.isin(ids, np.setdiff1d(a, b))].sum() - ms[np.isin(ids, np.setdiff1d(b, a))].sum()
        if len(b):
            worst_sub_rel = max(worst_sub_rel, d / len(b))
        if len(a) and len(b):
            if a[0] != b[0]:
                mb_diff.append(s)
            # energies of particles bound in both, by ID
            off = inp.offsets[s]
            ea = dict(zip(a.tolist(), got.energy[off:off + len(a)].tolist()))
            eb = got_e = None
            common = np.intersect1d(a, b, assume_unique=True)
            if len(common):
                eb = dict(zip(b.tolist(), ref.energy[off:off + len(b)].tolist()))
                ga = np.array([ea[i] for i in common[:2000]])
                gb = np.array([eb[i] for i in common[:2000]])
                e_rel.append(np.abs(ga - gb) / np.maximum(np.abs(gb), 1e-30))
    e_rel = np.concatenate(e_rel) if e_rel else np.zeros(1)
    m_got = float(np.sum(got.mbound.astype(np.float64)))
    m_ref = float(np.sum(ref.mbound.astype(np.float64)))
    return dict(
        membership=mism / max(tot_ref, 1),
        worst_sub_membership=worst_sub_rel,
        mass_rel=abs(m_got - m_ref) / max(m_ref, 1e-30),
        mass_rel_residual=abs((m_got - m_ref) - flip_mass) / max(m_ref, 1e-30),
        status_diff=status_diff,
        mostbound_diff=mb_diff,
        energy_rel_median=float(np.median(e_rel)),
        energy_rel_p99=float(np.percentile(e_rel, 99)),
        nbound_got=int(got.nbound.sum()),
        nbound_ref=int(ref.nbound.sum()),
    )


def most_bound_is_tie(inp, got, ref, s):
    """True if the two most-bound particles of subhalo s tie in the ref energies."""
    off = inp.offsets[s]
    nb = int(ref.nbound[s])
    ids_ref = inp.id[off + ref.order[off:off + nb]]
    e_ref = ref.energy[off:off + nb]
    gid = inp.id[off + got.order[off]]
    where = np.nonzero(ids_ref == gid)[0]
    if not len(where):
        return False
    e_min = float(e_ref[0])
    return abs(float(e_ref[where[0]]) - e_min) <= ENERGY_TIE_REL * abs(e_min)


def near_disruption(inp, out, s, params):
    """A subhalo within a few particles of the MinNumPartOfSub limit."""
    nb = int(out.nbound[s])
    return nb <= params.min_num_part + 2


def assert_parity(inp, got, ref, params, membership_tol=MEMBERSHIP_TOL, mass_tol=MASS_TOL):
    m = compare(inp, got, ref)
    bad_status = [s for s in m["status_diff"]
                  if not (near_disruption(inp, got, s, params) or near_disruption(inp, ref, s, params))]
    assert not bad_status, ("status differs", bad_status, got.status[bad_status], ref.status[bad_status])
    assert m["membership"] <= membership_tol, m
    assert m["mass_rel_residual"] <= mass_tol, m
    bad_mb = [s for s in m["mostbound_diff"] if not most_bound_is_tie(inp, got, ref, s)]
    assert not bad_mb, ("most-bound particle differs beyond a tie", bad_mb)
    return m


def check_invariants(inp, out, sorted_energies=True):
    """Structural invariants that hold at any size: order is a permutation of
    each subhalo, bound particles come first with E < 0 sorted ascending
    (not after RefineBindingEnergyOrder, which reorders the most-bound prefix
    without updating its energies), disrupted/empty subhaloes have Nbound = 0
    and identity order."""
    for s in range(inp.n_sub):
        off, end = inp.offsets[s], inp.offsets[s + 1]
        n = end - off
        o = out.order[off:end]
        assert np.array_equal(np.sort(o), np.arange(n)), ("order is not a permutation", s)
        nb = int(out.nbound[s])
        if out.status[s] in (1, 2):
            assert nb == 0
            assert np.array_equal(o, np.arange(n))
        else:
            e = out.energy[off:off + nb]
            assert np.all(e < 0), ("kept particle with E >= 0", s)
            if sorted_energies:
                assert np.all(np.diff(e) >= 0), ("bound set not sorted by energy", s)


# ---------------------------------------------------------------------------
# Full-output parity: every field one call returns.
#
# Bars for a subhalo whose bound ID set is the reference's ("matched"):
#   * bound order      position by position the reference's, except where the
#                      two particles' reference energies tie within
#                      ENERGY_TIE_REL * |potential| (FP32 walk vs the
#                      reference's double walk); skipped under
#                      RefineMostBoundParticle, whose prefix order comes from
#                      energies that are not returned
#   * unbound tail     (removal batches, most recent first, each sorted by
#                      energy; src/subhalo_unbind.cpp:673) the same particles
#                      at each position, except ties moved within a window of
#                      TAIL_WINDOW positions; and the source kept by
#                      TruncateSource (first SourceSubRelaxFactor * Nbound
#                      particles, src/subhalo_unbind.cpp:843-853) the same set
#   * energy, potential |got - ref| <= FLOAT_REL * |potential_ref| for all but
#                      FLOAT_OUTLIER_FRAC of the particles (a borderline
#                      opening decision moves one particle by the tree's own
#                      approximation error)
#   * counts per type  identical; masses (total and per type) FLOAT_REL
#   * frames, kinematics, core phase space  FLOAT_REL relative to the scale of
#                      the quantity (positions: the box, with two float ulps of
#                      the coordinate as a floor)
#   * tracer index, most-bound ID and position/velocity  identical (the
#                      most-bound ID up to an energy tie, as above)
#   * iterations       identical
# Particles near a pair closer than TreeNodeResolution are exempt from the
# energy, potential and order bars (not from membership, mass or IDs): when
# two particles share a cell smaller than the resolution the reference places
# one of them in a child drawn with drand48 (src/oct_tree.tpp:108-120), where
# the GPU keeps their geometric order.  Only targets that open such a cell
# (within len / theta of it, a few resolution lengths) see a different tree;
# the exemption covers everything within SUBRES_REACH resolution lengths.
# Over the whole batch: membership <= MEMBERSHIP_TOL and the raw total bound
# mass within MASS_TOL.
# ---------------------------------------------------------------------------
FLOAT_REL = 1e-5
FLOAT_OUTLIER_FRAC = 1e-3
TAIL_WINDOW = 8
SOURCE_RELAX = 3.0  # SourceSubRelaxFactor default (src/config_parser.cpp)
SUBRES_REACH = 10.0  # exemption radius around sub-resolution pairs, in resolution lengths


def _ulp32(x):
    x = np.abs(np.asarray(x, np.float32))
    return np.spacing(np.maximum(x, np.float32(1e-30))).astype(np.float64)


def _close(got, ref, scale, floor=None):
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    tol = FLOAT_REL * np.asarray(scale, np.float64)
    if floor is not None:
        tol = np.maximum(tol, floor)
    return np.abs(got - ref) <= tol


def compare_full(inp, got, ref, params, refine=None, box=None):
    """Compares every output of `got` with `ref` (same inputs).  Returns
    (metrics, violations): violations is a list of (field, subhalo, detail)."""
    if refine is None:
        refine = bool(params.max_sample_size > 0 and params.refine_most_bound)
    if box is None:
        box = float(params.box_size)
    viol = []
    base = compare(inp, got, ref)
    ns = inp.n_sub
    res = float(params.tree_node_resolution)
    near_ids = subresolution_neighbours(inp, res, SUBRES_REACH * res)
    matched = 0
    tail_moved = 0
    tail_checked = 0
    trunc_mism = 0
    trunc_total = 0
    n_float = 0
    n_float_bad = 0
    iter_diff = 0
    for s in range(ns):
        off, end = int(inp.offsets[s]), int(inp.offsets[s + 1])
        n = end - off
        nbg, nbr = int(got.nbound[s]), int(ref.nbound[s])
        ids_g = inp.id[off + got.order[off:end]]
        ids_r = inp.id[off + ref.order[off:end]]
        # TruncateSource keeps the first max(Nbound * relax, Nbound <= 1) particles
        keep = nbr if nbr <= 1 else min(n, int(nbr * SOURCE_RELAX))
        keep_g = nbg if nbg <= 1 else min(n, int(nbg * SOURCE_RELAX))
        trunc_mism += len(np.setxor1d(ids_g[:keep_g], ids_r[:keep], assume_unique=True))
        trunc_total += keep
        if got.status[s] != ref.status[s]:
            continue
        if nbg != nbr or not np.array_equal(np.sort(ids_g[:nbg]), np.sort(ids_r[:nbr])):
            continue
        matched += 1
        nb = nbr
        if got.iterations[s] != ref.iterations[s]:
            iter_diff += 1
            viol.append(("iterations", s, (int(got.iterations[s]), int(ref.iterations[s]))))
        # scales of this subhalo
        pot_r = ref.potential[off:off + nb] if (ref.potential is not None) else None
        e_r = ref.energy[off:off + nb].astype(np.float64) if ref.energy is not None else None
        escale = np.abs(pot_r).astype(np.float64) if pot_r is not None else (np.abs(e_r) if e_r is not None else None)
        # bound order (ties allowed)
        if nb and not refine and e_r is not None:
            pos_r = {int(i): k for k, i in enumerate(ids_r[:nb])}
            diff = np.nonzero(ids_g[:nb] != ids_r[:nb])[0]
            for k in diff:
                other = pos_r[int(ids_g[k])]
                if int(ids_g[k]) in near_ids or int(ids_r[k]) in near_ids:
                    continue
                if abs(e_r[other] - e_r[k]) > ENERGY_TIE_REL * max(escale[k], escale[other]):
                    viol.append(("bound_order", s, (int(k), int(ids_g[k]), int(ids_r[k]))))
                    break
        # unbound tail: ties moved within a window
        if got.iterations[s] == ref.iterations[s] and n > nb and got.status[s] in (0, 3):
            tg, tr = ids_g[nb:], ids_r[nb:]
            tail_checked += len(tr)
            where_r = {int(i): k for k, i in enumerate(tr)}
            moved = np.nonzero(tg != tr)[0]
            tail_moved += len(moved)
            for k in moved:
                if int(tg[k]) in near_ids or int(tr[k]) in near_ids:
                    continue
                if abs(where_r[int(tg[k])] - int(k)) > TAIL_WINDOW:
                    viol.append(("tail_order", s, (int(k), int(tg[k]), int(tr[k]))))
                    break
        if not nb:
            continue
        # per-particle floats of the bound set, matched by ID
        if escale is not None:
            idx_r = np.argsort(ids_r[:nb])
            idx_g = np.argsort(ids_g[:nb])
            sc = np.maximum(escale[idx_r], 1e-30)
            keep = ~np.isin(np.sort(ids_r[:nb]), np.fromiter(near_ids, np.int64, len(near_ids)))
            for field in ("energy", "potential"):
                a, b = getattr(got, field), getattr(ref, field)
                if a is None or b is None:
                    continue
                va = a[off:off + nb].astype(np.float64)[idx_g]
                vb = b[off:off + nb].astype(np.float64)[idx_r]
                bad = (np.abs(va - vb) > FLOAT_REL * sc) & keep
                n_float += int(keep.sum())
                n_float_bad += int(bad.sum())
        # counts and masses
        if not np.array_equal(got.nbound_type[s], ref.nbound_type[s]):
            viol.append(("nbound_type", s, (got.nbound_type[s].tolist(), ref.nbound_type[s].tolist())))
        if not _close(got.mbound[s], ref.mbound[s], abs(float(ref.mbound[s]))):
            viol.append(("mbound", s, (float(got.mbound[s]), float(ref.mbound[s]))))
        mt = float(np.abs(ref.mbound_type[s]).sum())
        if not np.all(_close(got.mbound_type[s], ref.mbound_type[s], mt)):
            viol.append(("mbound_type", s, (got.mbound_type[s].tolist(), ref.mbound_type[s].tolist())))
        # frames: positions against the box (two ulps floor), velocities against |V| + spread
        if not np.all(_close(got.ref_pos[s], ref.ref_pos[s], 0.0, floor=2 * _ulp32(ref.ref_pos[s]) + FLOAT_REL * 1e-3 * box)):
            viol.append(("ref_pos", s, (got.ref_pos[s].tolist(), ref.ref_pos[s].tolist())))
        vscale = np.linalg.norm(ref.ref_vel[s]) + np.sqrt(max(2.0 * abs(float(ref.kinematics[s][1])), 0.0))
        if not np.all(_close(got.ref_vel[s], ref.ref_vel[s], vscale)):
            viol.append(("ref_vel", s, (got.ref_vel[s].tolist(), ref.ref_vel[s].tolist())))
        # kinematics: energies against |<E-K>| + |<K>|, angular momentum against its norm + |r||v| floor
        kg, kr = got.kinematics[s].astype(np.float64), ref.kinematics[s].astype(np.float64)
        esc = abs(kr[0]) + abs(kr[1])
        lsc = np.linalg.norm(kr[2:5]) + np.sqrt(2.0 * abs(kr[1])) * float(ref.core[s][6] if ref.core is not None else 0.0)
        if not (np.all(_close(kg[:2], kr[:2], esc)) and np.all(_close(kg[2:], kr[2:], lsc))):
            viol.append(("kinematics", s, (kg.tolist(), kr.tolist())))
        # most-bound particle: position/velocity are its own input values
        if ids_g[0] == ids_r[0]:
            if not (np.array_equal(got.mostbound_pos[s], ref.mostbound_pos[s])
                    and np.array_equal(got.mostbound_vel[s], ref.mostbound_vel[s])):
                viol.append(("mostbound_pos_vel", s, None))
            if got.tracer_index[s] != ref.tracer_index[s] and not refine:
                viol.append(("tracer_index", s, (int(got.tracer_index[s]), int(ref.tracer_index[s]))))
            if got.most_bound_id[s] != ref.most_bound_id[s] and not most_bound_is_tie(inp, got, ref, s):
                viol.append(("most_bound_id", s, (int(got.most_bound_id[s]), int(ref.most_bound_id[s]))))
        # core phase space: only where both used the same core particles
        if got.core is not None and ref.core is not None:
            core_n = max(int(np.float32(nb) * np.float32(params.sub_core_size_factor)), int(params.sub_core_size_min))
            tr_mask = _tracer_mask(inp, params, off, end)
            cg = _core_ids(ids_g[:nb], got.order[off:off + nb], tr_mask, core_n)
            cr = _core_ids(ids_r[:nb], ref.order[off:off + nb], tr_mask, core_n)
            if np.array_equal(np.sort(cg), np.sort(cr)):
                c_g, c_r = got.core[s].astype(np.float64), ref.core[s].astype(np.float64)
                okp = _close(c_g[:3], c_r[:3], 0.0, floor=2 * _ulp32(c_r[:3]) + FLOAT_REL * 1e-3 * box)
                vsc = np.linalg.norm(c_r[3:6]) + c_r[7]
                okv = _close(c_g[3:6], c_r[3:6], vsc)
                oks = _close(c_g[6:8], c_r[6:8], np.abs(c_r[6:8]), floor=2 * _ulp32(c_r[6:8]))
                if not (np.all(okp) and np.all(okv) and np.all(oks)):
                    viol.append(("core", s, (c_g.tolist(), c_r.tolist())))
    if n_float and n_float_bad > FLOAT_OUTLIER_FRAC * n_float:
        viol.append(("energy/potential", -1, (n_float_bad, n_float)))
    # the truncated source differs only through membership flips (bounded above)
    # and tail ties moved across its end (bounded by the window check)
    if trunc_mism > 10 * MEMBERSHIP_TOL * max(trunc_total, 1):
        viol.append(("truncated_source", -1, (trunc_mism, trunc_total)))
    m = dict(base)
    m.update(matched=matched, n_sub=ns, subres_exempt=len(near_ids), tail_moved=tail_moved, tail_checked=tail_checked,
             trunc_mismatch=trunc_mism / max(trunc_total, 1), float_outliers=n_float_bad / max(n_float, 1),
             iter_diff=iter_diff)
    return m, viol


def subresolution_neighbours(inp, res, reach):
    """IDs of the particles within `reach` of a particle that has another one
    closer than `res` in its subhalo (positions as stored: the tree's cube
    is built on them)."""
    from scipy.spatial import cKDTree
    out = set()
    for s in range(inp.n_sub):
        off, end = int(inp.offsets[s]), int(inp.offsets[s + 1])
        if end - off < 2:
            continue
        x = np.asarray(inp.pos[off:end], np.float64)
        tree = cKDTree(x)
        pairs = tree.query_pairs(r=res, output_type="ndarray")
        if not len(pairs):
            continue
        members = np.unique(pairs.ravel())
        hit = set()
        for lst in tree.query_ball_point(x[members], r=reach):
            hit.update(lst)
        out.update(int(i) for i in inp.id[off + np.fromiter(hit, np.int64, len(hit))])
    return out


def _tracer_mask(inp, params, off, end):
    if params.dm_only or inp.type is None:
        return np.ones(end - off, bool)
    t = inp.type[off:end].astype(np.int64)
    return ((int(params.tracer_type_mask) >> t) & 1).astype(bool)


def _core_ids(ids_bound, order_bound, tracer_mask, core_n):
    """IDs of the particles GetCorePhaseSpaceProperties uses (first core_n
    tracers in bound order, then non-tracers; src/subhalo_merge.cpp:120-150)."""
    tr = tracer_mask[order_bound]
    first = ids_bound[tr][:core_n]
    if len(first) < core_n:
        first = np.concatenate([first, ids_bound[~tr][:core_n - len(first)]])
    return first


def assert_full_parity(inp, got, ref, params, membership_tol=MEMBERSHIP_TOL, mass_tol=MASS_TOL, **kw):
    """assert_parity plus every other output field (compare_full) and the raw
    total bound mass."""
    m0 = assert_parity(inp, got, ref, params, membership_tol=membership_tol, mass_tol=mass_tol)
    m, viol = compare_full(inp, got, ref, params, **kw)
    assert m0["mass_rel"] <= mass_tol, ("raw total bound mass", m0)
    assert not viol, (viol[:10], len(viol), m)
    return m
