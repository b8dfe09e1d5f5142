"""Seeded synthetic subhaloes (no simulation data is available; these stand
in for the reference's COLIBRE/FLAMINGO inputs with the shapes, sizes and
value distributions of the benchmark workloads).

Every generator returns an ``abi.Inputs`` batch: float32 positions in a
periodic box, float32 velocities, particle masses, int64 IDs, optional types
and thermal energies, and the initial reference frame the reference expects
before Unbind -- the mass-weighted centre of all source particles wrapped
about particle 0 (AveragePosition / AverageVelocity, src/snapshot.cpp:163-233).

Units: G = 1, particle mass 1 for dark matter.  A 1e5-particle c=10 NFW halo
has r_200 = 1; other haloes keep the same mean density inside r_200.

Workloads
  nfw_single       one 1e5 NFW halo, 10% interlopers at 3 v_esc, 100-unit box
  batched          N_p ~ N^-1.9 on [20, 1e6], c ~ logN(ln 8, 0.3),
                   f_unbound ~ U(0, 0.5) heated to U(1.5, 4) v_esc, 500-unit box
  hydro            55% DM, 35% gas (m=0.19, thermal u), 9.9% stars (Hernquist),
                   0.1% black holes (m=50) at the centre; N_p on [100, 2e5]
  precision_host   a 1e7 host (c=5) with satellites, straddling a box face
  stripped         tidally stripped NFW subhaloes with a previous-output bound
                   set (training and evaluation of the learned warm start)
"""
from __future__ import annotations

import numpy as np

from .abi import Inputs

TYPE_GAS, TYPE_DM, TYPE_STAR, TYPE_BH = 0, 1, 4, 5


def _m(x):
    """NFW enclosed-mass shape m(x) = ln(1+x) - x/(1+x)."""
    return np.log1p(x) - x / (1.0 + x)


class _NFWTables:
    """Universal NFW tables in units of r_s: inverse of m(x) and the isotropic
    Jeans dispersion sigma_r^2 = (G M200 / (r_s m(c))) * f(x)."""

    def __init__(self):
        x = np.logspace(-7, 4, 20001)
        self.x = x
        self.mx = _m(x)
        # f(x) = x (1+x)^2 * int_x^inf m(t) / (t^3 (1+t)^2) dt  (trapezoid on log grid)
        integrand = _m(x) / (x ** 3 * (1 + x) ** 2) * x  # d t = t d ln t
        lnx = np.log(x)
        seg = 0.5 * (integrand[1:] + integrand[:-1]) * np.diff(lnx)
        tail = np.concatenate([np.cumsum(seg[::-1])[::-1], [0.0]])
        self.f = x * (1 + x) ** 2 * tail

    def inv_m(self, y):
        return np.interp(y, self.mx, self.x)

    def sigma2_shape(self, xs):
        return np.interp(np.log(xs), np.log(self.x), self.f)


_TABLES = None


def _tables():
    global _TABLES
    if _TABLES is None:
        _TABLES = _NFWTables()
    return _TABLES


def r200_of(m200):
    """r_200 at the fixed mean density set by a 1e5-particle c=10 halo with r_200=1."""
    m200_ref = 1e5 * _m(10.0) / _m(20.0)
    return (m200 / m200_ref) ** (1.0 / 3.0)


def _random_dirs(rng, n):
    v = rng.standard_normal((n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v


def _wrap(x, box):
    x = np.mod(x, box)
    x[x >= box] -= box  # float64 mod can round up to box
    return x


def _initial_frame(pos32, vel32, mass32, offsets, box, periodic=True):
    """AveragePosition / AverageVelocity of each subhalo (src/snapshot.cpp:163-233):
    double sums, wrapped about the first particle, stored as float."""
    ns = len(offsets) - 1
    counts = np.diff(offsets)
    seg = np.repeat(np.arange(ns), counts)
    m = mass32.astype(np.float64)
    msum = np.bincount(seg, weights=m, minlength=ns)
    origin = np.zeros((ns, 3))
    has = counts > 0
    origin[has] = pos32[offsets[:-1][has]].astype(np.float64)
    half = np.float64(np.float32(box) / 2)
    ref_pos = np.zeros((ns, 3), np.float32)
    ref_vel = np.zeros((ns, 3), np.float32)
    for d in range(3):
        dx = pos32[:, d].astype(np.float64) - origin[seg, d]
        if periodic:
            dx = np.where(dx > half, dx - np.float32(box), np.where(dx < -half, dx + np.float32(box), dx))
        sx = np.bincount(seg, weights=dx * m, minlength=ns)
        sv = np.bincount(seg, weights=vel32[:, d].astype(np.float64) * m, minlength=ns)
        with np.errstate(invalid="ignore", divide="ignore"):
            ref_pos[:, d] = np.where(has, sx / msum + origin[:, d], 0.0)
            ref_vel[:, d] = np.where(has, sv / msum, 0.0)
    one = counts == 1
    ref_pos[one] = pos32[offsets[:-1][one]]
    ref_vel[one] = vel32[offsets[:-1][one]]
    return ref_pos, ref_vel


def _power_law_counts(rng, nmin, nmax, slope, total=None, count=None):
    """Draws N_p from dN/dN_p ~ N_p^-slope on [nmin, nmax] (inverse CDF) until
    `count` draws or until the sum reaches `total`."""
    a = 1.0 - slope
    lo, hi = nmin ** a, nmax ** a

    def draw(k):
        u = rng.random(k)
        return np.floor((lo + u * (hi - lo)) ** (1.0 / a)).astype(np.int64).clip(nmin, nmax)

    if count is not None:
        return draw(count)
    out, s = [], 0
    while s < total:
        chunk = draw(max(1024, int((total - s) / 300)))
        cs = np.cumsum(chunk)
        k = np.searchsorted(cs, total - s)
        take = chunk[: k + 1]
        out.append(take)
        s += int(take.sum())
    return np.concatenate(out)


def _nfw_halo_particles(rng, counts, conc, m_part, frac_heat, heat_lo, heat_hi, interloper, box, centres,
                        bulk_vel, do_wrap=True):
    """Positions/velocities of NFW haloes (truncated at 2 r_200), vectorised
    over haloes.  A fraction of particles is heated (speed U(heat_lo, heat_hi)
    v_esc, random direction) in place or, if `interloper`, replaced by
    interlopers uniform in the r < 2 r_200 sphere."""
    T = _tables()
    nh = len(counts)
    seg = np.repeat(np.arange(nh), counts)
    n = int(counts.sum())
    c = conc[seg]
    m200 = counts * m_part * _m(conc) / _m(2 * conc)
    r200 = r200_of(m200)
    rs = (r200 / conc)[seg]
    # radii by inverse CDF of m(x) truncated at x = 2c
    y = rng.random(n) * _m(2 * c)
    x = T.inv_m(y).clip(1e-7, None)
    r = x * rs
    pos = _random_dirs(rng, n) * r[:, None]
    vscale2 = (m200 / (r200 / conc) / _m(conc))[seg]  # G M200 / (r_s m(c)), G=1
    sig = np.sqrt(vscale2 * T.sigma2_shape(x))
    vel = rng.standard_normal((n, 3)) * sig[:, None]
    heated = rng.random(n) < frac_heat[seg]
    k = int(heated.sum())
    if k:
        if interloper:
            rr = 2.0 * r200[seg[heated]] * rng.random(k) ** (1.0 / 3.0)
            pos[heated] = _random_dirs(rng, k) * rr[:, None]
            xh = (rr / rs[heated]).clip(1e-7, None)
        else:
            xh = x[heated]
        vesc = np.sqrt(2.0 * vscale2[heated] * np.log1p(xh) / xh)  # untruncated NFW |phi|
        factor = rng.uniform(heat_lo, heat_hi, k) if heat_hi > heat_lo else np.full(k, heat_lo)
        vel[heated] = _random_dirs(rng, k) * (factor * vesc)[:, None]
    pos = pos + centres[seg]
    if do_wrap:
        pos = _wrap(pos, box)
    vel = vel + bulk_vel[seg]
    return pos, vel, seg, r200


def _finish(pos, vel, mass, counts, box, rng, typ=None, u=None, meta=None):
    offsets = np.zeros(len(counts) + 1, np.int64)
    np.cumsum(counts, out=offsets[1:])
    pos32 = pos.astype(np.float32)
    pos32[pos32 >= np.float32(box)] = 0.0  # float rounding onto the box edge
    vel32 = vel.astype(np.float32)
    mass32 = np.asarray(mass, dtype=np.float32)
    n = int(offsets[-1])
    ids = rng.permutation(n).astype(np.int64) * 7 + 11  # unique, unordered IDs
    ref_pos, ref_vel = _initial_frame(pos32, vel32, mass32, offsets, box)
    first = offsets[:-1].clip(0, max(n - 1, 0))
    has = counts > 0
    mb_pos = np.where(has[:, None], pos32[first] if n else 0, ref_pos).astype(np.float32)
    mb_vel = np.where(has[:, None], vel32[first] if n else 0, ref_vel).astype(np.float32)
    mb_id = np.where(has, ids[first] if n else -1, -1).astype(np.int64)
    return Inputs(offsets, pos32, vel32, mass32, ids, typ, None if u is None else u.astype(np.float32), ref_pos,
                  ref_vel, mb_pos, mb_vel, mb_id, meta or {})


def nfw_single(n=100_000, seed=0, conc=10.0, box=100.0, interloper_frac=0.1, interloper_speed=3.0):
    """One NFW subhalo of `n` m=1 DM particles (r_200 = 1 for n=1e5, c=10),
    with `interloper_frac` of them replaced by uniform interlopers within
    2 r_200 at `interloper_speed` times the local escape speed."""
    rng = np.random.Generator(np.random.PCG64(seed))
    counts = np.array([n], np.int64)
    centre = rng.random((1, 3)) * box
    bulk = rng.standard_normal((1, 3)) * 50.0
    pos, vel, seg, r200 = _nfw_halo_particles(rng, counts, np.array([conc]), 1.0, np.array([interloper_frac]),
                                              interloper_speed, interloper_speed, True, box, centre, bulk)
    return _finish(pos, vel, np.ones(n), counts, box, rng,
                   meta=dict(workload="nfw_single", n=n, seed=seed, box=box, r200=float(r200[0])))


def batched(total=50_000_000, seed=0, n_sub=None, nmin=20, nmax=1_000_000, box=500.0):
    """Batched plain workload: N_p ~ N^-1.9 on [nmin, nmax], drawn until the
    sum reaches `total` (or exactly `n_sub` subhaloes if given)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    counts = _power_law_counts(rng, nmin, nmax, 1.9, total=None if n_sub else total, count=n_sub)
    nh = len(counts)
    conc = np.exp(rng.normal(np.log(8.0), 0.3, nh))
    fheat = rng.uniform(0.0, 0.5, nh)
    centres = rng.random((nh, 3)) * box
    bulk = rng.standard_normal((nh, 3)) * 50.0
    pos, vel, seg, r200 = _nfw_halo_particles(rng, counts, conc, 1.0, fheat, 1.5, 4.0, False, box, centres, bulk)
    return _finish(pos, vel, np.ones(len(pos)), counts, box, rng,
                   meta=dict(workload="batched", seed=seed, box=box, n_sub=nh, n=int(counts.sum())))


def hydro(total=4_000_000, seed=0, n_sub=None, nmin=100, nmax=200_000, box=500.0):
    """Mixed-species workload: 55% DM (m=1), 35% gas (m=0.19, u ~ logN(ln 0.3 sigma^2, 0.5),
    0.3 v_circ rotation about z), 9.9% stars (m=0.19, Hernquist a = 0.05 r_200),
    0.1% black holes (m=50) within 0.01 r_200 of the centre."""
    rng = np.random.Generator(np.random.PCG64(seed))
    counts = _power_law_counts(rng, nmin, nmax, 1.9, total=None if n_sub else total, count=n_sub)
    nh = len(counts)
    conc = np.exp(rng.normal(np.log(8.0), 0.3, nh))
    fheat = rng.uniform(0.0, 0.3, nh)
    centres = rng.random((nh, 3)) * box
    bulk = rng.standard_normal((nh, 3)) * 50.0
    pos, vel, seg, r200 = _nfw_halo_particles(rng, counts, conc, 1.0, fheat, 1.5, 4.0, False, box, np.zeros((nh, 3)),
                                              bulk, do_wrap=False)
    n = len(pos)
    u01 = rng.random(n)
    typ = np.full(n, TYPE_DM, np.uint8)
    typ[u01 < 0.35] = TYPE_GAS
    typ[(u01 >= 0.35) & (u01 < 0.449)] = TYPE_STAR
    typ[(u01 >= 0.449) & (u01 < 0.45)] = TYPE_BH
    mass = np.ones(n)
    mass[typ == TYPE_GAS] = 0.19
    mass[typ == TYPE_STAR] = 0.19
    mass[typ == TYPE_BH] = 50.0
    rel = pos  # relative to the halo centre; centres are added below
    m200 = counts * _m(conc) / _m(2 * conc)
    vc = np.sqrt(m200 / r200_of(m200))  # circular speed at r_200, G=1
    # stars: Hernquist radii, a = 0.05 r_200, truncated at 2 r_200
    st = typ == TYPE_STAR
    if st.any():
        a = 0.05 * r200[seg[st]]
        rmax = 2 * r200[seg[st]]
        q = rng.random(int(st.sum())) * (rmax / (rmax + a)) ** 2
        rs_ = a * np.sqrt(q) / (1 - np.sqrt(q))
        rel[st] = _random_dirs(rng, int(st.sum())) * rs_[:, None]
    bh = typ == TYPE_BH
    if bh.any():
        rel[bh] = _random_dirs(rng, int(bh.sum())) * (0.01 * r200[seg[bh]] * rng.random(int(bh.sum())))[:, None]
        vel[bh] = bulk[seg[bh]] + rng.standard_normal((int(bh.sum()), 3)) * 0.05 * vc[seg[bh]][:, None]
    gas = typ == TYPE_GAS
    u = np.zeros(n)
    if gas.any():
        # rotation 0.3 v_circ about z on top of the Jeans velocities
        rg = rel[gas]
        phi_hat = np.stack([-rg[:, 1], rg[:, 0], np.zeros(len(rg))], 1)
        norm = np.linalg.norm(phi_hat, axis=1, keepdims=True)
        phi_hat = np.divide(phi_hat, norm, out=np.zeros_like(phi_hat), where=norm > 0)
        vel[gas] += 0.3 * vc[seg[gas]][:, None] * phi_hat
        sig2 = (vc[seg[gas]] ** 2) / 2.0
        u[gas] = np.exp(rng.normal(np.log(0.3 * sig2), 0.5))
    pos = _wrap(rel + centres[seg], box)
    return _finish(pos, vel, mass, counts, box, rng, typ=typ, u=u,
                   meta=dict(workload="hydro", seed=seed, box=box, n_sub=nh, n=n))


def precision_host(n_host=10_000_000, n_sat=200, seed=0, box=100.0):
    """A c=5 host of n_host particles with n_sat NFW satellites of 1e3-1e5
    particles on bound orbits inside it, centred 0.3 r_200 from a box face so
    that it straddles the periodic boundary.  Returned as one subhalo."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sat_counts = _power_law_counts(rng, 1000, 100_000, 1.9, count=n_sat)
    m200 = n_host * _m(5.0) / _m(10.0)
    r200h = r200_of(m200)
    centre = np.array([[0.3 * r200h, box / 2, box / 2]])
    hpos, hvel, _, _ = _nfw_halo_particles(rng, np.array([n_host]), np.array([5.0]), 1.0, np.array([0.0]), 1, 1,
                                           False, box, centre, np.zeros((1, 3)))
    sc = np.exp(rng.normal(np.log(10.0), 0.3, n_sat))
    rorb = r200h * rng.uniform(0.1, 1.0, n_sat)
    sat_centres = centre + _random_dirs(rng, n_sat) * rorb[:, None]
    vhost = np.sqrt(m200 * _m(5.0 * rorb / r200h) / _m(5.0) / rorb)  # circular speed, G=1
    sat_bulk = _random_dirs(rng, n_sat) * (0.7 * vhost)[:, None]
    spos, svel, _, _ = _nfw_halo_particles(rng, sat_counts, sc, 1.0, np.zeros(n_sat), 1, 1, False, box, sat_centres,
                                           sat_bulk)
    pos = np.concatenate([hpos, spos])
    vel = np.concatenate([hvel, svel])
    counts = np.array([len(pos)], np.int64)
    return _finish(pos, vel, np.ones(len(pos)), counts, box, rng,
                   meta=dict(workload="precision_host", seed=seed, box=box, n=len(pos), r200=float(r200h)))


def stripped(n_sub=20_000, seed=0, nmin=20, nmax=1_000_000, box=500.0, flip=0.05, with_prior=True):
    """Tidally stripped NFW subhaloes with a previous-output bound set.

    N_p ~ N^-1.9 on [nmin, nmax]; c ~ logN(ln 8, 0.3).  Each is truncated at a
    radius U(0.2, 1.5) r_200 (the remnant keeps the Jeans velocities of the
    untruncated halo), and a fraction U(0, 0.6) of its particles receives a
    tidal kick of U(0.2, 1.5) v_esc in a random direction.  The previous
    output's view is the un-kicked particle in the untruncated potential:
    bound where 1/2 v^2 + phi_NFW(r) < 0, with a fraction `flip` of the
    memberships flipped at random, and that energy as its binding energy.
    As in HBT-HERONS, each subhalo lists its previously bound particles first
    (prior_nbound of them, prior_energy their energies)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    T = _tables()
    counts = _power_law_counts(rng, nmin, nmax, 1.9, count=n_sub)
    nh = len(counts)
    conc = np.exp(rng.normal(np.log(8.0), 0.3, nh))
    rt_frac = rng.uniform(0.2, 1.5, nh)
    fkick = rng.uniform(0.0, 0.6, nh)
    seg = np.repeat(np.arange(nh), counts)
    n = int(counts.sum())
    m200 = counts / _m(conc * rt_frac) * _m(conc)  # unit-mass particles fill the truncated remnant
    r200 = r200_of(m200)
    rs = (r200 / conc)[seg]
    xt = (conc * rt_frac)[seg]
    x = T.inv_m(rng.random(n) * _m(xt)).clip(1e-7, None)
    r = x * rs
    pos = _random_dirs(rng, n) * r[:, None]
    vscale2 = (m200 / (r200 / conc) / _m(conc))[seg]
    vel = rng.standard_normal((n, 3)) * np.sqrt(vscale2 * T.sigma2_shape(x))[:, None]
    phi = -vscale2 * np.log1p(x) / x
    e_prev = 0.5 * np.sum(vel * vel, axis=1) + phi
    prev = e_prev < 0
    prev ^= rng.random(n) < flip
    kicked = rng.random(n) < fkick[seg]
    k = int(kicked.sum())
    if k:
        vesc = np.sqrt(2.0 * -phi[kicked])
        vel[kicked] += _random_dirs(rng, k) * (rng.uniform(0.2, 1.5, k) * vesc)[:, None]
    centres = rng.random((nh, 3)) * box
    bulk = rng.standard_normal((nh, 3)) * 50.0
    pos = _wrap(pos + centres[seg], box)
    vel = vel + bulk[seg]
    # previously bound particles first within each subhalo (stable)
    order = np.lexsort((~prev, seg))
    pos, vel, e_prev, prev = pos[order], vel[order], e_prev[order], prev[order]
    inp = _finish(pos, vel, np.ones(n), counts, box, rng,
                  meta=dict(workload="stripped", seed=seed, box=box, n_sub=nh, n=n))
    if with_prior:
        inp.prior_nbound = np.bincount(seg, weights=prev, minlength=nh).astype(np.int64)
        inp.prior_energy = e_prev.astype(np.float32)
    return inp


def nested_system(seed=0, n_host=20_000, n_sat=6, n_subsat=3, box=100.0, n_merge=0):
    """A FoF-like subhalo tree for nested unbinding: a host NFW halo (c=6),
    n_sat satellites (NFW, 300-3000 particles, 20 % heated) on orbits inside it,
    and n_subsat sub-satellites (NFW, 60-300 particles) inside the first
    satellites.  Every subhalo's source is its own particles; the host centre
    sits near a box corner so the system straddles the periodic boundary.
    With n_merge > 0, compact satellites that overlap a subhalo in phase
    space are added (MergeRecursively's case): the first at the host's centre
    with the host's velocity, the second at the first satellite's centre with
    its velocity (nested in it), alternating.
    Returns (nested.Particles, members, parent, frames)."""
    from .nested import Particles
    rng = np.random.Generator(np.random.PCG64(seed))
    comps, parent = [], []
    m200 = n_host * _m(6.0) / _m(12.0)
    r200h = r200_of(m200)
    centre = np.array([[0.2 * r200h, box - 0.1 * r200h, box / 2]])
    hp, hv, _, _ = _nfw_halo_particles(rng, np.array([n_host]), np.array([6.0]), 1.0, np.array([0.1]), 1.5, 3.0,
                                       False, box, centre, np.zeros((1, 3)), do_wrap=False)
    comps.append((hp, hv))
    parent.append(-1)
    sat_centres = []
    for i in range(n_sat):
        n = int(rng.integers(300, 3000))
        rr = r200h * rng.uniform(0.2, 0.8)
        c = centre + _random_dirs(rng, 1) * rr
        vc = np.sqrt(m200 * _m(6.0 * rr / r200h) / _m(6.0) / rr)
        v = _random_dirs(rng, 1) * 0.7 * vc
        p, vel, _, _ = _nfw_halo_particles(rng, np.array([n]), np.array([10.0]), 1.0, np.array([0.2]), 1.5, 3.0,
                                           False, box, c, v, do_wrap=False)
        comps.append((p, vel))
        parent.append(0)
        sat_centres.append((c, v, r200_of(n * _m(10.0) / _m(20.0))))
    for j in range(n_subsat):
        c0, v0, r0 = sat_centres[j % len(sat_centres)]
        n = int(rng.integers(60, 300))
        c = c0 + _random_dirs(rng, 1) * r0 * rng.uniform(0.2, 0.6)
        p, vel, _, _ = _nfw_halo_particles(rng, np.array([n]), np.array([10.0]), 1.0, np.array([0.2]), 1.5, 3.0,
                                           False, box, c, v0, do_wrap=False)
        comps.append((p, vel))
        parent.append(1 + (j % len(sat_centres)))
    for k in range(n_merge):
        n = int(rng.integers(200, 600))
        if k % 2 == 0 or not sat_centres:
            c, v, host = centre, np.zeros((1, 3)), 0
        else:
            c, v, _ = sat_centres[0]
            host = 1
        p, vel, _, _ = _nfw_halo_particles(rng, np.array([n]), np.array([15.0]), 1.0, np.array([0.0]), 1.5, 3.0,
                                           False, box, c + 1e-4 * _random_dirs(rng, 1), v, do_wrap=False)
        comps.append((p, vel))
        parent.append(host)
    counts = np.array([len(p) for p, _ in comps], np.int64)
    pos = _wrap(np.concatenate([p for p, _ in comps]), box)
    vel = np.concatenate([v for _, v in comps])
    inp = _finish(pos, vel, np.ones(len(pos)), counts, box, rng)
    parts = Particles(inp.pos, inp.vel, inp.mass, inp.id)
    members = [np.arange(inp.offsets[s], inp.offsets[s + 1], dtype=np.int64) for s in range(len(counts))]
    frames = dict(ref_pos=inp.ref_pos, ref_vel=inp.ref_vel, mostbound_pos=inp.mostbound_pos,
                  mostbound_vel=inp.mostbound_vel, most_bound_id=inp.most_bound_id)
    return parts, members, np.array(parent, np.int64), frames


def small_cases(seed=0, box=100.0):
    """A small mixed batch for parity tests: NFW haloes of 20-3000 particles,
    one empty subhalo, one single-particle subhalo, a halo straddling the box
    corner, coincident particles, and a halo that disrupts."""
    rng = np.random.Generator(np.random.PCG64(seed))
    parts = []

    def nfw(n, c, fheat, centre, speed=(1.5, 4.0)):
        p, v, _, _ = _nfw_halo_particles(rng, np.array([n]), np.array([c]), 1.0, np.array([fheat]), speed[0],
                                         speed[1], False, box, np.asarray(centre, float)[None], rng.standard_normal(
                                             (1, 3)) * 30)
        return p, v

    sizes = [20, 25, 40, 64, 100, 257, 600, 1500, 3000]
    for i, n in enumerate(sizes):
        parts.append(nfw(n, 8.0, 0.2 + 0.03 * i, rng.random(3) * box))
    parts.append((np.zeros((0, 3)), np.zeros((0, 3))))  # empty (orphan)
    parts.append(nfw(1, 8.0, 0.0, rng.random(3) * box))  # single particle: disrupts
    parts.append(nfw(2000, 6.0, 0.3, [0.05, box - 0.02, 0.01]))  # straddles a box corner
    p, v = nfw(500, 8.0, 0.1, rng.random(3) * box)
    p[100:140] = p[99]  # coincident particles (below the tree resolution)
    parts.append((p, v))
    parts.append(nfw(300, 8.0, 0.0, rng.random(3) * box, speed=(5, 5)))
    p, v = parts[-1]
    v[:] = rng.standard_normal(v.shape) * 1e4  # everything unbound -> disrupted
    parts[-1] = (p, v)
    counts = np.array([len(p) for p, _ in parts], np.int64)
    pos = _wrap(np.concatenate([p for p, _ in parts]), box)
    vel = np.concatenate([v for _, v in parts])
    return _finish(pos, vel, np.ones(len(pos)), counts, box, rng, meta=dict(workload="small_cases", seed=seed,
                                                                            box=box))


def small_hydro(seed=0, n_sub=12, box=200.0):
    """A small mixed-species batch for parity tests."""
    return hydro(seed=seed, n_sub=n_sub, nmin=100, nmax=3000, box=box)


def fof_groups(seed=0, n_groups=6, n_sat=3, box=300.0, swap=0.1):
    """FoF groups for particle reassignment: each group is a hydro host halo
    (2,000-8,000 particles) and `n_sat` satellites (200-1,000) placed inside
    it, with a fraction `swap` of every subhalo's gas particles exchanged with
    another subhalo of the same group (gas listed in the wrong source).
    Returns (Inputs with the subhaloes grouped, group_off)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    per = 1 + n_sat
    counts = np.concatenate([[rng.integers(2000, 8000)] + list(rng.integers(200, 1000, n_sat)) for _ in range(n_groups)])
    base = hydro(seed=seed + 1000, n_sub=len(counts), nmin=200, nmax=8000, box=box)
    # resample each subhalo to its planned size by taking its first particles (its own profile)
    sizes = np.diff(base.offsets)
    take = np.minimum(sizes, counts)
    rows = [np.arange(base.offsets[s], base.offsets[s] + take[s]) for s in range(len(counts))]
    pos = [base.pos[r].astype(np.float64) for r in rows]
    for g in range(n_groups):
        h = g * per
        hc = pos[h].mean(0)
        spread = np.std(pos[h] - hc) + 1e-3
        for k in range(1, per):
            c = pos[h + k].mean(0)
            pos[h + k] += hc + rng.normal(0, 0.6 * spread, 3) - c
    members = [list(range(len(r))) for r in rows]
    pos_all = [p for p in pos]
    src = [(s, i) for s in range(len(rows)) for i in range(len(rows[s]))]
    lists = [[(s, i) for i in range(len(rows[s]))] for s in range(len(rows))]
    for g in range(n_groups):
        subs = list(range(g * per, (g + 1) * per))
        for s in subs:
            gas = [t for t in lists[s] if base.type[rows[t[0]][t[1]]] == 0]
            n_move = int(swap * len(gas))
            pick = rng.choice(len(gas), n_move, replace=False) if n_move else []
            for q in pick:
                other = int(rng.choice([u for u in subs if u != s]))
                lists[s].remove(gas[q])
                lists[other].append(gas[q])
    P = np.concatenate([[pos_all[s][i] for (s, i) in L] for L in lists if L]).astype(np.float32)
    V = np.concatenate([[base.vel[rows[s][i]] for (s, i) in L] for L in lists if L]).astype(np.float32)
    M = np.concatenate([[base.mass[rows[s][i]] for (s, i) in L] for L in lists if L]).astype(np.float32)
    T = np.concatenate([[base.type[rows[s][i]] for (s, i) in L] for L in lists if L]).astype(np.uint8)
    U = np.concatenate([[base.u[rows[s][i]] for (s, i) in L] for L in lists if L]).astype(np.float32)
    cnt = np.array([len(L) for L in lists], np.int64)
    P = _wrap(P.astype(np.float64), box).astype(np.float32)
    inp = _finish(P, V, M, cnt, box, rng, typ=T, u=U, meta=dict(workload="fof_groups", seed=seed))
    group_off = np.arange(0, len(cnt) + 1, per, dtype=np.int64)
    return inp, group_off
