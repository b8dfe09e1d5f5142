"""The C++ host shim's properties() and reassign() (hbtg_unbind_shim.hpp),
compiled into a program that links libhbtg.so and run on the GPU:
properties() against the reference's own CalculateProfileProperties /
CalculateShape / TruncateSource outputs (src/subhalo.cpp:175-309,
src/subhalo_unbind.cpp:843-853), reassign() against the moves of the
reference's ReassignParticles over its own GeoTree_t search
(src/subhalo_reassign_gas.cpp:65-197) applied as that function applies them:
appended in subhalo then particle order, dropped with the bound/unbound split
kept (KickNullParticles, src/subhalo.cpp:394-430), types counted again
(CountParticleTypes, src/subhalo.cpp:311-392)."""
import glob
import importlib.util
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from test_gpu_properties import _check, _golden

HERE = os.path.dirname(os.path.abspath(__file__))
PROPS = sorted(glob.glob(os.path.join(HERE, "golden", "properties_*.npz")))
REASSIGN = os.path.join(HERE, "golden", "reassign_fof.npz")


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    from hbtg.build import LIB, build_library
    build_library()
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("shim") / "shim_steps_driver")
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-Wno-deprecated-declarations", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "hbt-herons_gb300", "host"), os.path.join(HERE, "shim_steps_driver.cpp"),
           "-o", exe, "-L", os.path.dirname(LIB), "-lhbtg", "-Wl,-rpath," + os.path.dirname(LIB)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return exe


def _raw(a, dt):
    return np.ascontiguousarray(a, dt).tobytes()


class _Props:
    pass


@pytest.mark.gpu
@pytest.mark.parametrize("path", PROPS, ids=[os.path.basename(p)[:-4] for p in PROPS])
def test_shim_properties_match_reference(driver, tmp_path, path):
    inp, prm, ref, init, props, snap, relax = _golden(path)
    S, N = inp.n_sub, inp.n_particles
    inf, outf = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    with open(inf, "wb") as f:
        f.write(bytes(prm))
        f.write(_raw([S, N, snap], np.int64))
        f.write(_raw([relax], np.float64))
        f.write(_raw(inp.offsets, np.int64))
        f.write(_raw(inp.pos, np.float32))
        f.write(_raw(inp.mass, np.float32))
        f.write(_raw(ref.order, np.int64))
        f.write(_raw(ref.nbound, np.int64))
        f.write(_raw(ref.mbound, np.float32))
        f.write(_raw(ref.mostbound_pos, np.float32))
        for k, dt in (("last_vmax", np.float32), ("rmax_last", np.float32), ("snap_last", np.int32),
                      ("r200", np.float32), ("m200", np.float32)):
            f.write(_raw(init[k], dt))
    r = subprocess.run([driver, "props", inf, outf], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-4000:]
    rec = np.dtype([("a", "<f4", 8), ("snap", "<i4"), ("I", "<f4", 6), ("Iw", "<f4", 6), ("kept", "<i8")])
    assert rec.itemsize == 92
    raw = np.fromfile(outf, rec)
    assert len(raw) == S
    got = _Props()
    for i, k in enumerate(("rmax", "vmax", "rhalf", "renclose", "r200", "m200", "last_vmax", "rmax_last")):
        setattr(got, k, raw["a"][:, i])
    got.snap_last, got.inertia, got.inertia_w, got.nsource = raw["snap"], raw["I"], raw["Iw"], raw["kept"]
    _check(got, props)


def _expected_reassign(offsets, group_off, nbound, mass, type_, dest, mask):
    """ReassignParticles' application of the moves, restated in Python."""
    S = len(offsets) - 1
    lists = [list(range(offsets[s], offsets[s + 1])) for s in range(S)]
    moved = 0
    for s in range(S):
        for g in range(offsets[s], offsets[s + 1]):
            if dest[g] >= 0:
                lists[dest[g]].append(g)
                moved += 1
    nb = np.array(nbound, np.int64)
    tracer = np.zeros(S, np.int64)
    ntype = np.zeros((S, 6), np.int64)
    mtype = np.zeros((S, 6), np.float32)
    for h in range(len(group_off) - 1):
        a, b = group_off[h], group_off[h + 1]
        t = type_[offsets[a]:offsets[b]]
        if not np.any(((1 << t.astype(np.int64)) & mask) == 0):
            continue
        for s in range(a, b):
            n0 = offsets[s + 1] - offsets[s]
            nbs = min(nb[s], len(lists[s]))
            keep, kept_bound = [], 0
            for k, g in enumerate(lists[s]):
                if k < n0 and dest[offsets[s] + k] >= 0:
                    continue
                kept_bound += k < nbs
                keep.append(g)
            lists[s], nb[s] = keep, kept_bound
            first = -1
            for k in range(kept_bound):
                g = keep[k]
                ntype[s, type_[g]] += 1
                mtype[s, type_[g]] = np.float32(mtype[s, type_[g]] + mass[g])
                if first < 0 and (1 << int(type_[g])) & mask:
                    first = k
            tracer[s] = max(first, 0)
    return moved, lists, nb, tracer, ntype, mtype


@pytest.mark.gpu
@pytest.mark.parametrize("k", [1, 10, 32])
def test_shim_reassign_applies_reference_moves(driver, tmp_path, k):
    z = np.load(REASSIGN)
    prm = __import__("hbtg.abi", fromlist=["Params"]).Params()
    for name, _ in type(prm)._fields_:
        setattr(prm, name, z["prm_" + name].item())
    offsets, group_off, pos, type_ = z["in_offsets"], z["group_off"], z["in_pos"], z["in_type"]
    S, N, G = len(offsets) - 1, int(offsets[-1]), len(group_off) - 1
    rng = np.random.default_rng(5)
    nbound = np.diff(offsets) // 2  # a bound head and an unbound tail in every source
    mass = rng.uniform(0.5, 2.0, N).astype(np.float32)
    inf, outf = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    with open(inf, "wb") as f:
        f.write(bytes(prm))
        f.write(_raw([G, S, N, k], np.int64))
        f.write(_raw(group_off, np.int64))
        f.write(_raw(offsets, np.int64))
        f.write(_raw(nbound, np.int64))
        f.write(_raw(pos, np.float32))
        f.write(_raw(mass, np.float32))
        f.write(_raw(type_, np.uint8))
    r = subprocess.run([driver, "reassign", inf, outf], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-4000:]
    raw = open(outf, "rb").read()
    moved, lists, nb, tracer, ntype, mtype = _expected_reassign(offsets, group_off, nbound, mass, type_,
                                                                z["dest_%d" % k], int(prm.tracer_type_mask))
    assert moved > 0
    assert int(np.frombuffer(raw, np.int64, 1, 0)[0]) == moved
    at = 8
    for s in range(S):
        rec = np.frombuffer(raw, np.int64, 3, at)
        at += 24
        nt = np.frombuffer(raw, np.int64, 6, at)
        at += 48
        mt = np.frombuffer(raw, np.float32, 6, at)
        at += 24
        ids = np.frombuffer(raw, np.int64, int(rec[2]), at)
        at += 8 * int(rec[2])
        assert ids.tolist() == lists[s], s
        assert (int(rec[0]), int(rec[1])) == (int(nb[s]), int(tracer[s])), s
        assert np.array_equal(nt, ntype[s]) and np.array_equal(mt, mtype[s]), s
    assert at == len(raw)
