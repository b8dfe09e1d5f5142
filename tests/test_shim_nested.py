"""The C++ host shim's recursive_unbind (SubhaloSnapshot_t::RefineParticles'
nested part: Subhalo_t::RecursiveUnbind with MergeRecursively,
src/subhalo_unbind.cpp:810-841, src/subhalo_merge.cpp:46-92), compiled into a
program that links libhbtg.so and run on the GPU, against the golden outputs
of the reference's own recursion on the same nesting forest (with
MergeTrappedSubhalos on and off)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "nested_merge.npz")


def _params(z):
    from hbtg import abi
    prm = abi.Params()
    for k, _ in abi.Params._fields_:
        setattr(prm, k, z["prm_" + k].item())
    return prm


def _write_input(path, z, merge_trapped, snapshot):
    prm = _params(z)
    S = len(z["parent"])
    frame = np.concatenate([np.asarray(z["frame_" + k], np.float32).ravel()
                            for k in ("ref_pos", "ref_vel", "mostbound_pos", "mostbound_vel")])
    with open(path, "wb") as f:
        f.write(bytes(prm))
        f.write(np.array([len(z["mass"]), S, merge_trapped, snapshot], np.int64).tobytes())
        for k, dt in (("pos", np.float32), ("vel", np.float32), ("mass", np.float32), ("id", np.int64),
                      ("member_off", np.int64), ("member_idx", np.int64), ("parent", np.int64)):
            f.write(np.ascontiguousarray(z[k], dt).tobytes())
        f.write(frame.tobytes())
        f.write(np.ascontiguousarray(z["frame_most_bound_id"], np.int64).tobytes())


def _read_output(path, S):
    raw = open(path, "rb").read()
    at, out = 0, []
    for _ in range(S):
        rec = np.frombuffer(raw, np.int64, 6, at)
        at += 48
        mb = float(np.frombuffer(raw, np.float32, 1, at)[0])
        at += 4
        ids = np.frombuffer(raw, np.int64, int(rec[5]), at).copy()
        at += 8 * int(rec[5])
        out.append(dict(nbound=int(rec[0]), most_bound_id=int(rec[1]), sink_track=int(rec[2]), snap_sink=int(rec[3]),
                        snap_death=int(rec[4]), mbound=mb, ids=ids))
    return out


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    from hbtg.build import LIB, build_library
    build_library()
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("shim") / "shim_nested_driver")
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-Wno-deprecated-declarations", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "hbt-herons_gb300", "host"), os.path.join(HERE, "shim_nested_driver.cpp"),
           "-o", exe, "-L", os.path.dirname(LIB), "-lhbtg", "-Wl,-rpath," + os.path.dirname(LIB)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return exe


@pytest.mark.gpu
@pytest.mark.parametrize("merge_trapped", [1, 0])
def test_shim_recursive_unbind_matches_reference(driver, tmp_path, merge_trapped):
    z = np.load(GOLDEN)
    S = len(z["parent"])
    snap = 9
    inp, outp = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    _write_input(inp, z, merge_trapped, snap)
    r = subprocess.run([driver, inp, outp], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-4000:]
    got = _read_output(outp, S)
    pre = "ref%d_" % merge_trapped
    ref_ids = [z[pre + "ids"][z[pre + "ids_off"][s]:z[pre + "ids_off"][s + 1]] for s in range(S)]
    # merger bookkeeping: identical
    for k in ("sink_track", "snap_sink", "snap_death"):
        assert [g[k] for g in got] == z[pre + k].tolist(), k
    if merge_trapped:
        assert any(g["sink_track"] >= 0 for g in got)  # the planted overlaps merged
    # bound sets and final sources: membership within the plain path's bar
    mism = tot = 0
    for s in range(S):
        nb_r = int(z[pre + "nbound"][s])
        a, b = set(got[s]["ids"][:got[s]["nbound"]].tolist()), set(ref_ids[s][:nb_r].tolist())
        mism += len(a ^ b)
        tot += len(b)
        assert set(got[s]["ids"].tolist()) == set(ref_ids[s].tolist()) or len(a ^ b) > 0, s
    assert mism <= max(1, 1e-4 * tot), (mism, tot)
    m_got = sum(g["mbound"] for g in got)
    m_ref = float(np.sum(z[pre + "mbound"].astype(np.float64)))
    assert abs(m_got - m_ref) <= 1e-5 * m_ref
