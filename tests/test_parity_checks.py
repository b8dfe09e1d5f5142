"""The full-output parity check (tests/parity.py) itself: the reference's own
outputs pass against themselves, and a mistake planted in a copy of them (on
the CPU) is caught field by field."""
import copy
import glob
import importlib.util
import os

import numpy as np
import pytest

from parity import compare_full

HERE = os.path.dirname(os.path.abspath(__file__))


def _load(name):
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "golden", "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.load(os.path.join(HERE, "golden", name + ".npz"))


def _fields(viol):
    return {v[0] for v in viol}


@pytest.mark.parametrize("path", sorted(p for p in glob.glob(os.path.join(HERE, "golden", "*.npz"))
                                         if not os.path.basename(p).startswith(("nested", "reassign"))),
                         ids=lambda p: os.path.basename(p)[:-4])
def test_reference_passes_against_itself(path):
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "golden", "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    inp, prm, ref = mod.load(path)
    m, viol = compare_full(inp, ref, ref, prm)
    assert not viol
    assert m["matched"] == inp.n_sub


def _big_sub(inp, ref, min_tail=40):
    for s in np.argsort(-np.diff(inp.offsets)):
        off, end = int(inp.offsets[s]), int(inp.offsets[s + 1])
        if ref.status[s] == 0 and end - off - ref.nbound[s] >= min_tail and ref.nbound[s] >= 100:
            return int(s), off, end
    raise AssertionError("no suitable subhalo")


def test_tail_order_mistake_is_caught():
    inp, prm, ref = _load("batched_200")
    s, off, end = _big_sub(inp, ref)
    bad = copy.deepcopy(ref)
    nb = int(ref.nbound[s])
    i, j = off + nb, end - 1  # first and last tail particles swap
    bad.order[i], bad.order[j] = ref.order[j], ref.order[i]
    _, viol = compare_full(inp, bad, ref, prm)
    assert "tail_order" in _fields(viol)


def test_bound_order_mistake_is_caught():
    inp, prm, ref = _load("nfw_10k")
    bad = copy.deepcopy(ref)
    off = int(inp.offsets[0])
    nb = int(ref.nbound[0])
    bad.order[off + 5], bad.order[off + nb - 5] = ref.order[off + nb - 5], ref.order[off + 5]
    _, viol = compare_full(inp, bad, ref, prm)
    assert "bound_order" in _fields(viol)


@pytest.mark.parametrize("field,index,scale", [
    ("core", 0, 1e-3),         # core position moved by 1e-3 of itself
    ("core", 7, 1e-3),         # sigma_v
    ("kinematics", 1, 1e-4),   # <K>
    ("ref_vel", 2, 1e-3),
    ("mbound", None, 1e-4),
])
def test_float_mistakes_are_caught(field, index, scale):
    inp, prm, ref = _load("batched_200")
    s, _, _ = _big_sub(inp, ref)
    bad = copy.deepcopy(ref)
    arr = getattr(bad, field)
    if index is None:
        arr[s] = arr[s] * (1 + scale)
    else:
        arr[s, index] = arr[s, index] * (1 + scale) + (scale if arr[s, index] == 0 else 0)
    _, viol = compare_full(inp, bad, ref, prm)
    assert field in _fields(viol)


def test_tracer_and_type_mistakes_are_caught():
    inp, prm, ref = _load("small_hydro")
    s = int(np.argmax(ref.nbound))
    bad = copy.deepcopy(ref)
    bad.tracer_index[s] += 1
    bad.nbound_type[s, 0] += 1
    _, viol = compare_full(inp, bad, ref, prm)
    assert {"tracer_index", "nbound_type"} <= _fields(viol)


def test_energy_outliers_are_caught():
    inp, prm, ref = _load("nfw_10k")
    bad = copy.deepcopy(ref)
    off = int(inp.offsets[0])
    nb = int(ref.nbound[0])
    k = np.arange(off, off + nb, 50)  # 2 % of the bound particles
    bad.potential[k] *= 1 + 1e-3
    _, viol = compare_full(inp, bad, ref, prm)
    assert "energy/potential" in _fields(viol)
