"""Build recipe for the oracle (TEST INFRASTRUCTURE, not product code).

Builds:
  oracle/build/liboracle.so    the project's own CPU restatement of the
                               reference unbinding (oracle/unbind_port.cpp);
                               built everywhere, also the CPU baseline.
  oracle/_ref/libref_dmo.so    the reference's own Subhalo_t::Unbind compiled
  oracle/_ref/libref_hydro.so  from its sources where they lie (read-only
                               reference tree) against oracle/stub/*.h, with
                               oracle/ref_driver.cpp as the batch driver.
                               Built only when the reference tree is present.

Both use -ffp-contract=off so that float/double rounding is the same on x86
and Arm and between the two builds.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
REF_ROOT = os.environ.get("HBTG_REFERENCE_ROOT", "/root/reference")
REF_SOURCES = ["subhalo_unbind", "gravity_tree", "config_parser", "mymath", "mpi_wrapper",
               "subhalo", "subhalo_merge", "snapshot", "geometric_tree"]
COMMON = ["-std=c++14", "-O3", "-fopenmp", "-fPIC", "-ffp-contract=off", "-DHBT_INT8", "-DINPUT_INT8"]
VARIANTS = {
    "dmo": ["-DDM_ONLY", "-DMEASURE_UNBINDING_TIME"],
    "hydro": ["-DUNBIND_WITH_THERMAL_ENERGY", "-DMEASURE_UNBINDING_TIME"],
}


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps if os.path.exists(d))


def build_port(force=False):
    out_dir = os.path.join(HERE, "build")
    os.makedirs(out_dir, exist_ok=True)
    src = os.path.join(HERE, "unbind_port.cpp")
    out = os.path.join(out_dir, "liboracle.so")
    deps = [src, os.path.join(REPO, "include", "hbt_unbind_gpu.h")]
    if not force and _newer(out, deps):
        return out
    _run(["g++", *COMMON, "-shared", "-I", os.path.join(REPO, "include"), src, "-o", out])
    return out


def reference_available():
    return os.path.isfile(os.path.join(REF_ROOT, "src", "subhalo_unbind.cpp"))


def build_reference(force=False):
    """Compile the reference unbinding sources in place into oracle/_ref/."""
    if not reference_available():
        return []
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    inc = ["-I", os.path.join(HERE, "stub"), "-I", os.path.join(REF_ROOT, "src"), "-I", REF_ROOT,
           "-I", os.path.join(REPO, "include")]
    driver = os.path.join(HERE, "ref_driver.cpp")
    jobs, outs = [], []
    for name, flags in VARIANTS.items():
        lib = os.path.join(out_dir, "libref_%s.so" % name)
        outs.append(lib)
        srcs = [os.path.join(REF_ROOT, "src", s + ".cpp") for s in REF_SOURCES] + [driver]
        if not force and _newer(lib, srcs + [os.path.join(HERE, "stub", "mpi.h")]):
            continue
        objs = []
        for s in srcs:
            obj = os.path.join(out_dir, "%s_%s.o" % (os.path.splitext(os.path.basename(s))[0], name))
            objs.append(obj)
            jobs.append(["g++", *COMMON, *flags, *inc, "-c", s, "-o", obj])
        outs[-1] = (lib, objs)
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(_run, jobs))
    result = []
    for item in outs:
        if isinstance(item, tuple):
            lib, objs = item
            _run(["g++", "-shared", "-fopenmp", *objs, "-o", lib])
            for o in objs:
                os.remove(o)
            result.append(lib)
        else:
            result.append(item)
    return result


def build_all(force=False):
    libs = [build_port(force)]
    libs += build_reference(force)
    return libs


if __name__ == "__main__":
    for lib in build_all(force="--force" in sys.argv):
        print(lib)
