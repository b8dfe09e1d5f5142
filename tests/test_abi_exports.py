"""The C-ABI library builds, loads without a GPU and exports every function
that include/*.h declares (no compute calls: this runs on CPU)."""
import ctypes
import glob
import os
import re

from conftest import ROOT


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)  # drop comments
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(hbtg_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_the_entry_points():
    names = declared_functions()
    for required in ("hbtg_create", "hbtg_unbind_batch", "hbtg_unbind_batch_device", "hbtg_unbind_batch_noalloc",
                     "hbtg_unbind_batch_learned", "hbtg_mlp_forward", "hbtg_mlp_backward", "hbtg_adam_step"):
        assert required in names, required


def test_library_exports_every_declared_symbol():
    from hbtg.build import build_library
    lib = ctypes.CDLL(build_library())
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    lib.hbtg_status_string.restype = ctypes.c_char_p  # a pure host entry point needs no device
    assert lib.hbtg_status_string(0) == b"ok"


def test_launch_setting_entry_points_reject_bad_arguments_without_a_device():
    """hbtg_get_tuning / hbtg_set_tuning / hbtg_autotune check their arguments
    before any CUDA call: a null handle is HBTG_ERR_INVALID (1)."""
    from hbtg.abi import CTuning
    from hbtg.build import build_library
    lib = ctypes.CDLL(build_library())
    t = CTuning(8192, 0, 8, 0.0)
    lib.hbtg_get_tuning.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.hbtg_set_tuning.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.hbtg_autotune.argtypes = [ctypes.c_void_p] * 5 + [ctypes.c_int, ctypes.c_void_p]
    assert lib.hbtg_get_tuning(None, ctypes.byref(t)) == 1
    assert lib.hbtg_set_tuning(None, ctypes.byref(t)) == 1
    assert lib.hbtg_autotune(None, None, None, None, None, 0, None) == 1
