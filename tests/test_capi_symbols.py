"""The C-ABI library loads and exports every entry point include/cupss_gb300.h
declares (no compute calls: runs without a GPU)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "cupss_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(cupssgb_[a-z0-9_]+)\s*\(", src)))


def test_every_declared_symbol_is_exported(built_lib):
    from cupss_gb300 import capi
    lib = ctypes.CDLL(capi.LIB_PATH)
    names = declared_symbols()
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # the Python binding types every declared symbol
    assert set(names) <= set(capi.SIGNATURES), set(names) - set(capi.SIGNATURES)


def test_error_path_without_gpu(built_lib):
    from cupss_gb300 import capi
    lib = capi.load()
    h = ctypes.c_void_p()
    # unsupported grid size is rejected on the host, with a message
    rc = lib.cupssgb_solver_create(10, 1, 1, 1.0, 1.0, 1.0, 0.1, ctypes.byref(h))
    assert rc == capi.ERR_UNSUPPORTED
    assert b"3*2^a" in lib.cupssgb_last_error()
    assert lib.cupssgb_solver_add_field(None, 1) == capi.ERR_INVALID
