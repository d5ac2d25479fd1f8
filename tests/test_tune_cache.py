"""The autotuner's cache file (cupss_gb300/csrc/tune_cache.cpp), without a GPU.

prepare stores the winning launch shapes per phase under a key naming the GPU, grid,
batch span and update program; later solvers with that key read them instead of timing.
Here the file format through the C-ABI: where the file lives, appending entries, the last
entry of a key winning, lines of other formats ignored, and the cache switched off.
The GPU side (a cached plan gives the fields of an untuned one) is in
tests/test_gpu_tune.py.
"""
import ctypes as C
import os

import pytest


@pytest.fixture()
def lib(built_lib, tmp_path, monkeypatch):
    monkeypatch.setenv("CUPSSGB_TUNE_CACHE", str(tmp_path / "sub" / "tune.txt"))
    return built_lib


def path_of(lib):
    buf = C.create_string_buffer(4096)
    lib.cupssgb_tune_cache_path(buf, len(buf))
    return buf.value.decode()


def lookup(lib, key):
    buf = C.create_string_buffer(4096)
    n = lib.cupssgb_tune_cache_lookup(key.encode(), buf, len(buf))
    return None if n < 0 else buf.value.decode()


def test_store_and_lookup(lib, tmp_path):
    assert path_of(lib) == str(tmp_path / "sub" / "tune.txt")
    assert lookup(lib, "k1") is None
    assert lib.cupssgb_tune_cache_store(b"k1", b"W=8 warps=16 split=0 plane_c=4 ms=0.05") == 0
    assert lib.cupssgb_tune_cache_store(b"k2", b"W=4 warps=24 split=1 plane_c=0 ms=0.01") == 0
    assert lookup(lib, "k1") == "W=8 warps=16 split=0 plane_c=4 ms=0.05"
    # a later entry for the same key replaces the earlier one
    assert lib.cupssgb_tune_cache_store(b"k1", b"W=2 warps=16 split=0 plane_c=2 ms=0.04") == 0
    assert lookup(lib, "k1") == "W=2 warps=16 split=0 plane_c=2 ms=0.04"
    assert lookup(lib, "k2") == "W=4 warps=24 split=1 plane_c=0 ms=0.01"
    with open(path_of(lib)) as fh:
        lines = fh.read().splitlines()
    assert len(lines) == 3
    assert all(l.split("\t")[0] == "cupssgb-tune-v1" and len(l.split("\t")) == 3 for l in lines)


def test_foreign_and_broken_lines_are_ignored(lib):
    p = path_of(lib)
    os.makedirs(os.path.dirname(p), exist_ok=True)
    with open(p, "w") as fh:
        fh.write("garbage without tabs\n")
        fh.write("cupssgb-tune-v0\tk\tW=1\n")          # another format version
        fh.write("cupssgb-tune-v1\tk\n")               # no value field
        fh.write("cupssgb-tune-v1\tk\tW=16 warps=16 split=0 plane_c=0 ms=1\n")
    assert lookup(lib, "k") == "W=16 warps=16 split=0 plane_c=0 ms=1"
    # keys and values with tabs or newlines are refused
    assert lib.cupssgb_tune_cache_store(b"a\tb", b"W=1") < 0
    assert lib.cupssgb_tune_cache_store(b"a", b"W=1\n") < 0


def test_cache_off(built_lib, monkeypatch):
    monkeypatch.setenv("CUPSSGB_TUNE_CACHE", "off")
    assert path_of(built_lib) == ""
    assert built_lib.cupssgb_tune_cache_store(b"k", b"W=1") < 0
    assert lookup(built_lib, "k") is None


def test_default_location(built_lib, monkeypatch, tmp_path):
    monkeypatch.delenv("CUPSSGB_TUNE_CACHE", raising=False)
    monkeypatch.setenv("XDG_CACHE_HOME", str(tmp_path / "xdg"))
    assert path_of(built_lib) == str(tmp_path / "xdg" / "cupss_gb300" / "tune_v1.txt")
    monkeypatch.delenv("XDG_CACHE_HOME")
    monkeypatch.setenv("HOME", str(tmp_path / "home"))
    assert path_of(built_lib) == str(tmp_path / "home" / ".cache" / "cupss_gb300" / "tune_v1.txt")
