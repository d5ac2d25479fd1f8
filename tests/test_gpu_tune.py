"""The autotuner on the GPU: shapes timed at prepare, stored in the cache, read back.

The first solver of a system times the candidates (tile width, resident-warp target, the
FFT form of 1024-point lines, the 3D plane pass per cluster size or the row pass; all
but the width only from 2^20 grid points on) and writes the winners
to the cache file; a second solver of the same system reads them and times nothing.  The
launch shape changes which threads and CTAs do the arithmetic, not the arithmetic, so
the fields agree with those of an untuned solver (CUPSSGB_TUNE=0) to rounding, and a
hand-written cache entry that picks other shapes is honoured with the same fields.
"""
import ctypes as C
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EQ = "dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3"


@pytest.fixture(autouse=True)
def _env(tmp_path, monkeypatch, built_lib):
    monkeypatch.chdir(tmp_path)
    monkeypatch.setenv("CUPSSGB_TUNE_CACHE", str(tmp_path / "tune.txt"))
    monkeypatch.delenv("CUPSSGB_TUNE", raising=False)


def solve(shape, init, steps=30):
    import cupss_gb300 as c
    lib = c.load()
    e = c.Evolver(True, *shape, dt=0.005, write_every=10 ** 9)
    e.createField("phi", True)
    for k, v in {"a": -1.0, "b": 1.0, "k": 1.0, "T": 0.01}.items():
        e.addParameter(k, v)
    e.addEquation(EQ)
    e.addNoise("phi", "2*T*q^2")
    e.setNoiseSeed(5)
    e.setReal("phi", init)
    e.prepareProblem()
    h = lib.cupssgb_evolver_solver(e.h)
    buf = C.create_string_buffer(8192)
    lib.cupssgb_solver_tune_report(h, buf, len(buf))
    rep = json.loads(buf.value.decode())
    e.advanceTime(steps)
    out = e.getReal("phi").astype(np.float64)
    e.close()
    return rep, out


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("shape", [(1024, 1024, 1), (256, 256, 16)])
def test_cached_plan_gives_the_fields_of_an_untuned_one(shape, monkeypatch):
    sx, sy, sz = shape
    init = np.random.default_rng(1).uniform(-0.05, 0.05, sx * sy * sz).astype(np.float32)
    rep1, f1 = solve(shape, init)
    ph = rep1["phase1"]
    assert not ph["cached"] and ph["ms"], rep1
    names = set(ph["ms"])
    assert any(n.startswith("W=") for n in names) and any(n.startswith("warps=") for n in names)
    if sy >= 512:   # 1024-point lines: the split form is a candidate
        assert any(n.startswith("split=") for n in names)
    if sz > 1:
        # both 3D product forms were timed: the plane pass (per cluster size) and the row pass
        assert any(n.startswith("plane_c=") for n in names) and "plane=0" in names
    rep2, f2 = solve(shape, init)
    ph2 = rep2["phase1"]
    assert ph2["cached"] and not ph2["ms"], rep2
    for k in ("W", "warps", "split", "plane", "plane_c"):
        assert ph2[k] == ph[k]
    assert np.array_equal(f1, f2)
    monkeypatch.setenv("CUPSSGB_TUNE", "0")
    rep3, f3 = solve(shape, init)
    assert not rep3["phase1"]["ms"]
    err = rel(f1, f3)
    print(shape, "tuned", {k: ph[k] for k in ("W", "warps", "split", "plane", "plane_c")}, "ms", ph["ms"],
          "vs untuned: rel L2 %.2e" % err)
    assert err < 1e-6


def test_hand_written_entry_is_honoured(tmp_path):
    import cupss_gb300 as c
    shape = (256, 256, 16)
    init = np.random.default_rng(2).uniform(-0.05, 0.05, 256 * 256 * 16).astype(np.float32)
    rep1, f1 = solve(shape, init)
    lib = c.load()
    # rewrite the phase's entry with other shapes: narrowest width, 24 warps, the plane pass
    # on two CTAs per plane
    key = None
    with open(str(tmp_path / "tune.txt")) as fh:
        for line in fh:
            tag, k, v = line.rstrip("\n").split("\t")
            if "/p1/" in k:
                key = k
    assert key
    assert lib.cupssgb_tune_cache_store(key.encode(), b"W=2 warps=24 split=0 plane=1 plane_c=2 ms=1") == 0
    rep2, f2 = solve(shape, init)
    ph = rep2["phase1"]
    assert ph["cached"] and ph["W"] == 2 and ph["warps"] == 24 and ph["plane"] == 1 and ph["plane_c"] == 2, rep2
    assert rel(f2, f1) < 1e-6
