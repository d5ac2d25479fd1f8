"""Batches and ensembles against single solves.

A batch member must follow the trajectory a single solver (the drop-in evolver path)
gives for the same system values, seed and initial field: the member's noise counter
is its own step count and its values come from its own row of the value table, so
the arithmetic is the same.  Tolerance: relative L2 1e-6 (the kernels are the same
code; only the source of the prefactor values differs).  One member is also checked
against the FP64 oracle directly.
"""
import numpy as np
import pytest

from cupss_gb300.workloads import splitmix64_uniform

pytestmark = pytest.mark.gpu

KPZ = dict(
    fields=[("h", True), ("iqxh", False), ("iqyh", False)],
    params={"nu": 1.0, "lam": 1.0, "D": 1.0},
    eqs=["dt h + nu*q^2*h = 0.5*lam*iqxh^2 + 0.5*lam*iqyh^2", "iqxh = iqx*h", "iqyh = iqy*h"],
    noise=[("h", "2*D")],
)
CH = dict(
    fields=[("phi", True)],
    params={"a": -1.0, "b": 1.0, "k": 1.0, "T": 0.01},
    eqs=["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3"],
    noise=[("phi", "2*T*q^2")],
)


def rel(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


@pytest.fixture(autouse=True)
def _in_tmp(tmp_path, monkeypatch, built_lib):
    monkeypatch.chdir(tmp_path)


def plain(system, shape, dt, values, seed, inits, nsteps):
    import cupss_gb300 as c
    sx, sy, sz = shape
    e = c.Evolver(True, sx, sy, sz, dt=dt, write_every=10 ** 9)
    for nm, dyn in system["fields"]:
        e.createField(nm, dyn)
    for k, v in system["params"].items():
        e.addParameter(k, values.get(k, v))
    for q in system["eqs"]:
        e.addEquation(q)
    for f, a in system["noise"]:
        e.addNoise(f, a)
    e.setNoiseSeed(seed)
    for nm, arr in inits.items():
        e.setReal(nm, arr)
    e.prepareProblem()
    e.advanceTime(nsteps)
    out = {nm: e.getReal(nm) for nm, _ in system["fields"]}
    e.close()
    return out


def make_ensemble(system):
    import cupss_gb300 as c
    e = c.Ensemble()
    for nm, dyn in system["fields"]:
        e.createField(nm, dyn)
    for k, v in system["params"].items():
        e.addParameter(k, v)
    for q in system["eqs"]:
        e.addEquation(q)
    for f, a in system["noise"]:
        e.addNoise(f, a)
    return e


def members_spec(n, shapes, rng_seed):
    rng = np.random.default_rng(rng_seed)
    out = []
    for i in range(n):
        shape = shapes[i % len(shapes)]
        vals = {"nu": float(rng.uniform(0.5, 2.0)), "lam": float(rng.uniform(0.0, 4.0))}
        init = splitmix64_uniform(int(np.prod(shape)), 100 + i, -0.5, 0.5).reshape(shape[::-1])
        out.append((shape, vals, 1000 + 7 * i, init))
    return out


@pytest.mark.parametrize("nsteps", [5, 37])
def test_ensemble_members_match_single_solves(nsteps):
    """Mixed sizes in one ensemble; 37 steps = two 16-step graph replays + 5 eager."""
    spec = members_spec(6, [(64, 64, 1), (128, 64, 1), (32, 32, 1)], 1)
    e = make_ensemble(KPZ)
    for shape, vals, seed, _ in spec:
        e.addMember(*shape, dt=0.005, seed=seed, **vals)
    e.prepare()
    assert e.groups == 3
    for m, (_, _, _, init) in enumerate(spec):
        e.setReal(m, "h", init)
    e.advance(nsteps)
    for m, (shape, vals, seed, init) in enumerate(spec):
        ref = plain(KPZ, shape, 0.005, vals, seed, {"h": init}, nsteps)
        for nm in ("h", "iqxh", "iqyh"):
            err = rel(e.getReal(m, nm), ref[nm])
            assert err < 1e-6, (m, nm, err)
    d = e.describe()
    assert len(d["groups"]) == 3 and all(g["tune"] for g in d["groups"])
    # three 2D grid sizes of one system: stepped by the fused launches
    assert d["fused"] is not None, d


def test_ensemble_3d_noisy_matches_single_solves():
    spec = [((16, 16, 16), {}, 11), ((16, 16, 16), {"T": 0.05, "k": 2.0}, 12), ((32, 16, 8), {"a": -0.5}, 13)]
    e = make_ensemble(CH)
    inits = []
    for i, (shape, vals, seed) in enumerate(spec):
        e.addMember(*shape, dt=0.01, seed=seed, **vals)
        inits.append(splitmix64_uniform(int(np.prod(shape)), 40 + i, -0.3, 0.3).reshape(shape[::-1]))
    e.prepare()
    for m, init in enumerate(inits):
        e.setReal(m, "phi", init)
    e.advance(20)
    for m, (shape, vals, seed) in enumerate(spec):
        ref = plain(CH, shape, 0.01, vals, seed, {"phi": inits[m]}, 20)
        err = rel(e.getReal(m, "phi"), ref["phi"])
        assert err < 1e-6, (m, err)


def test_ensemble_member_against_oracle():
    from oracle.philox import NoiseProvider
    from oracle.ref_parser import System
    from oracle.ref_solver import RefSolver
    shape, vals, seed = (64, 32, 1), {"nu": 1.3, "lam": 2.5}, 77
    init = splitmix64_uniform(64 * 32, 5, -0.5, 0.5).reshape(1, 32, 64)
    e = make_ensemble(KPZ)
    e.addMember(32, 32, 1, dt=0.005, seed=1, nu=0.7)      # another group
    m = e.addMember(*shape, dt=0.005, seed=seed, **vals)
    e.addMember(*shape, dt=0.005, seed=seed + 1, nu=1.9)   # same group, other values
    e.prepare()
    e.setReal(m, "h", init)
    e.advance(40)
    s = System()
    for nm, dyn in KPZ["fields"]:
        s.create_field(nm, dyn)
    for k, v in KPZ["params"].items():
        s.add_parameter(k, vals.get(k, v))
    for q in KPZ["eqs"]:
        s.add_equation(q)
    s.add_noise("h", "2*D")
    r = RefSolver(s, *shape, dt=0.005, noise=NoiseProvider(*shape, seed))
    r.set_real("h", init)
    r.prepare()
    r.advance(40)
    assert rel(e.getReal(m, "h"), r.real_field("h")) < 3e-5


def test_batch_solver_inactive_and_reset():
    """Inactive members are untouched and count no steps; reset gives a fresh solve."""
    import cupss_gb300 as c
    from cupss_gb300.capi import Pres
    s = c.Solver(32, 32, 1, dt=0.01)
    f = s.add_field(True)
    s.set_implicit(f, [Pres(-1.0, 1, 0, 0, 0, 0)])
    s.set_noise(f, Pres(0.02, 0, 0, 0, 0, 0))
    s.set_members(3)
    s.prepare()
    init = splitmix64_uniform(32 * 32, 9, -1, 1).reshape(1, 32, 32)
    for m in range(3):
        s.set_real_member(f, m, init)
    s.set_member_active(1, False)
    before = s.get_real_member(f, 1)   # the state's round trip (FFT rounding), not init
    s.advance(20)
    assert [s.member_step(m) for m in range(3)] == [20, 0, 20]
    assert np.array_equal(s.get_real_member(f, 1), before)
    assert rel(s.get_real_member(f, 0), init) > 1e-3
    # members 0 and 2 have different default seeds, so different noise
    assert rel(s.get_real_member(f, 0), s.get_real_member(f, 2)) > 1e-4
    s.set_member_active(1, True)
    s.reset_member(0)
    assert s.member_step(0) == 0
    assert np.abs(s.get_real_member(f, 0)).max() == 0.0
    s.set_real_member(f, 0, init)
    s.advance(20)
    # member 0 after the reset == a single solve with member 0's (default) seed
    s2 = c.Solver(32, 32, 1, dt=0.01)
    g = s2.add_field(True)
    s2.set_implicit(g, [Pres(-1.0, 1, 0, 0, 0, 0)])
    s2.set_noise(g, Pres(0.02, 0, 0, 0, 0, 0))
    s2.prepare()
    s2.set_real(g, init)
    s2.advance(20)
    assert rel(s.get_real_member(f, 0), s2.get_real(g)) < 1e-6
    assert s.member_step(1) == 20 and s.member_step(2) == 40
    s.close()
    s2.close()


def test_batch_trailing_inactive_members_are_not_launched():
    """Launches cover members up to the last active one: deactivating the trailing
    members shrinks the launches (and their graphs), reactivating one regrows them, and
    every member's result stays that of its own solve."""
    import cupss_gb300 as c
    from cupss_gb300.capi import Pres

    def system(s):
        f = s.add_field(True)
        s.set_implicit(f, [Pres(-1.0, 1, 0, 0, 0, 0)])
        s.set_noise(f, Pres(0.02, 0, 0, 0, 0, 0))
        return f

    s = c.Solver(32, 16, 8, dt=0.01)
    f = system(s)
    s.set_members(4)
    for m in range(4):
        s.set_member_seed(m, 100 + m)
    s.prepare()
    init = splitmix64_uniform(32 * 16 * 8, 11, -1, 1).reshape(8, 16, 32)
    for m in range(4):
        s.set_real_member(f, m, init)
    s.set_member_active(2, False)
    s.set_member_active(3, False)
    held = [s.get_real_member(f, m) for m in (2, 3)]
    s.advance(32)   # two graph replays over members 0 and 1
    assert [s.member_step(m) for m in range(4)] == [32, 32, 0, 0]
    assert np.array_equal(s.get_real_member(f, 2), held[0])
    assert np.array_equal(s.get_real_member(f, 3), held[1])
    s.set_member_active(3, True)
    s.advance(16)
    assert [s.member_step(m) for m in range(4)] == [48, 48, 0, 16]
    assert np.array_equal(s.get_real_member(f, 2), held[0])

    def single(seed, nsteps):
        s2 = c.Solver(32, 16, 8, dt=0.01)
        g = system(s2)
        s2.set_seed(seed)
        s2.prepare()
        s2.set_real(g, init)
        s2.advance(nsteps)
        out = s2.get_real(g)
        s2.close()
        return out

    assert rel(s.get_real_member(f, 0), single(100, 48)) < 1e-6
    assert rel(s.get_real_member(f, 3), single(103, 16)) < 1e-6
    s.close()


def launches_per_step(sizes, per_size=2, steps=32):
    e = make_ensemble(KPZ)   # CUPSSGB_FUSE=1 set by the caller: the fused form, untimed
    k = 0
    for side in sizes:
        for _ in range(per_size):
            e.addMember(side, side, 1, dt=0.005, seed=500 + k)
            k += 1
    e.prepare()
    e.advance(16)   # the graphs are captured here
    l0 = e.launch_count
    e.advance(steps)
    n = (e.launch_count - l0) / steps
    d = e.describe()
    e.close()
    return n, d


def test_fused_launches_do_not_grow_with_the_number_of_grid_sizes(monkeypatch):
    # KPZ: phase 0 (iqxh, iqyh) is one turnaround, phase 1 a row pass and a turnaround,
    # and one step-count update per 16-step graph -- for one grid size (the solver's own
    # graphs) as for four (the fused launches)
    monkeypatch.setenv("CUPSSGB_FUSE", "1")
    n1, d1 = launches_per_step([128])
    n2, d2 = launches_per_step([64, 256])
    n4, d4 = launches_per_step([64, 128, 256, 512])
    assert d1["fused"] is None and d2["fused"] is not None and d4["fused"] is not None, (d1, d2, d4)
    assert len(d4["fused"]["classes"]) == 4 and d4["fused"]["form"] == "fused"
    assert d4["fused"]["launches_per_step"] == 3
    assert n4 == n2 == 3 + 1 / 16, (n2, n4)
    assert n4 <= n1, (n1, n4)


def test_fused_off_by_environment(monkeypatch):
    monkeypatch.setenv("CUPSSGB_FUSE", "0")
    n4, d4 = launches_per_step([64, 128, 256, 512], steps=16)
    assert d4["fused"] is None and d4["why_not_fused"] == "CUPSSGB_FUSE=0"
    assert n4 > 4 * 3


@pytest.mark.parametrize("fuse", ["1", None])
def test_fused_four_sizes_match_single_solves(monkeypatch, tmp_path, fuse):
    """Forced fused form, and the timed choice (which steps both forms on the fresh
    buffers and restarts them): either way every member equals its single solve."""
    if fuse:
        monkeypatch.setenv("CUPSSGB_FUSE", fuse)
    else:
        monkeypatch.delenv("CUPSSGB_FUSE", raising=False)
        monkeypatch.setenv("CUPSSGB_TUNE_CACHE", str(tmp_path / "tune.txt"))   # timed, not cached
    sizes = [64, 128, 256, 512]
    e = make_ensemble(KPZ)
    spec = []
    for i, side in enumerate(sizes * 2):
        vals = {"nu": 0.5 + 0.2 * i, "lam": 0.3 * i}
        init = splitmix64_uniform(side * side, 70 + i, -0.2, 0.2).reshape(side, side)
        e.addMember(side, side, 1, dt=0.005, seed=900 + i, **vals)
        spec.append(((side, side, 1), vals, 900 + i, init))
    e.prepare()
    f = e.describe()["fused"]
    assert f is not None
    if fuse is None:
        assert not f["cached"] and f["ms_per_step"]["fused"] > 0 and f["ms_per_step"]["grouped"] > 0
        assert f["form"] == ("fused" if f["ms_per_step"]["fused"] <= f["ms_per_step"]["grouped"] else "grouped")
        assert "multi1/" in (tmp_path / "tune.txt").read_text()
    for m, (_, _, _, init) in enumerate(spec):
        e.setReal(m, "h", init)
    e.advance(21)
    for m, (shape, vals, seed, init) in enumerate(spec):
        ref = plain(KPZ, shape, 0.005, vals, seed, {"h": init}, 21)
        for nm in ("h", "iqxh", "iqyh"):
            err = rel(e.getReal(m, nm), ref[nm])
            assert err < 1e-6, (m, shape, nm, err)


def test_fused_1d_and_radix3_grids_match_single_solves(monkeypatch):
    """The fused launches over 1D grids (one-point lines, most of a tile idle) and lengths
    3*2^a, forced (CUPSSGB_FUSE=1): every member equals its single solve."""
    monkeypatch.setenv("CUPSSGB_FUSE", "1")
    shapes = [(256, 1, 1), (96, 96, 1), (192, 96, 1), (64, 64, 1), (512, 1, 1)]
    e = make_ensemble(KPZ)
    spec = []
    for i, shape in enumerate(shapes):
        vals = {"nu": 0.8 + 0.1 * i, "lam": 0.5 + 0.2 * i}
        init = splitmix64_uniform(int(np.prod(shape)), 300 + i, -0.2, 0.2).reshape(shape[::-1])
        e.addMember(*shape, dt=0.005, seed=40 + i, **vals)
        spec.append((shape, vals, 40 + i, init))
    e.prepare()
    d = e.describe()
    assert d["fused"] is not None and d["fused"]["form"] == "fused", d
    for m, (_, _, _, init) in enumerate(spec):
        e.setReal(m, "h", init)
    e.advance(19)
    for m, (shape, vals, seed, init) in enumerate(spec):
        ref = plain(KPZ, shape, 0.005, vals, seed, {"h": init}, 19)
        for nm in ("h", "iqxh", "iqyh"):
            err = rel(e.getReal(m, nm), ref[nm])
            assert err < 1e-6, (m, shape, nm, err)
    e.close()
