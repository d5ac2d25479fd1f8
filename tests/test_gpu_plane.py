"""The 3D xy-plane pass (cupss_gb300/csrc/plane.cuh) against the form it replaces.

A 3D phase whose products are one channel's power (Cahn-Hilliard's phi^3) computes
them with one kernel per step: y-inverse, x inverse real FFT, power, x forward real FFT
and y forward FFT of each z plane, with the plane in the shared memory of a thread-block
cluster.  The same step with CUPSSGB_PLANE=0 runs the row pass and two y line passes
instead.  Both apply the same FFT decompositions to the same values, so the fields
agree to rounding; the tests also check that the plane kernel is the one that ran, on
every instantiated plane shape (one CTA per plane up to 128^2, a two-CTA cluster at
256^2), with conserved noise, over batches, and against the FP64 oracle.
"""
import ctypes as C
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EQ = "dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3"
PARAMS = {"a": -1.0, "b": 1.0, "k": 1.0, "T": 0.01}


@pytest.fixture(autouse=True)
def _in_tmp(tmp_path, monkeypatch, built_lib):
    monkeypatch.chdir(tmp_path)


def make(shape, init, seed=7):
    import cupss_gb300 as c
    e = c.Evolver(True, *shape, dt=0.005, write_every=10 ** 9)
    e.createField("phi", True)
    for k, v in PARAMS.items():
        e.addParameter(k, v)
    e.addEquation(EQ)
    e.addNoise("phi", "2*T*q^2")
    e.setNoiseSeed(seed)
    e.setReal("phi", init)
    e.prepareProblem()
    return e


def kernels_run(e, steps):
    import cupss_gb300 as c
    lib = c.load()
    h = lib.cupssgb_evolver_solver(e.h)
    lib.cupssgb_solver_set_kernel_timing(h, 1)
    e.advanceTime(steps)
    buf = C.create_string_buffer(4096)
    lib.cupssgb_solver_kernel_report(h, buf, len(buf))
    lib.cupssgb_solver_set_kernel_timing(h, 0)
    return json.loads(buf.value.decode())


@pytest.mark.parametrize("shape", [(16, 16, 8), (32, 32, 32), (64, 64, 16), (128, 128, 8), (256, 256, 4)])
def test_plane_pass_equals_row_pass_form(shape, monkeypatch):
    sx, sy, sz = shape
    init = np.random.default_rng(sx + sz).uniform(-0.05, 0.05, sx * sy * sz).astype(np.float32)
    monkeypatch.setenv("CUPSSGB_PLANE", "1")
    a = make(shape, init)
    ka = kernels_run(a, 3)
    a.advanceTime(37)
    got = a.getReal("phi")
    a.close()
    monkeypatch.setenv("CUPSSGB_PLANE", "0")
    b = make(shape, init)
    kb = kernels_run(b, 3)
    b.advanceTime(37)
    want = b.getReal("phi")
    b.close()
    assert "plane_pass" in ka and "row_pass" not in ka and "line_inv_y" not in ka, ka
    assert "plane_pass" not in kb and "row_pass" in kb, kb
    err = float(np.linalg.norm(got.astype(np.float64) - want) / np.linalg.norm(want))
    print(shape, "plane vs row-pass form, 40 steps: rel L2 %.2e" % err)
    assert err < 1e-6


def test_plane_pass_in_a_batch_equals_single_solves(monkeypatch):
    import cupss_gb300 as c
    monkeypatch.setenv("CUPSSGB_PLANE", "1")
    from cupss_gb300.workloads import SYSTEMS, declare
    shape = (32, 32, 32)
    ens = c.Ensemble()
    declare(ens, SYSTEMS["ch"])
    seeds = [11, 12, 13]
    for s in seeds:
        ens.addMember(*shape, dt=0.005, seed=s)
    ens.prepare()
    rng = np.random.default_rng(3)
    inits = [rng.uniform(-0.05, 0.05, 32 ** 3).astype(np.float32) for _ in seeds]
    for i, arr in enumerate(inits):
        ens.setReal(i, "phi", arr)
    ens.advance(25)
    outs = [ens.getReal(i, "phi") for i in range(len(seeds))]
    ens.close()
    for i, s in enumerate(seeds):
        e = c.Evolver(True, *shape, dt=0.005, write_every=10 ** 9)
        sd = SYSTEMS["ch"]
        for nm, dyn in sd["fields"]:
            e.createField(nm, dyn)
        for k, v in sd["params"].items():
            e.addParameter(k, v)
        for q in sd["eqs"]:
            e.addEquation(q)
        for f, a in sd["noise"]:
            e.addNoise(f, a)
        e.setNoiseSeed(s)
        e.setReal("phi", inits[i])
        e.prepareProblem()
        e.advanceTime(25)
        ref = e.getReal("phi")
        e.close()
        got = outs[i].reshape(ref.shape).astype(np.float64)
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-6, "member %d" % i
