"""Grids with axes of 3 * 2^a points (96, 192, ...) against the FP64 oracle.

The reference plans cuFFT for any size (src/field_init.cpp:70,119 of cuPSS); this
library's FFTs take lengths 2^a and 3 * 2^a (radix-3 butterflies in the register DFTs,
cupss_gb300/csrc/fft.cuh): x up to 384 points, y and z up to 192.  The cases cover the
row pass (packed x rows of 3 * 2^a complex values), the y and z line passes, the paired
z-line turnaround of 3D grids, multi-field phases (model H, KPZ), noise, batches mixing
such grids with powers of two, and the reference-layout Fourier readout.
"""
import numpy as np
import pytest

from test_gpu_parity import init_field, rel_l2, run_case

pytestmark = pytest.mark.gpu

CH_NOISE = ([("phi", 1)], {"a": -1.0, "b": 1.0, "k": 1.0, "T": 0.01},
            ["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3"], [("phi", "2*T*q^2")])


@pytest.fixture(autouse=True)
def _in_tmp(tmp_path, monkeypatch, built_lib):
    monkeypatch.chdir(tmp_path)


@pytest.mark.parametrize("shape", [(96, 96, 96), (96, 64, 48), (48, 192, 24), (12, 6, 6), (384, 12, 6)])
def test_cahn_hilliard_3d_noise(shape):
    r, e, _ = run_case(CH_NOISE, shape, 0.005, 30, {"phi": init_field(shape, -0.05, 0.05)}, seed=17)
    err = rel_l2(e.getReal("phi"), r.real_field("phi"))
    print(shape, "3D CH + noise, 30 steps: rel L2 %.2e" % err)
    assert err < 2e-5


@pytest.mark.parametrize("shape", [(192, 96, 1), (384, 192, 1), (96, 128, 1), (6, 1, 1), (192, 1, 1)])
def test_cahn_hilliard_2d_and_1d(shape):
    spec = ([("phi", 1)], {"a": -1.0, "b": 1.0, "k": 1.0}, ["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3"], [])
    r, e, _ = run_case(spec, shape, 0.01, 100, {"phi": init_field(shape)})
    err = rel_l2(e.getReal("phi"), r.real_field("phi"))
    print(shape, "CH, 100 steps: rel L2 %.2e" % err)
    assert err < 2e-5
    F = e.getFourier("phi")
    assert rel_l2(F, np.fft.fftn(r.real_field("phi"))) < 2e-5


def test_model_h_on_a_96_by_192_grid():
    shape = (96, 192, 1)
    spec = ([("phi", 1), ("iqxphi", 0), ("iqyphi", 0), ("lapphi", 0), ("vx", 0), ("vy", 0)],
            {"a": -1.0, "b": 1.0, "k": 4.0, "eta": 1.0, "T": 0.001},
            ["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3 - vx*iqxphi - vy*iqyphi",
             "iqxphi = iqx*phi", "iqyphi = iqy*phi", "lapphi = -q^2*phi",
             "vx*eta*q^2 = -k*iqxphi*lapphi - k*iqx^2*1/q^2*iqxphi*lapphi - k*iqx*iqy*1/q^2*iqyphi*lapphi",
             "vy*eta*q^2 = -k*iqyphi*lapphi - k*iqy^2*1/q^2*iqyphi*lapphi - k*iqx*iqy*1/q^2*iqxphi*lapphi"],
            [("phi", "2*T")])
    r, e, names = run_case(spec, shape, 0.01, 40, {"phi": init_field(shape, -0.5, 0.5)}, seed=11)
    for n in names:
        err = rel_l2(e.getReal(n), r.real_field(n))
        assert err < 5e-5, (n, err)


def test_kpz_192():
    shape = (192, 192, 1)
    spec = ([("h", 1), ("iqxh", 0), ("iqyh", 0)], {"nu": 1.3, "lambda": 2.0, "D": 1.0},
            ["dt h + nu*q^2*h = 0.5*lambda*iqxh^2 + 0.5*lambda*iqyh^2", "iqxh = iqx*h", "iqyh = iqy*h"],
            [("h", "2*D")])
    r, e, names = run_case(spec, shape, 0.005, 60, {"h": init_field(shape, -0.2, 0.2)}, seed=3)
    for n in names:
        err = rel_l2(e.getReal(n), r.real_field(n))
        assert err < 3e-5, (n, err)


def test_ensemble_mixing_96_and_64():
    import cupss_gb300 as c
    from cupss_gb300.workloads import SYSTEMS, declare
    sizes = [(96, 96, 1), (64, 64, 1), (96, 96, 1), (48, 48, 48)]
    ens = c.Ensemble()
    declare(ens, SYSTEMS["ch"])
    for i, s in enumerate(sizes):
        ens.addMember(*s, dt=0.005, seed=100 + i)
    ens.prepare()
    inits = [init_field(s, -0.05, 0.05) for s in sizes]
    for i, a in enumerate(inits):
        ens.setReal(i, "phi", a)
    ens.advance(20)
    outs = [ens.getReal(i, "phi") for i in range(len(sizes))]
    ens.close()
    sd = SYSTEMS["ch"]
    for i, s in enumerate(sizes):
        e = c.Evolver(True, *s, dt=0.005, write_every=10 ** 9)
        declare(e, sd)
        e.setNoiseSeed(100 + i)
        e.setReal("phi", inits[i])
        e.prepareProblem()
        e.advanceTime(20)
        ref = e.getReal("phi")
        e.close()
        assert rel_l2(outs[i].reshape(ref.shape), ref) < 1e-6, s
