"""Pins the CPU oracle to the reference's own known-answer fixtures.

tests/golden/reference_base_truths.npz holds the reference's base_truths
(tests/tests.cpp:64-422 of cuPSS): droplet initial conditions on 16, 16^2, 16^3
grids and the one-step lap / iqx / iqy / iqz / 1/q operators in 1D and 3D from
both the reference CPU (FFTW) and GPU (cuFFT) paths.  The reference tests use
EXPECT_NEAR(..., 1e-4); the oracle must meet the same bound (it does to ~2e-6).
"""
import os

import numpy as np
import pytest

from oracle.ref_parser import System
from oracle.ref_solver import RefSolver, droplet

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_base_truths.npz"))
TOL = 1e-4


@pytest.mark.parametrize("dim,shape", [(1, (16, 1, 1)), (2, (16, 16, 1)), (3, (16, 16, 16))])
def test_droplet_init(dim, shape):
    ph = droplet(shape, 0, 1, 16 / 8, 4, 8, 8 if dim > 1 else 0, 0)
    assert np.abs(ph.ravel() - GOLD["phi_%dd" % dim]).max() < TOL


def operator_system(dim, dev):
    s = System()
    sfx = "_%s_%dd" % (dev, dim)
    names = ["phi", "lapphi", "iqxphi"] + (["iqyphi", "iqzphi"] if dim == 3 else []) + ["invqphi"]
    for n in names:
        s.create_field(n + sfx, n == "phi")
    s.add_equation("dt phi%s+q^2*phi%s = iqxphi%s^2" % (sfx, sfx, sfx))
    s.add_equation("lapphi%s = -q^2*phi%s" % (sfx, sfx))
    s.add_equation("iqxphi%s =  iqx*phi%s" % (sfx, sfx))
    if dim == 3:
        s.add_equation("iqyphi%s =  iqy*phi%s" % (sfx, sfx))
        s.add_equation("iqzphi%s =  iqz*phi%s" % (sfx, sfx))
    s.add_equation("invqphi%s =  1/q*phi%s" % (sfx, sfx))
    return s, sfx, names


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("dev", ["cpu", "gpu"])
@pytest.mark.parametrize("dim", [1, 3])
def test_one_step_operators(dim, dev, precision):
    s, sfx, names = operator_system(dim, dev)
    shape = (16, 1, 1) if dim == 1 else (16, 16, 16)
    r = RefSolver(s, *shape, dt=1.0, precision=precision)
    r.set_real("phi" + sfx, droplet(shape, 0, 1, 2, 4, 8, 8 if dim == 3 else 0, 0))
    r.prepare()
    r.advance(1)
    checked = 0
    for n in names[1:]:
        key = n + sfx
        if key in GOLD.files:
            err = np.abs(r.real_field(key).ravel() - GOLD[key]).max()
            assert err < TOL, (key, err)
            checked += 1
    assert checked == len(names) - 1


def test_oracle_noise_is_hermitian_white():
    from oracle.philox import fourier_noise
    xi = fourier_noise(16, 8, 4, seed=7, step=3, field_id=1)
    real = np.fft.ifftn(xi)            # xi = FFT(w) with w white N(0,1)
    assert np.abs(real.imag).max() < 1e-12
    assert abs(np.var(real.real) - 1.0) < 0.2


def test_philox_known_answer():
    """Philox4x32-10 known-answer vectors of the Random123 distribution (kat_vectors)."""
    from oracle.philox import philox4x32_10
    out = philox4x32_10(0, 0, 0, 0, 0, 0)
    assert [int(v) for v in out] == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    out = philox4x32_10(0xffffffff, 0xffffffff, 0xffffffff, 0xffffffff, 0xffffffff, 0xffffffff)
    assert [int(v) for v in out] == [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    out = philox4x32_10(0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344, 0xa4093822, 0x299f31d0)
    assert [int(v) for v in out] == [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]


@pytest.mark.parametrize("shape", [(16, 1, 1), (2, 1, 1), (8, 8, 1), (1024, 2, 1), (4, 4, 4), (16, 8, 4),
                                   (64, 32, 16)])
def test_noise_c_restatement_equals_numpy(shape):
    # oracle/noise.c (the fast path the tests use) against the numpy definition
    from oracle import philox
    assert philox._c_lib() is not None, "oracle/noise.c did not build"
    a = philox.fourier_noise(*shape, 0x0123456789ABCDEF, 11, 2)
    b = philox.fourier_noise_numpy(*shape, 0x0123456789ABCDEF, 11, 2)
    assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max()
