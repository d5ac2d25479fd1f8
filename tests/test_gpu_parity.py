"""GPU parity: the CUDA engine, driven through the C-ABI, against the CPU oracle.

The oracle (oracle/ref_solver.py) restates the reference GPU path step by step
with full complex FFTs in float64; it is pinned to the reference's own goldens
(tests/test_oracle_golden.py).  Noise: the engine's Fourier-space Philox stream is
restated by oracle/philox.py and fed to the oracle, so noisy runs compare
realisation by realisation.

Tolerances (relative L2 over the whole field, FP32 engine vs FP64 oracle) are
stated per test; the reference goldens use the reference's absolute 1e-4.
"""
import os

import numpy as np
import pytest

from oracle.philox import NoiseProvider
from oracle.ref_parser import System
from oracle.ref_solver import RefSolver, droplet

pytestmark = pytest.mark.gpu

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_base_truths.npz"))


@pytest.fixture(autouse=True)
def _in_tmp(tmp_path, monkeypatch, built_lib):
    monkeypatch.chdir(tmp_path)      # prepareProblem writes data/parameter_list.txt.0


def rel_l2(a, b):
    a = np.asarray(a).astype(np.complex128).ravel()
    b = np.asarray(b).astype(np.complex128).ravel()
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def run_case(spec, shape, dt, nsteps, inits, seed=1234, d=(1.0, 1.0, 1.0), chunks=None,
             precision="f64"):
    import cupss_gb300 as c
    fields, params, eqs, noises = spec
    sx, sy, sz = shape
    s = System()
    for n, dyn in fields:
        s.create_field(n, bool(dyn))
    for k, v in params.items():
        s.add_parameter(k, v)
    for q in eqs:
        s.add_equation(q)
    for f, a in noises:
        s.add_noise(f, a)
    r = RefSolver(s, sx, sy, sz, *d, dt=dt, precision=precision,
                  noise=NoiseProvider(sx, sy, sz, seed))
    e = c.Evolver(True, sx, sy, sz, *d, dt=dt, write_every=10 ** 9)
    for n, dyn in fields:
        e.createField(n, bool(dyn))
    for k, v in params.items():
        e.addParameter(k, v)
    for q in eqs:
        e.addEquation(q)
    for f, a in noises:
        e.addNoise(f, a)
    e.setNoiseSeed(seed)
    for n, arr in inits.items():
        r.set_real(n, arr)
        e.setReal(n, arr)
    r.prepare()
    e.prepareProblem()
    for k in (chunks or [nsteps]):
        r.advance(k)
        e.advanceTime(k)
    return r, e, [n for n, _ in fields]


def init_field(shape, lo=-0.1, hi=0.1, seed=20261203):
    from cupss_gb300.workloads import splitmix64_uniform
    sx, sy, sz = shape
    return splitmix64_uniform(sx * sy * sz, seed, lo, hi).reshape(sz, sy, sx)


CH = ([("phi", 1)], {"a": -1.0, "b": 1.0, "k": 1.0},
      ["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3"], [])


# ---------------------------------------------------------------------------------------------
# the reference's own known-answer tests, through this library (tests/tests.cpp:64-422)
@pytest.mark.parametrize("dim", [1, 2, 3])
def test_reference_init_goldens(dim):
    # the library's own evolver::initializeDroplet (src/initializers.cpp:142-177), called
    # through the C-ABI with the reference test's arguments (tests/tests.cpp:64-189), then
    # uploaded, transformed and read back by the engine
    import cupss_gb300 as c
    shape = {1: (16, 1, 1), 2: (16, 16, 1), 3: (16, 16, 16)}[dim]
    e = c.Evolver(True, *shape, dt=1.0, write_every=1)
    e.createField("phi", True)
    e.initializeDroplet("phi", 0, 1, 16 / 8, 4, 8, 8 if dim > 1 else 0, 0)
    e.prepareProblem()
    got = e.getReal("phi").ravel()
    assert np.abs(got - GOLD["phi_%dd" % dim]).max() < 1e-4


@pytest.mark.parametrize("dev", ["cpu", "gpu"])
@pytest.mark.parametrize("dim", [1, 3])
def test_reference_operator_goldens(dim, dev):
    sfx = "_%s_%dd" % (dev, dim)
    names = ["phi", "lapphi", "iqxphi"] + (["iqyphi", "iqzphi"] if dim == 3 else []) + ["invqphi"]
    eqs = ["dt phi%s+q^2*phi%s = iqxphi%s^2" % (sfx, sfx, sfx), "lapphi%s = -q^2*phi%s" % (sfx, sfx),
           "iqxphi%s =  iqx*phi%s" % (sfx, sfx)]
    if dim == 3:
        eqs += ["iqyphi%s =  iqy*phi%s" % (sfx, sfx), "iqzphi%s =  iqz*phi%s" % (sfx, sfx)]
    eqs += ["invqphi%s =  1/q*phi%s" % (sfx, sfx)]
    spec = ([(n + sfx, n == "phi") for n in names], {}, eqs, [])
    shape = (16, 1, 1) if dim == 1 else (16, 16, 16)
    init = {"phi" + sfx: droplet(shape, 0, 1, 2, 4, 8, 8 if dim == 3 else 0, 0)}
    r, e, _ = run_case(spec, shape, 1.0, 1, init)
    for n in names[1:]:
        key = n + sfx
        got = e.getReal(key).ravel()
        assert np.abs(got - GOLD[key]).max() < 1e-4, key
        assert np.abs(got - r.real_field(key).ravel()).max() < 2e-6, key


# ---------------------------------------------------------------------------------------------
@pytest.mark.parametrize("shape,nsteps", [((64, 64, 1), 200), ((32, 64, 1), 100), ((128, 16, 1), 100)])
def test_cahn_hilliard_2d(shape, nsteps):
    r, e, _ = run_case(CH, shape, 0.01, nsteps, {"phi": init_field(shape)})
    err = rel_l2(e.getReal("phi"), r.real_field("phi"))
    assert err < 2e-5, err
    # Fourier-space readout in the reference layout equals FFT of the real field
    F = e.getFourier("phi")
    assert rel_l2(F, np.fft.fftn(r.real_field("phi"))) < 2e-5


def test_cahn_hilliard_3d_conserved_noise():
    shape = (32, 32, 32)
    spec = ([("phi", 1)], {"a": -1.0, "b": 1.0, "k": 1.0, "T": 0.01},
            ["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3"], [("phi", "2*T*q^2")])
    r, e, _ = run_case(spec, shape, 0.005, 40, {"phi": init_field(shape, -0.05, 0.05)}, seed=99)
    err = rel_l2(e.getReal("phi"), r.real_field("phi"))
    assert err < 2e-5, err


@pytest.mark.parametrize("shape", [(16, 8, 32), (8, 32, 16), (64, 4, 4)])
def test_3d_rectangular(shape):
    spec = ([("phi", 1)], {"a": -1.0, "b": 1.0, "k": 1.0},
            ["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3 + 0.3*iqz*phi^2"], [("phi", "0.0001")])
    r, e, _ = run_case(spec, shape, 0.01, 25, {"phi": init_field(shape, -0.3, 0.3)}, seed=5)
    err = rel_l2(e.getReal("phi"), r.real_field("phi"))
    assert err < 2e-5, err


def test_kpz_2d_with_nondynamic_fields():
    shape = (32, 32, 1)
    spec = ([("h", 1), ("iqxh", 0), ("iqyh", 0)], {"nu": 1.3, "lambda": 2.0, "D": 1.0},
            ["dt h + nu*q^2*h = 0.5*lambda*iqxh^2 + 0.5*lambda*iqyh^2", "iqxh = iqx*h", "iqyh = iqy*h"],
            [("h", "2*D")])
    r, e, names = run_case(spec, shape, 0.005, 60, {"h": init_field(shape, -0.2, 0.2)}, seed=3)
    for n in names:
        err = rel_l2(e.getReal(n), r.real_field(n))
        assert err < 3e-5, (n, err)


@pytest.mark.parametrize("shape", [(32, 32, 1), (1024, 16, 1), (16, 1024, 1), (32, 512, 1)])
def test_model_h_2d(shape):
    """Model H, 6 fields.  The long-line shapes run the split line FFT (512 and 1024
    points) in the multi-input row pass and in the multi-field turnaround."""
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


def test_model_h_explicit_velocity_example_system():
    """System of examples/04_model_h/modelh_explicit_velocity.cpp (reduced size)."""
    shape = (32, 32, 1)
    spec = ([("phi", 1), ("iqxphi", 0), ("iqyphi", 0), ("sigxx", 0), ("sigxy", 0), ("vx", 0), ("vy", 0),
             ("w", 0)],
            {"a": -1.0, "b": 1.0, "k": 4.0, "eta": 1.0, "friction": 0.0, "ka": -4.0, "D": 0.01},
            ["dt phi + ( a *q^2 + k*q^4)*phi= - b* q^2* phi^3 -vx*iqxphi - vy*iqyphi",
             "iqxphi = iqx*phi", "iqyphi = iqy*phi",
             "sigxx = - 0.5*ka *iqxphi * iqxphi + 0.5*ka*iqyphi*iqyphi",
             "sigxy = - ka *iqxphi * iqyphi",
             "vx * (friction + eta*q^2) = (iqx + iqx^3*1/q^2 - iqx*iqy^2*1/q^2) * sigxx + (iqy + iqx^2* iqy*1/q^2 + iqx^2*iqy*1/q^2) * sigxy",
             "vy * (friction + eta*q^2) = (iqx + iqx*iqy^2*1/q^2 + iqx*iqy^2*1/q^2) * sigxy + (-iqy - iqy^3*1/q^2 + iqx^2*iqy*1/q^2) * sigxx",
             "w = 0.5*iqx * vy - 0.5*iqy*vx "], [])
    r, e, names = run_case(spec, shape, 0.05, 30, {"phi": init_field(shape, -0.5, 0.5)})
    for n in names:
        err = rel_l2(e.getReal(n), r.real_field(n))
        assert err < 5e-5, (n, err)


def test_1d_noisy_ch():
    shape = (128, 1, 1)
    spec = ([("phi", 1)], {"a": -1.0, "b": 1.0, "k": 1.0, "T": 0.01},
            ["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3"], [("phi", "2*T*q^2")])
    r, e, _ = run_case(spec, shape, 0.01, 150, {"phi": init_field(shape)}, seed=8)
    err = rel_l2(e.getReal("phi"), r.real_field("phi"))
    assert err < 2e-5, err


def test_edge_terms():
    """Constant source, mixed i-parity group, noise-only non-dynamic field, field with no
    equation, non-dynamic implicit with 1/q, quadratic product (2/3 rule)."""
    shape = (16, 32, 1)
    spec = ([("u", 1), ("n", 0), ("idle", 0), ("v", 0)], {"a": 0.5},
            ["dt u + a*q^2*u = 0.25 + iqx*u + 0.1*u - 0.3*u^2 + v",
             "v*(1 + q^2 + 1/q) = iqy*u + u^2"],
            [("n", "0.01*q^2")])
    r, e, names = run_case(spec, shape, 0.02, 30, {"u": init_field(shape, -0.5, 0.5),
                                                   "idle": init_field(shape, 0, 1, seed=4)}, seed=21)
    for n in names:
        err = rel_l2(e.getReal(n), r.real_field(n))
        assert err < 3e-5, (n, err)


def test_update_parameter_mid_run():
    import cupss_gb300 as c
    shape = (32, 32, 1)
    init = init_field(shape)
    r, e, _ = run_case(CH, shape, 0.01, 20, {"phi": init})
    e.updateParameter("b", 2.0)
    e.updateParameter("a", -0.5)
    r.sys.update_parameter("b", 2.0)
    r.sys.update_parameter("a", -0.5)
    r.prepare_tables_only()
    e.advanceTime(20)
    r.advance(20)
    assert rel_l2(e.getReal("phi"), r.real_field("phi")) < 2e-5


def test_deterministic_rerun():
    shape = (32, 32, 8)
    spec = ([("phi", 1)], {"a": -1.0, "b": 1.0, "k": 1.0, "T": 0.01},
            ["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3"], [("phi", "2*T*q^2")])
    outs = []
    for _ in range(2):
        import cupss_gb300 as c
        e = c.Evolver(True, *shape, dt=0.01, write_every=10 ** 9)
        e.createField("phi", True)
        for k, v in spec[1].items():
            e.addParameter(k, v)
        e.addEquation(spec[2][0])
        e.addNoise("phi", spec[3][0][1])
        e.setNoiseSeed(77)
        e.setReal("phi", init_field(shape))
        e.prepareProblem()
        e.advanceTime(20)
        outs.append(e.getReal("phi"))
    assert np.array_equal(outs[0], outs[1])


def test_edwards_wilkinson_stationary_spectrum():
    """EW: phi'(q) = (phi(q) + A xi(q)) / (1 + c), c = dt D q^2, A^2 = dt 2D / dV,
    E|xi|^2 = N  =>  stationary E|phi(q)|^2 = A^2 N / (c (2 + c))  (q != 0)."""
    import cupss_gb300 as c
    sx = sy = 64
    dt, D = 0.1, 1.0
    e = c.Evolver(True, sx, sy, 1, dt=dt, write_every=10 ** 9)
    e.createField("phi", True)
    e.addParameter("D", D)
    e.addEquation("dt phi + D * q^2 * phi = 0")
    e.addNoise("phi", "2*D")
    e.setNoiseSeed(2024)
    e.prepareProblem()
    e.advanceTime(300)
    qx = np.fft.fftfreq(sx) * 2 * np.pi
    qy = np.fft.fftfreq(sy) * 2 * np.pi
    QY, QX = np.meshgrid(qy, qx, indexing="ij")
    q2 = (QX ** 2 + QY ** 2)[None]
    cq = dt * D * q2
    N = sx * sy
    with np.errstate(divide="ignore", invalid="ignore"):
        theory = (dt * 2 * D) * N / (cq * (2 + cq))
    acc = np.zeros((1, sy, sx))
    nsamp = 200
    for _ in range(nsamp):
        e.advanceTime(5)
        F = e.getFourier("phi")
        acc += np.abs(F) ** 2
    acc /= nsamp
    sel = (q2 > 0.5) & np.isfinite(theory)
    ratio = acc[sel] / theory[sel]
    assert abs(ratio.mean() - 1.0) < 0.02, ratio.mean()
    bins = np.digitize(np.sqrt(q2[sel]), [1.0, 1.5, 2.0, 2.5, 3.0])
    for b in np.unique(bins):
        assert abs(ratio[bins == b].mean() - 1.0) < 0.06, (b, ratio[bins == b].mean())


@pytest.mark.parametrize("shape", [(2, 1, 1), (4, 1, 1), (8, 1, 1), (2048, 1, 1), (4, 2, 1), (16, 1024, 1),
                                   (1024, 4, 1), (4, 4, 2), (8, 2, 1024), (4, 256, 8), (512, 2, 4),
                                   (4, 512, 4), (8, 4, 512), (4, 1024, 2), (2048, 2, 2), (8, 4, 256)])
def test_fft_sizes_round_trip_and_one_step(shape):
    import cupss_gb300 as c
    sx, sy, sz = shape
    init = init_field(shape, -1, 1)
    s = c.Solver(sx, sy, sz, dt=0.01)
    f = s.add_field(True)
    s.set_implicit(f, [(-1.0, 1, 0, 0, 0, 0)])
    s.prepare()
    s.set_real(f, init)
    back = s.get_real(f)
    assert np.abs(back - init).max() < 2e-6 * max(1.0, np.log2(sx * sy * sz))
    F = s.get_fourier(f)
    assert rel_l2(F, np.fft.fftn(init.astype(np.float64))) < 3e-6
    spec = ([("phi", 1)], {"a": -1.0, "b": 1.0, "k": 1.0},
            ["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3 + iqx*iqy*phi^2"], [("phi", "0.001*q^2")])
    r, e, _ = run_case(spec, shape, 0.01, 3, {"phi": init}, seed=6)
    assert rel_l2(e.getReal("phi"), r.real_field("phi")) < 3e-6


@pytest.mark.parametrize("which", ["modelh2d", "ch3d"])
def test_generated_program_matches_table_driven(which, monkeypatch):
    """The update program compiled for the system (default) and the table-driven
    update kernel (CUPSSGB_JIT=0) give the same fields."""
    if which == "modelh2d":
        shape = (32, 32, 1)
        spec = ([("phi", 1), ("iqxphi", 0), ("iqyphi", 0), ("lapphi", 0), ("vx", 0), ("vy", 0)],
                {"a": -1.0, "b": 1.0, "k": 4.0, "eta": 1.0, "T": 0.001},
                ["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3 - vx*iqxphi - vy*iqyphi",
                 "iqxphi = iqx*phi", "iqyphi = iqy*phi", "lapphi = -q^2*phi",
                 "vx*eta*q^2 = -k*iqxphi*lapphi - k*iqx^2*1/q^2*iqxphi*lapphi - k*iqx*iqy*1/q^2*iqyphi*lapphi",
                 "vy*eta*q^2 = -k*iqyphi*lapphi - k*iqy^2*1/q^2*iqyphi*lapphi - k*iqx*iqy*1/q^2*iqxphi*lapphi"],
                [("phi", "2*T")])
    else:
        shape = (32, 16, 32)
        spec = ([("phi", 1)], {"a": -1.0, "b": 1.0, "k": 1.0, "T": 0.01},
                ["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3"], [("phi", "2*T*q^2")])
    init = {spec[0][0][0]: init_field(shape, -0.5, 0.5)}
    monkeypatch.setenv("CUPSSGB_JIT", "0")
    _, e0, names = run_case(spec, shape, 0.01, 20, init, seed=4)
    monkeypatch.setenv("CUPSSGB_JIT", "1")
    _, e1, _ = run_case(spec, shape, 0.01, 20, init, seed=4)
    for n in names:
        assert rel_l2(e1.getReal(n), e0.getReal(n)) < 5e-6, n


@pytest.mark.parametrize("shape", [(32, 16, 32), (64, 64, 1)])
def test_early_noise_order_gives_the_same_fields(shape, monkeypatch):
    """The generated turnaround may draw the first field's noise while the first product's
    loads are in flight (the default for spectra of 64 MB and more); the fields are the
    same either way, bit for bit (same noise values, same arithmetic)."""
    spec = ([("phi", 1)], {"a": -1.0, "b": 1.0, "k": 1.0, "T": 0.01},
            ["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3"], [("phi", "2*T*q^2")])
    init = {"phi": init_field(shape, -0.5, 0.5)}
    monkeypatch.setenv("CUPSSGB_EARLY_NOISE", "0")
    r, late, _ = run_case(spec, shape, 0.01, 20, init, seed=8)
    monkeypatch.setenv("CUPSSGB_EARLY_NOISE", "1")
    _, early, _ = run_case(spec, shape, 0.01, 20, init, seed=8)
    assert np.array_equal(early.getReal("phi"), late.getReal("phi"))
    assert rel_l2(late.getReal("phi"), r.real_field("phi")) < 2e-5


KPZ2 = ([("h", 1), ("iqxh", 0), ("iqyh", 0)], {"nu": 1.0, "la": 1.0, "lb": 1.0, "D": 1.0},
        ["dt h + nu*q^2*h = 0.5*la*iqxh^2 + 0.5*lb*iqyh^2", "iqxh = iqx*h", "iqyh = iqy*h"],
        [("h", "2*D")])


def test_merged_products_split_when_their_prefactors_part():
    """la = lb: the two squares share one product channel (summed in real space); after
    updateParameter("lb") the terms differ, the solver re-plans without merging at the next
    step, and the run still matches the oracle (which never merges)."""
    shape = (64, 32, 1)
    init = init_field(shape, -0.3, 0.3)
    r, e, _ = run_case(KPZ2, shape, 0.005, 20, {"h": init})
    assert rel_l2(e.getReal("h"), r.real_field("h")) < 3e-5
    e.updateParameter("lb", 2.5)
    r.sys.update_parameter("lb", 2.5)
    r.prepare_tables_only()
    e.advanceTime(20)
    r.advance(20)
    for nm in ("h", "iqxh", "iqyh"):
        assert rel_l2(e.getReal(nm), r.real_field(nm)) < 3e-5, nm
