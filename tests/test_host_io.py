"""Host-side parts of the drop-in API that need no GPU, called through the C-ABI.

* writeOut's file format: cupssgb_write_field_csv against a restatement of the
  reference's writer (src/field.cpp:350-402 of cuPSS): header "x, [y, [z, ]]name",
  then "i, [j, [k, ]]value" lines with writePrecision decimals, index order
  k*sx*sy + j*sx + i; a NaN value is an error.
* The initial conditions (src/initializers.cpp:14-267): the library's
  initializeDroplet against the reference's own droplet goldens
  (tests/base_truths/phi_1d|2d|3d, tests/tests.cpp:64-189, tolerance 1e-4 as there),
  the other initializers against the formulas, and initializeFromFile on a file
  written in the output format.
* createFromFile (src/parser.cpp:11-96): a system file gives the same IR as the same
  system declared call by call.
An evolver touches the GPU only from prepareProblem on, so all of this runs here.
"""
import os

import numpy as np
import pytest

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_base_truths.npz"))


@pytest.fixture(autouse=True)
def _lib(built_lib, tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)


def reference_csv(name, values, shape, precision):
    """The text the reference's field::writeToFile writes for these values."""
    sx, sy, sz = shape
    dim = 1 if sy == 1 and sz == 1 else (2 if sz == 1 else 3)
    head = {1: "x, ", 2: "x, y, ", 3: "x, y, z, "}[dim] + name + "\n"
    vfmt = "%." + str(precision) + "f\n"
    v = np.asarray(values, np.float32).reshape(-1)
    out = [head]
    idx = 0
    for k in range(sz):
        for j in range(sy):
            for i in range(sx):
                coords = {1: "%i, " % i, 2: "%i, %i, " % (i, j), 3: "%i, %i, %i, " % (i, j, k)}[dim]
                out.append(coords + vfmt % float(v[idx]))
                idx += 1
    return "".join(out)


@pytest.mark.parametrize("shape,precision", [((16, 1, 1), 6), ((8, 4, 1), 6), ((4, 4, 2), 3), ((8, 2, 2), 8)])
def test_csv_bytes_match_reference_format(shape, precision):
    from cupss_gb300.api import write_field_csv
    sx, sy, sz = shape
    rng = np.random.default_rng(7)
    vals = (rng.standard_normal(sx * sy * sz) * 10.0 ** rng.integers(-4, 3, sx * sy * sz)).astype(np.float32)
    vals[0] = -0.0
    vals[1] = 123456.789
    write_field_csv("f.csv", "phi", vals.reshape(sz, sy, sx), precision=precision)
    with open("f.csv") as fh:
        got = fh.read()
    assert got == reference_csv("phi", vals, shape, precision)


def test_csv_nan_is_an_error():
    from cupss_gb300.api import write_field_csv
    from cupss_gb300.capi import CupssError
    vals = np.zeros((4, 4), np.float32)
    vals[2, 1] = np.nan
    with pytest.raises(CupssError, match="NaN found in field rho"):
        write_field_csv("g.csv", "rho", vals)


def make(shape, name="phi"):
    import cupss_gb300 as c
    e = c.Evolver(True, *shape, dt=0.01, write_every=1)
    e.createField(name, True)
    return e


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_library_droplet_matches_reference_goldens(dim):
    shape = {1: (16, 1, 1), 2: (16, 16, 1), 3: (16, 16, 16)}[dim]
    e = make(shape)
    # the reference test's call: initializeDroplet(f, 0, 1, 16/8, 4, 16/2, 16/2 (or 0), 0)
    e.initializeDroplet("phi", 0, 1, 16 / 8, 4, 8, 8 if dim > 1 else 0, 0)
    got = e.getHostReal("phi").ravel()
    assert np.abs(got - GOLD["phi_%dd" % dim]).max() < 1e-4
    e.close()


def droplet_formula(shape, vout, vin, radius, width, c):
    sx, sy, sz = shape
    k, j, i = np.meshgrid(np.arange(sz), np.arange(sy), np.arange(sx), indexing="ij")
    x0, y0, z0 = c[0] % sx, c[1] % sy, c[2] % sz
    rc = np.sqrt(((i - x0) ** 2 + (j - y0) ** 2 + (k - z0) ** 2).astype(np.float32))
    return vout + (vin - vout) * 0.5 * (1.0 + np.tanh((rc - radius) / (np.sqrt(2.0) * width)))


def test_initializers_follow_the_reference_formulas():
    shape = (12, 10, 6)
    sx, sy, sz = shape
    e = make(shape)
    e.createField("psi", False)
    e.initializeUniform("phi", 0.25)
    assert np.all(e.getHostReal("phi") == np.float32(0.25))
    # half system along each axis: v1 + (v2 - v1)/2 (1 + tanh((r - L/2) / (sqrt 2 w)))
    for direction, n in ((1, sx), (2, sy), (3, sz)):
        e.initializeHalfSystem("phi", -1.0, 2.0, 1.5, direction)
        k, j, i = np.meshgrid(np.arange(sz), np.arange(sy), np.arange(sx), indexing="ij")
        r = (i, j, k)[direction - 1]
        want = -1.0 + 3.0 * 0.5 * (1.0 + np.tanh((r - n // 2) / (np.sqrt(2.0) * 1.5)))
        assert np.abs(e.getHostReal("phi") - want).max() < 1e-6
    # droplet, then a second droplet added on top (centres wrap modulo the grid)
    e.initializeDroplet("psi", 0.1, 0.9, 3.0, 1.0, 15, 4, 2)
    base = droplet_formula(shape, 0.1, 0.9, 3.0, 1.0, (15, 4, 2))
    assert np.abs(e.getHostReal("psi") - base).max() < 1e-6
    e.addDroplet("psi", 0.5, 2.0, 0.7, 1, 1, 1)
    k, j, i = np.meshgrid(np.arange(sz), np.arange(sy), np.arange(sx), indexing="ij")
    rc = np.sqrt(((i - 1) ** 2 + (j - 1) ** 2 + (k - 1) ** 2).astype(np.float32))
    want = base + 0.5 * 0.5 * (1.0 + np.tanh((2.0 - rc) / (np.sqrt(2.0) * 0.7)))
    assert np.abs(e.getHostReal("psi") - want).max() < 2e-6
    # uniform noise: amplitude * 0.01 * (rand() % 200 - 100), so multiples of amplitude/100 in [-a, a)
    e.initializeUniformNoise("phi", 0.5)
    u = e.getHostReal("phi").astype(np.float64) / 0.005
    assert np.abs(u - np.round(u)).max() < 1e-3 and u.min() >= -100.5 and u.max() <= 99.5
    assert len(np.unique(np.round(u))) > 50
    # normal noise: Box-Muller of pairs scaled by sigma^2 (the reference's sigma*sigma) plus the mean
    e.initializeNormalNoise("phi", 3.0, 0.5)
    g = e.getHostReal("phi")
    assert abs(g.mean() - 3.0) < 0.05 and 0.15 < g.std() < 0.35
    e.close()


def test_initializer_errors_are_reported():
    from cupss_gb300.capi import CupssError
    e = make((8, 8, 1))
    with pytest.raises(CupssError, match="no field"):
        e.initializeUniform("nope", 1.0)
    with pytest.raises(CupssError, match="interface width"):
        e.initializeHalfSystem("phi", 0.0, 1.0, 0.0, 1)
    with pytest.raises(CupssError, match="direction"):
        e.initializeHalfSystem("phi", 0.0, 1.0, 1.0, 4)
    with pytest.raises(CupssError, match="radius"):
        e.initializeDroplet("phi", 0.0, 1.0, -1.0, 1.0, 0, 0, 0)
    with pytest.raises(CupssError, match="not found"):
        e.initializeFromFile("phi", "missing.csv", 1, ",")
    e.close()


@pytest.mark.parametrize("shape", [(16, 1, 1), (8, 6, 1), (4, 3, 5)])
def test_initialize_from_file_reads_the_output_format(shape):
    from cupss_gb300.api import write_field_csv
    sx, sy, sz = shape
    vals = np.random.default_rng(3).uniform(-1, 1, sx * sy * sz).astype(np.float32)
    write_field_csv("init.csv", "phi", vals.reshape(sz, sy, sx))
    e = make(shape)
    e.initializeFromFile("phi", "init.csv", 1, ",")   # skip the header line
    got = e.getHostReal("phi").ravel()
    assert np.abs(got - vals).max() <= 5.1e-7
    e.close()


SYSTEM_FILE = """# model B with an auxiliary field
Fields
phi 1 1
mu 0 0

Parameters
a -1.0
b 1.0
k 2.5

Equations
mu = a*phi + b*phi^3 - k*q^2*phi
dt phi = -q^2*mu
"""


def test_create_from_file_equals_calls():
    import cupss_gb300 as c
    with open("system.txt", "w") as fh:
        fh.write(SYSTEM_FILE)
    a = c.Evolver(True, 32, 32, 1, dt=0.01, write_every=1)
    a.createFromFile("system.txt")
    b = c.Evolver(True, 32, 32, 1, dt=0.01, write_every=1)
    b.createField("phi", True)
    b.createField("mu", False)
    b.setOutputField("phi", 1)
    for k, v in (("a", -1.0), ("b", 1.0), ("k", 2.5)):
        b.addParameter(k, v)
    b.addEquation("mu = a*phi + b*phi^3 - k*q^2*phi")
    b.addEquation("dt phi = -q^2*mu")
    assert a.describe() == b.describe()
    assert a.getParameter("k") == pytest.approx(2.5)
    a.close()
    b.close()


def test_create_from_file_rejects_a_bad_file():
    import cupss_gb300 as c
    from cupss_gb300.capi import CupssError
    with open("bad.txt", "w") as fh:
        fh.write("phi 1 1\n")
    e = c.Evolver(True, 16, 16, 1, dt=0.01, write_every=1)
    with pytest.raises(CupssError):
        e.createFromFile("bad.txt")
    with pytest.raises(CupssError):
        e.createFromFile("no_such_file.txt")
    e.close()


def test_device_info_without_a_gpu_is_not_an_error():
    from cupss_gb300.api import device_info
    n, text = device_info()
    assert n >= 0
    assert "runtime" in text
