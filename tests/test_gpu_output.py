"""writeOut on the GPU path: files written in the background while the steps go on.

evolver::writeOut (src/evolver.cpp:228-232, src/field.cpp:350-402 of cuPSS) writes
data/<field>.csv.<step> every writeEveryNSteps steps, before the step.  Here the field
is copied out on the engine's output stream and a background thread writes the file;
the tests check the files' bytes against the reference format applied to the field
the engine holds at that step (an identical twin evolver, advanced to the same step),
and the NaN rule.
"""
import os

import numpy as np
import pytest

from test_host_io import reference_csv

pytestmark = pytest.mark.gpu

CH = ({"a": -1.0, "b": 1.0, "k": 1.0}, "dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3")


@pytest.fixture(autouse=True)
def _in_tmp(tmp_path, monkeypatch, built_lib):
    monkeypatch.chdir(tmp_path)


def make(shape, write_every, init, output=True):
    import cupss_gb300 as c
    e = c.Evolver(True, *shape, dt=0.01, write_every=write_every)
    e.createField("phi", True)
    for k, v in CH[0].items():
        e.addParameter(k, v)
    e.addEquation(CH[1])
    if output:
        e.setOutputField("phi", 1)
    e.setReal("phi", init)
    e.prepareProblem()
    return e


@pytest.mark.parametrize("shape", [(64, 32, 1), (16, 16, 8)])
def test_written_files_match_the_field_at_their_step(shape):
    sx, sy, sz = shape
    init = np.random.default_rng(5).uniform(-0.1, 0.1, sx * sy * sz).astype(np.float32)
    e = make(shape, 5, init)
    e.advanceTime(12)          # files at steps 0, 5 and 10 (each before its step)
    e.flushOutput()
    names = sorted(os.listdir("data"))
    assert names == ["parameter_list.txt.0", "phi.csv.0", "phi.csv.10", "phi.csv.5"]
    for step in (0, 5, 10):
        twin = make(shape, 10 ** 9, init, output=False)
        twin.advanceTime(step)
        want = reference_csv("phi", twin.getReal("phi"), shape, 6)
        twin.close()
        with open("data/phi.csv.%d" % step) as fh:
            assert fh.read() == want, "file of step %d" % step
    e.close()


def test_many_files_in_flight_and_a_direct_write_out():
    shape = (32, 32, 1)
    init = np.random.default_rng(6).uniform(-0.1, 0.1, 32 * 32).astype(np.float32)
    e = make(shape, 1, init)
    e.advanceTime(20)          # one file per step: more than the writer keeps in flight
    e.writeOut()               # step 20, written on request
    e.flushOutput()
    for step in range(21):
        assert os.path.exists("data/phi.csv.%d" % step)
    twin = make(shape, 10 ** 9, init, output=False)
    twin.advanceTime(20)
    with open("data/phi.csv.20") as fh:
        assert fh.read() == reference_csv("phi", twin.getReal("phi"), shape, 6)
    twin.close()
    e.close()


def test_nan_in_an_output_field_is_reported():
    from cupss_gb300.capi import CupssError
    init = np.zeros(16 * 16, np.float32)
    init[17] = np.nan          # spreads through the transforms: the written field holds NaNs
    e = make((16, 16, 1), 1, init)
    with pytest.raises(CupssError, match="NaN found in field phi"):
        e.writeOut()
        e.flushOutput()
    e.close()
