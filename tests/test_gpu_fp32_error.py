"""FP32 error of the engine against the FP64 oracle, per configuration.

The configurations of the bench and parity plan at their physical parameters, with
grids and step counts reduced where the FP64 oracle would take minutes.  Noisy runs use
the identical noise realisation (oracle/philox.py).  Each test prints its relative L2
error (run with -s to see the table) and checks it against a bound a few times above
the value measured on a GB300, so a regression shows without making the test flaky.
"""
import numpy as np
import pytest

from tests.test_gpu_parity import init_field, rel_l2, run_case

pytestmark = pytest.mark.gpu

CH = (["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3"])
MODEL_H = ["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3 - vx*iqxphi - vy*iqyphi",
           "iqxphi = iqx*phi", "iqyphi = iqy*phi", "lapphi = -q^2*phi",
           "vx*eta*q^2 = -k*iqxphi*lapphi - k*iqx^2*1/q^2*iqxphi*lapphi - k*iqx*iqy*1/q^2*iqyphi*lapphi",
           "vy*eta*q^2 = -k*iqyphi*lapphi - k*iqy^2*1/q^2*iqyphi*lapphi - k*iqx*iqy*1/q^2*iqxphi*lapphi"]

CASES = {
    # 2D Cahn-Hilliard 256^2, no noise, dt 0.01 (2000 of the plan's 10,000 steps)
    "ch2d-256": dict(spec=([("phi", 1)], {"a": -1.0, "b": 1.0, "k": 1.0}, CH, []), shape=(256, 256, 1),
                     dt=0.01, steps=2000, init=(-0.1, 0.1), bound=1e-3),
    # 3D Cahn-Hilliard with conserved noise T = 0.01, dt 0.005 on a 64^3 grid
    "ch3d-64-noise": dict(spec=([("phi", 1)], {"a": -1.0, "b": 1.0, "k": 1.0, "T": 0.01}, CH,
                                [("phi", "2*T*q^2")]), shape=(64, 64, 64), dt=0.005, steps=400,
                          init=(-0.05, 0.05), bound=1e-4),
    # 2D model H, k = 4, eta = 1, T = 0.001, dt 0.01 on a 128^2 grid
    "modelh-128": dict(spec=([("phi", 1), ("iqxphi", 0), ("iqyphi", 0), ("lapphi", 0), ("vx", 0), ("vy", 0)],
                             {"a": -1.0, "b": 1.0, "k": 4.0, "eta": 1.0, "T": 0.001}, MODEL_H, [("phi", "2*T")]),
                       shape=(128, 128, 1), dt=0.01, steps=200, init=(-0.1, 0.1), bound=2e-4),
    # 2D KPZ, nu = 1, lambda = 2, D = 1, dt 0.005 on a 128^2 grid
    "kpz-128": dict(spec=([("h", 1), ("iqxh", 0), ("iqyh", 0)], {"nu": 1.0, "lam": 2.0, "D": 1.0},
                          ["dt h + nu*q^2*h = 0.5*lam*iqxh^2 + 0.5*lam*iqyh^2", "iqxh = iqx*h", "iqyh = iqy*h"],
                          [("h", "2*D")]), shape=(128, 128, 1), dt=0.005, steps=400, init=(0.0, 0.0),
                    bound=1e-4),
    # 2D Edwards-Wilkinson, nu = 1, D = 1, dt 0.005 on a 128^2 grid
    "ew-128": dict(spec=([("h", 1)], {"nu": 1.0, "D": 1.0}, ["dt h + nu*q^2*h = 0"], [("h", "2*D")]),
                   shape=(128, 128, 1), dt=0.005, steps=400, init=(0.0, 0.0), bound=1e-5),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_fp32_error_against_fp64_oracle(name):
    c = CASES[name]
    first = c["spec"][0][0][0]
    init = {first: init_field(c["shape"], *c["init"])}
    r, e, names = run_case(c["spec"], c["shape"], c["dt"], c["steps"], init, seed=20261203)
    errs = {n: rel_l2(e.getReal(n), r.real_field(n)) for n in names}
    print("\nFP32 vs FP64 oracle, %s (%s, %d steps): %s" % (
        name, "x".join(str(s) for s in c["shape"] if s > 1), c["steps"],
        ", ".join("%s %.2e" % kv for kv in errs.items())))
    assert all(np.isfinite(v) for v in errs.values())
    assert errs[first] < c["bound"], errs
