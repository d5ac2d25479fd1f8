"""The served form: requests of different systems, grids and step counts submitted
while others run, admitted into batch-solver slots within an HBM budget.  Every
request's result must equal the same solve run alone through the plain evolver
(relative L2 1e-6: same kernels, only the source of the prefactor values and the
noise key differ in form, not in value)."""
import time

import numpy as np
import pytest

from cupss_gb300.workloads import SYSTEMS, declare, splitmix64_uniform

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _in_tmp(tmp_path, monkeypatch, built_lib):
    monkeypatch.chdir(tmp_path)


def rel(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


def alone(kind, shape, dt, nsteps, seed, params, init):
    import cupss_gb300 as c
    sysd = SYSTEMS[kind]
    e = c.Evolver(True, *shape, dt=dt, write_every=10 ** 9)
    for nm, dyn in sysd["fields"]:
        e.createField(nm, dyn)
    for k, v in sysd["params"].items():
        e.addParameter(k, params.get(k, v))
    for q in sysd["eqs"]:
        e.addEquation(q)
    for f, a in sysd["noise"]:
        e.addNoise(f, a)
    e.setNoiseSeed(seed)
    for nm, arr in init.items():
        e.setReal(nm, arr)
    e.prepareProblem()
    e.advanceTime(nsteps)
    out = e.getReal(sysd["out"])
    e.close()
    return out


REQS = [
    ("kpz", (64, 64, 1), 0.005, 120, {"nu": 1.2, "lam": 1.5}),
    ("ch", (64, 64, 1), 0.01, 75, {"T": 0.0}),
    ("ew", (128, 64, 1), 0.01, 200, {"nu": 0.7}),
    ("kpz", (64, 64, 1), 0.005, 33, {"nu": 0.9, "lam": 0.5}),
    ("ch", (16, 16, 16), 0.01, 90, {"T": 0.02}),
    ("kpz", (32, 32, 1), 0.005, 257, {"nu": 1.7, "lam": 2.0}),
    ("ch", (64, 64, 1), 0.01, 40, {"T": 0.01}),
    ("ew", (128, 64, 1), 0.01, 18, {"nu": 1.4}),
]


def init_of(kind, shape, i):
    n = int(np.prod(shape))
    field = SYSTEMS[kind]["out"]
    return {field: splitmix64_uniform(n, 300 + i, -0.2, 0.2).reshape(shape[::-1])}


@pytest.mark.parametrize("max_chunk", [16, 64])
def test_served_results_equal_alone(max_chunk):
    import cupss_gb300 as c
    srv = c.Server(hbm_budget=4e9, max_slots=3, max_chunk=max_chunk)
    sids = {k: srv.addSystem(SYSTEMS[k]) for k in ("kpz", "ch", "ew")}
    ids = []
    for i, (kind, shape, dt, n, params) in enumerate(REQS):
        ids.append(srv.submit(sids[kind], shape, dt, n, seed=5000 + i, params=params,
                              init=init_of(kind, shape, i)))
        time.sleep(0.01 * (i % 3))   # some arrive while others run
    for rid in ids:
        assert srv.wait(rid, 120.0)
    st = srv.stats()
    assert st["done"] == len(REQS) and st["queued"] == 0 and not st["error"]
    for i, (kind, shape, dt, n, params) in enumerate(REQS):
        ref = alone(kind, shape, dt, n, 5000 + i, params, init_of(kind, shape, i))
        got = srv.result(ids[i])
        assert rel(got, ref) < 1e-6, (i, kind, rel(got, ref))
        t_sub, t_adm, t_fin = srv.times(ids[i])
        assert 0 <= t_sub <= t_adm <= t_fin
    srv.close()


def test_budget_admission_serialises_pools():
    """A budget that holds one pool at a time: requests of the second key wait until the
    first pool is idle and freed, and still give the same results."""
    import cupss_gb300 as c
    from tests.test_codegen import solver_from_ir
    from tests.test_parser_parity import build_lib

    def pool_bytes(kind):
        sd = SYSTEMS[kind]
        s = solver_from_ir(build_lib(sd["fields"], sd["params"], sd["eqs"], sd["noise"]), (64, 64, 1))
        b = s.estimate_bytes(2)
        s.close()
        return b

    kb, cb = pool_bytes("kpz"), pool_bytes("ch")
    budget = max(kb, cb) * 1.05
    assert budget < kb + cb
    srv = c.Server(hbm_budget=budget, max_slots=2, max_chunk=32)
    k = srv.addSystem(SYSTEMS["kpz"])
    h = srv.addSystem(SYSTEMS["ch"])
    r1 = srv.submit(k, (64, 64, 1), 0.005, 100, seed=1, params={"lam": 1.0})
    r2 = srv.submit(h, (64, 64, 1), 0.01, 60, seed=2, init=init_of("ch", (64, 64, 1), 2))
    r3 = srv.submit(k, (64, 64, 1), 0.005, 50, seed=3, params={"lam": 3.0})
    for r in (r1, r2, r3):
        assert srv.wait(r, 120.0)
    assert srv.times(r2)[1] >= max(srv.times(r1)[2], srv.times(r3)[2])
    assert rel(srv.result(r1), alone("kpz", (64, 64, 1), 0.005, 100, 1, {"lam": 1.0}, {})) < 1e-6
    assert rel(srv.result(r2), alone("ch", (64, 64, 1), 0.01, 60, 2, {}, init_of("ch", (64, 64, 1), 2))) < 1e-6
    assert rel(srv.result(r3), alone("kpz", (64, 64, 1), 0.005, 50, 3, {"lam": 3.0}, {})) < 1e-6
    srv.close()
