"""Synthetic workload definitions (seeded initial fields, equation strings).

Initial fields come from a seeded SplitMix64 stream mapped to uniform floats, so
the same field can be regenerated bit-for-bit anywhere (seed 20261203 by default).
"""
from __future__ import annotations

import numpy as np

DEFAULT_SEED = 20261203


def splitmix64_uniform(n, seed=DEFAULT_SEED, lo=-0.1, hi=0.1):
    """n float32 values uniform in [lo, hi) from SplitMix64 (Steele, Lea, Flood 2014)."""
    with np.errstate(over="ignore"):
        idx = np.arange(1, n + 1, dtype=np.uint64)
        z = np.uint64(seed) + idx * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    u = (z >> np.uint64(40)).astype(np.float64) * 2.0 ** -24
    return (lo + (hi - lo) * u).astype(np.float32)


# Equation strings in reference syntax (cf. examples/02_cahn_hilliard, 03_cahn_hilliard_3d,
# 05_edwards_wilkinson, 06_kpz of the reference).
CH_EQ = "dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3"
CH_NOISE = "2*T*q^2"

# Systems of the batched and served workloads, as evolver declarations.
SYSTEMS = {
    "kpz": dict(fields=[("h", True), ("iqxh", False), ("iqyh", False)],
                params={"nu": 1.0, "lam": 1.0, "D": 1.0},
                eqs=["dt h + nu*q^2*h = 0.5*lam*iqxh^2 + 0.5*lam*iqyh^2", "iqxh = iqx*h", "iqyh = iqy*h"],
                noise=[("h", "2*D")], out="h"),
    "ew": dict(fields=[("h", True)], params={"nu": 1.0, "D": 1.0}, eqs=["dt h + nu*q^2*h = 0"],
               noise=[("h", "2*D")], out="h"),
    "ch": dict(fields=[("phi", True)], params={"a": -1.0, "b": 1.0, "k": 1.0, "T": 0.01},
               eqs=[CH_EQ], noise=[("phi", CH_NOISE)], out="phi"),
}


def declare(target, system):
    """Declares a SYSTEMS entry on an Evolver or Ensemble (same method names)."""
    for nm, dyn in system["fields"]:
        target.createField(nm, dyn)
    for k, v in system["params"].items():
        target.addParameter(k, v)
    for q in system["eqs"]:
        target.addEquation(q)
    for f, a in system["noise"]:
        target.addNoise(f, a)


def kpz_ensemble(n=512, seed=DEFAULT_SEED, sizes=(64, 128, 256, 512)):
    """Members of the KPZ ensemble: square 2D grids drawn uniformly from `sizes` (log-
    uniform in N), nu ~ U[0.5, 2], lambda ~ U[0, 4], D = 1, own Philox seed each, h0 = 0.
    Returns a list of dicts (n_side, nu, lam, seed)."""
    rng = np.random.default_rng(seed)
    side = rng.choice(np.asarray(sizes), size=n)
    nu = rng.uniform(0.5, 2.0, size=n)
    lam = rng.uniform(0.0, 4.0, size=n)
    return [dict(side=int(side[i]), nu=float(nu[i]), lam=float(lam[i]), seed=int(seed) * 4096 + i)
            for i in range(n)]


def served_stream(n=64, rate=2.0, seed=DEFAULT_SEED, steps_range=(1e3, 1e5)):
    """Poisson stream of solve requests drawn uniformly from {2D Edwards-Wilkinson, 2D
    KPZ, 2D Cahn-Hilliard, 3D Cahn-Hilliard}: 2D sides uniform over {64, 96, 128, 192, 256,
    512, 1024}, 3D sides over {64, 96, 128, 192} (the sizes 2^a and 3 * 2^a in 64..192), step counts
    log-uniform in steps_range (default [1e3, 1e5]), seeded parameters (nu ~ U[0.5, 2], KPZ lambda ~ U[0, 1],
    CH T ~ U[0, 0.01]) and seeded initial fields (CH: U[-0.1, 0.1]; EW, KPZ: flat).
    arrival: seconds after the first request."""
    rng = np.random.default_rng(seed)
    kinds = ["ew", "kpz", "ch2d", "ch3d"]
    gaps = rng.exponential(1.0 / rate, size=n)
    gaps[0] = 0.0
    arrival = np.cumsum(gaps)
    out = []
    for i in range(n):
        kind = kinds[int(rng.integers(4))]
        steps = int(round(10.0 ** rng.uniform(np.log10(steps_range[0]), np.log10(steps_range[1]))))
        if kind == "ch3d":
            side = int(rng.choice([64, 96, 128, 192]))
            shape = (side, side, side)
        else:
            side = int(rng.choice([64, 96, 128, 192, 256, 512, 1024]))
            shape = (side, side, 1)
        if kind == "ew":
            params, dt = {"nu": float(rng.uniform(0.5, 2.0))}, 0.01
        elif kind == "kpz":
            params, dt = {"nu": float(rng.uniform(0.5, 2.0)), "lam": float(rng.uniform(0.0, 1.0))}, 0.005
        else:
            params, dt = {"T": float(rng.uniform(0.0, 0.01))}, (0.01 if kind == "ch2d" else 0.005)
        out.append(dict(kind=kind, system="ch" if kind.startswith("ch") else kind, shape=shape, dt=dt,
                        steps=steps, params=params, seed=int(seed) * 8192 + i, init_seed=int(seed) + 17 * i,
                        arrival=float(arrival[i])))
    return out


def initial_fields(req):
    """Initial fields of a served_stream request (output field only; others start at 0)."""
    if req["system"] != "ch":
        return {}
    n = int(np.prod(req["shape"]))
    return {"phi": splitmix64_uniform(n, req["init_seed"], -0.1, 0.1).reshape(req["shape"][::-1])}
