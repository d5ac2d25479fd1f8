"""Benchmark of the GB300 pseudospectral step (cuPSS drop-in).

Default workload: 3D Cahn-Hilliard with conserved noise on a 256^3 periodic grid,
FP32, a=-1, b=1, k=1, dt=0.005, T=0.01, phi0 ~ U[-0.05, 0.05] from SplitMix64
seed 20261203, equations in reference syntax:
    dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3      noise "2*T*q^2"
A bench step is one time step (evolver::advanceTime) of the whole grid; the
metric is grid-point-steps per second.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Under torchrun (N > 1) every rank advances its own independent replica (a single
solve does not shard); value = all ranks' point-steps / max rank time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "ch3d-256": dict(shape=(256, 256, 256), dt=0.005, params={"a": -1.0, "b": 1.0, "k": 1.0, "T": 0.01},
                     eqs=["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3"], noise=[("phi", "2*T*q^2")],
                     init=(-0.05, 0.05), solve_steps=2000, steps=2000, warmup=20),
    "ch3d-128": dict(shape=(128, 128, 128), dt=0.005, params={"a": -1.0, "b": 1.0, "k": 1.0, "T": 0.01},
                     eqs=["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3"], noise=[("phi", "2*T*q^2")],
                     init=(-0.05, 0.05), solve_steps=2000, steps=500, warmup=10),
    "ch3d-512": dict(shape=(512, 512, 512), dt=0.005, params={"a": -1.0, "b": 1.0, "k": 1.0, "T": 0.01},
                     eqs=["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3"], noise=[("phi", "2*T*q^2")],
                     init=(-0.05, 0.05), solve_steps=2000, steps=200, warmup=5),
    "ch2d-256": dict(shape=(256, 256, 1), dt=0.01, params={"a": -1.0, "b": 1.0, "k": 1.0},
                     eqs=["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3"], noise=[],
                     init=(-0.1, 0.1), solve_steps=10000, steps=10000, warmup=50),
    "ch2d-1024": dict(shape=(1024, 1024, 1), dt=0.01, params={"a": -1.0, "b": 1.0, "k": 1.0},
                      eqs=["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3"], noise=[],
                      init=(-0.1, 0.1), solve_steps=5000, steps=2000, warmup=20),
    "ch2d-2048x1024": dict(shape=(2048, 1024, 1), dt=0.01, params={"a": -1.0, "b": 1.0, "k": 1.0},
                           eqs=["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3"], noise=[],
                           init=(-0.1, 0.1), solve_steps=5000, steps=2000, warmup=20),
    # 2D model H: Cahn-Hilliard advected by the Stokes velocity of the Korteweg stress,
    # transverse projection in Fourier space (reference examples/04_model_h)
    "modelh-1024": dict(shape=(1024, 1024, 1), dt=0.01,
                        params={"a": -1.0, "b": 1.0, "k": 4.0, "eta": 1.0, "T": 0.001},
                        fields=[("phi", True), ("iqxphi", False), ("iqyphi", False), ("lapphi", False),
                                ("vx", False), ("vy", False)],
                        eqs=["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3 - vx*iqxphi - vy*iqyphi",
                             "iqxphi = iqx*phi", "iqyphi = iqy*phi", "lapphi = -q^2*phi",
                             "vx*eta*q^2 = -k*iqxphi*lapphi - k*iqx^2*1/q^2*iqxphi*lapphi"
                             " - k*iqx*iqy*1/q^2*iqyphi*lapphi",
                             "vy*eta*q^2 = -k*iqyphi*lapphi - k*iqy^2*1/q^2*iqyphi*lapphi"
                             " - k*iqx*iqy*1/q^2*iqxphi*lapphi"],
                        noise=[("phi", "2*T")], init=(-0.1, 0.1), solve_steps=5000, steps=1000, warmup=10,
                        B_alg=80.0, products=5),
}
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM = 6800.0


def peak_hbm():
    try:
        with open(PEAKS_FILE) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM, "fallback"


# --------------------------------------------------------------------------------------
# clocks sampler (nvidia-smi during the timed region)
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        time.sleep(0.15)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = list(self.rows)
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if "Active" in r[5 + i] and "Not" not in r[5 + i]})
        pw = [float(r[3]) for r in rows if r[3].replace(".", "").isdigit()]
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "power_w_max": max(pw) if pw else None}


# --------------------------------------------------------------------------------------
def make_evolver(wl, seed=42):
    import cupss_gb300 as c
    sx, sy, sz = wl["shape"]
    e = c.Evolver(True, sx, sy, sz, 1.0, 1.0, 1.0, dt=wl["dt"], write_every=10 ** 9)
    for nm, dyn in wl.get("fields", [("phi", True)]):
        e.createField(nm, dyn)
    for k, v in wl["params"].items():
        e.addParameter(k, v)
    for q in wl["eqs"]:
        e.addEquation(q)
    for f, a in wl["noise"]:
        e.addNoise(f, a)
    e.setNoiseSeed(seed)
    init = c.splitmix64_uniform(sx * sy * sz, 20261203, *wl["init"])
    e.setReal("phi", init)
    e.prepareProblem()
    return e, init


class _SolverView:
    """Solver-level calls on the solver owned by an Evolver."""

    def __init__(self, handle, shape):
        from cupss_gb300.api import Solver
        import cupss_gb300.capi as capi
        self.lib = capi.load()
        self.h = handle
        self.shape = (shape[2], shape[1], shape[0])
        self.N = shape[0] * shape[1] * shape[2]
        for name in ("time_advance", "set_kernel_timing", "kernel_report", "set_real_ptr", "get_real_ptr",
                     "snapshot_real_ptr", "synchronize", "advance", "tune_report"):
            setattr(self, name, getattr(Solver, name).__get__(self))

    @property
    def launch_count(self):
        return self.lib.cupssgb_solver_launch_count(self.h)


def device_bytes_estimate(wl):
    """Device arrays of the step, 4 B per grid point each (packed half spectra): two states
    and one dealiased channel per field (3D grids in the row-pass form keep a second one
    for the z inverse; the xy-plane pass of square planes up to 256^2 needs none), one
    product spectrum per distinct product, the real and spectral scratch arrays."""
    sx, sy, sz = wl["shape"]
    arr = 4.0 * sx * sy * sz
    nf = len(wl.get("fields", [None]))
    plane = sz > 1 and sx == sy and sx <= 256 and "fields" not in wl
    return arr * (3 * nf + (nf if sz > 1 and not plane else 0) + wl.get("products", 1) + 2)


def l2_note(dev_bytes):
    """Working set of the step against the 126 MB L2."""
    l2 = 126e6
    if dev_bytes > l2:
        return "working set about %.0f MB (states x2, dealiased copies, product spectra), larger than the " \
               "126 MB L2" % (dev_bytes / 1e6)
    return "working set about %.0f MB, within the 126 MB L2: the step runs L2-resident (timed without a " \
           "flush)" % (dev_bytes / 1e6)


def kernel_bytes(kind, wl):
    """Algorithmic bytes per launch of each kernel of the 3D/2D Cahn-Hilliard step
    (None for the multi-field workloads, which are reported against their step model).
    Spectral arrays are packed half spectra: 8 B per complex = 4 B per grid point.
    Dealiased channels (order 3, |n| <= N/4) are written only where unmasked, at the
    engine's tile granularity (W columns x line pairs)."""
    if "fields" in wl:
        return None
    sx, sy, sz = wl["shape"]
    N = sx * sy * sz
    arr = 4.0 * N
    Lx = sx // 2
    mx = sx // 4
    cols = (mx + 1) / Lx        # unmasked x columns (kx' <= sx/4) of a dealiased channel
    if sz > 1:
        W, Wi = 8, 16           # turnaround / y-inverse tile widths (column granularity of writes)
        fx = min(Lx, (mx // W + 1) * W) / Lx
        fxi = min(Lx, (mx // Wi + 1) * Wi) / Lx
        fy = min(sy // 2, sy // 4 + 1) / (sy // 2)
        rows = (2 * (sy // 4) + 1) / sy   # unmasked rows |n_y| <= sy/4 of H'
        return {"turnaround_z": 3 * arr + fx * fy * arr,     # read G'', read/write state, write H'
                "plane_pass": cols * rows * arr + arr,       # read H' (unmasked columns and rows), write G''
                "line_inv_y": fxi * fy * arr + fxi * arr,    # read H' (unmasked rows), write H
                "row_pass": cols * arr + arr,                # read H (unmasked columns), write G'
                "line_fwd_y": 2 * arr}[kind]                 # G' -> G''
    W = 16
    fx = min(Lx, (mx // W + 1) * W) / Lx
    return {"turnaround_y": 3 * arr + fx * arr, "row_pass": cols * arr + arr}[kind]


def run_cpu_baseline(wl, steps_budget_s=20.0, max_steps=None, workers=None):
    """Times the oracle restatement of the reference CPU path (float32, multithreaded
    scipy FFT, real white noise + FFT like the reference) on a bounded sample."""
    from oracle.ref_parser import System
    from oracle.ref_solver import RefSolver
    from cupss_gb300.workloads import splitmix64_uniform
    workers = workers or os.cpu_count() or 1
    sizes = [wl["shape"]]
    sx, sy, sz = wl["shape"]
    while sizes[-1][0] > 32:
        a, b, c = sizes[-1]
        sizes.append((a // 2, b // 2 if b > 1 else 1, c // 2 if c > 1 else 1))

    def build(shape):
        s = System()
        for nm, dyn in wl.get("fields", [("phi", True)]):
            s.create_field(nm, dyn)
        for k, v in wl["params"].items():
            s.add_parameter(k, v)
        for q in wl["eqs"]:
            s.add_equation(q)
        for f, a in wl["noise"]:
            s.add_noise(f, a)
        r = RefSolver(s, *shape, dt=wl["dt"], precision="f32", fft_workers=workers)
        r.set_real("phi", splitmix64_uniform(shape[0] * shape[1] * shape[2], 20261203, *wl["init"]))
        r.prepare()
        return r

    # pick the largest sample whose single step fits the budget comfortably
    chosen = None
    for shape in sizes[::-1]:
        r = build(shape)
        t0 = time.perf_counter()
        r.advance(1)
        dt1 = time.perf_counter() - t0
        chosen = (shape, r, dt1)
        if dt1 * 8 > steps_budget_s:
            break
    shape, r, dt1 = chosen
    n = max(1, int(steps_budget_s / max(dt1, 1e-6)))
    if max_steps:
        n = min(n, max_steps)
    t0 = time.perf_counter()
    r.advance(n)
    el = time.perf_counter() - t0
    pts = shape[0] * shape[1] * shape[2]
    return {"value": pts * n / el, "unit": "pt-steps/s", "cores": workers, "kind": "port",
            "sample": "%d time steps of the same system on a %dx%dx%d grid (float32 oracle restatement of "
                      "the reference CPU path, scipy.fft with %d threads), %.1f s" % (
                          n, shape[0], shape[1], shape[2], workers, el)}


def cufft_reference_schedule(wl, steps, warmup):
    """The reference GPU step restated op for op with cuFFT (torch.fft) on this GPU.

    Per time step of a dynamic field with one product term and noise, the reference
    runs (src/field.cpp:15-92, src/term.cpp:12-25): real N(0,1) noise + C2C FFT, the
    product of the dealiased real field, its C2C FFT, the prefactor multiply, the
    semi-implicit update, the dealias mask, two inverse C2C FFTs, two normalisations
    and two forward C2C FFTs.  Tables (prefactor, implicit, noise amplitude) are
    precomputed like the reference does.  Timed with CUDA events on torch's stream."""
    import torch
    sx, sy, sz = wl["shape"]
    dev = torch.device("cuda")
    N = sx * sy * sz
    pi = 3.1415926535
    def qax(n):
        i = torch.arange(n, device=dev)
        return torch.where(i < (n + 1) // 2, i, i - n).float() * (2 * pi / n)
    qz, qy, qx = torch.meshgrid(qax(sz), qax(sy), qax(sx), indexing="ij")
    q2 = qx * qx + qy * qy + qz * qz
    a, b, k, T = (wl["params"][n] for n in ("a", "b", "k", "T"))
    dt = wl["dt"]
    pre = (-b * q2).float()                                  # term prefactor table
    imp = (1.0 + dt * (a * q2 + k * q2 * q2)).float()        # 1 - dt * sum implicit
    amp = (torch.sqrt(torch.tensor(dt * 2 * T)) * torch.sqrt(q2)).float() if wl["noise"] else None
    def nk(i, n):
        return torch.where(i > n // 2, i - n, i).abs()
    kz, ky, kx = torch.meshgrid(torch.arange(sz, device=dev), torch.arange(sy, device=dev),
                                torch.arange(sx, device=dev), indexing="ij")
    mask = ((nk(kx, sx) <= sx // 4) & (nk(ky, sy) <= sy // 4) & (nk(kz, sz) <= sz // 4)).float()
    from cupss_gb300.workloads import splitmix64_uniform
    real = torch.from_numpy(splitmix64_uniform(N, 20261203, *wl["init"]).reshape(sz, sy, sx)).to(dev)
    comp = torch.fft.fftn(real.to(torch.complex64))
    real_d = torch.zeros_like(real)
    inv_n = 1.0 / N

    def step():
        nonlocal comp, real_d
        noise = torch.fft.fftn(torch.randn(sz, sy, sx, device=dev).to(torch.complex64)) if amp is not None else None
        term = torch.fft.fftn((real_d * real_d * real_d).to(torch.complex64)) * pre
        c = comp + dt * term
        if noise is not None:
            c = c + amp * noise
        c = c / imp
        cd = c * mask
        r = torch.fft.ifftn(c, norm="forward").real * inv_n
        real_d = torch.fft.ifftn(cd, norm="forward").real * inv_n
        comp = torch.fft.fftn(r.to(torch.complex64))
        torch.fft.fftn(real_d.to(torch.complex64))           # the reference's unused dealiased FFT

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    return {"ms_per_step": ms, "value": N / (ms * 1e-3), "unit": "pt-steps/s", "steps": steps,
            "what": "reference GPU step sequence restated with cuFFT C2C via torch.fft (6 FFTs + "
                    "elementwise passes per step, no device syncs), same workload and GPU"}


def bench_ensemble(args):
    """KPZ ensemble: 512 independent 2D solves (64^2..512^2, own nu, lambda, seed), 1000
    steps each, advanced together by the batched ensemble vs one after another with the
    plain evolver.  A solve = its 1000 steps + reading its h field back to the host;
    building and preparing (parsing, allocation, NVRTC, autotuning) is outside both timings."""
    import cupss_gb300 as c
    from cupss_gb300 import build as b
    from cupss_gb300.workloads import SYSTEMS, declare, kpz_ensemble
    b.build()
    sysd = SYSTEMS["kpz"]
    n = args.members
    steps = args.steps if args.steps is not None else 1000
    members = kpz_ensemble(n)
    dt = 0.005
    pts = sum(m["side"] ** 2 for m in members)

    def run(fuse, sample_clocks):
        # fuse "0": every grid size stepped by its own graphs on its own stream; "1": the
        # fused launches; None: the form prepare times as faster
        old = os.environ.get("CUPSSGB_FUSE")
        if fuse is None:
            os.environ.pop("CUPSSGB_FUSE", None)
        else:
            os.environ["CUPSSGB_FUSE"] = fuse
        try:
            t0 = time.perf_counter()
            ens = c.Ensemble()
            declare(ens, sysd)
            for m in members:
                ens.addMember(m["side"], m["side"], 1, dt=dt, seed=m["seed"], nu=m["nu"], lam=m["lam"])
            ens.prepare()
            prep = time.perf_counter() - t0
        finally:
            if old is None:
                os.environ.pop("CUPSSGB_FUSE", None)
            else:
                os.environ["CUPSSGB_FUSE"] = old
        ens.advance(3)   # captures the step graphs
        clocks = Clocks(0) if sample_clocks else None
        if clocks:
            clocks.start()
        l0 = ens.launch_count
        t0 = time.perf_counter()
        ens.advance(steps)
        res = [ens.getReal(i, "h") for i in range(n)]
        t = time.perf_counter() - t0
        r = {"seconds": t, "prepare_seconds": prep, "launches": ens.launch_count - l0, "outs": res,
             "describe": ens.describe(), "device_bytes": ens.device_bytes,
             "clocks": clocks.stop() if clocks else None}
        ens.close()
        return r

    chosen = run(None, True)
    forms = {"fused": run("1", False), "grouped": run("0", False)}
    t_ens, prep_s, launches, outs = chosen["seconds"], chosen["prepare_seconds"], chosen["launches"], chosen["outs"]
    clk, groups, dev_bytes = chosen["clocks"], chosen["describe"], chosen["device_bytes"]
    finite = [bool(np.isfinite(o).all()) for o in outs]

    def worst_vs_chosen(r):
        # both forms run the same arithmetic per member
        return max((float(np.linalg.norm(a.astype(np.float64) - b) / max(np.linalg.norm(b), 1e-30))
                    for a, b in zip(r["outs"], outs) if np.isfinite(a).all() and np.isfinite(b).all()), default=0.0)

    # the same solves with the plain evolver, one after another
    nplain = n if args.plain_members is None else min(n, args.plain_members)
    t_plain = 0.0
    pts_plain = 0
    agree, worst = 0, 0.0
    for i, m in enumerate(members[:nplain]):
        e = c.Evolver(True, m["side"], m["side"], 1, dt=dt, write_every=10 ** 9)
        for nm, dyn in sysd["fields"]:
            e.createField(nm, dyn)
        for k, v in sysd["params"].items():
            e.addParameter(k, {"nu": m["nu"], "lam": m["lam"]}.get(k, v))
        for q in sysd["eqs"]:
            e.addEquation(q)
        for f, a in sysd["noise"]:
            e.addNoise(f, a)
        e.setNoiseSeed(m["seed"])
        e.prepareProblem()
        t1 = time.perf_counter()
        e.advanceTime(steps)
        ref = e.getReal("h")
        t_plain += time.perf_counter() - t1
        e.advanceTime(3)   # the ensemble's 3 warm-up steps, so both have taken steps + 3
        ref = e.getReal("h")
        # same result as the member of the ensemble (both finite and close, or both not)
        ok = bool(np.isfinite(ref).all())
        if ok and finite[i]:
            d = float(np.linalg.norm(outs[i].astype(np.float64) - ref) / max(np.linalg.norm(ref), 1e-30))
            worst = max(worst, d)
            agree += d < 1e-5
        else:
            agree += ok == finite[i]
        pts_plain += m["side"] ** 2
        e.close()
    # per-solve time of the plain path, scaled to all members if only a sample ran
    t_plain_all = t_plain * (pts / pts_plain) if nplain < n else t_plain
    peak, peak_kind = peak_hbm()
    B_alg = 32.0
    value = n / t_ens
    line = {"metric": "ensemble solves/s", "value": value, "unit": "solves/s", "n_gpus": 1, "steps": steps,
            "warmup": 3, "ms_per_step": 1e3 * t_ens / steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: %d KPZ members, sides uniform over {64,128,256,512}, nu~U[0.5,2], "
                    "lambda~U[0,4], D=1, own Philox seeds, h0=0" % n,
            "config": {"workload": "kpz-ensemble: %d x 2D KPZ, dt=%g, %d steps, FP32" % (n, dt, steps),
                       "members": n, "total_points": pts, "groups": groups, "device_bytes": dev_bytes,
                       "l2": "working set %.1f GB, larger than L2" % (dev_bytes / 1e9)},
            "pt_steps_per_s": pts * steps / t_ens,
            "roofline": {"bound": "hbm", "achieved": B_alg * pts * steps / t_ens / 1e9, "peak": peak,
                         "unit": "GB/s", "frac": B_alg * pts * steps / t_ens / 1e9 / peak,
                         "peak_source": peak_kind, "model": "B_alg = 32 B/pt-step (KPZ) x pt-steps/s"},
            "plain_sequential": {"value": n / t_plain_all, "unit": "solves/s", "seconds": t_plain_all,
                                 "members_run": nplain, "pt_steps_per_s": pts_plain * steps / t_plain},
            "speedup_vs_plain": t_plain_all / t_ens, "seconds": t_ens, "prepare_seconds": prep_s,
            "gpu_launches": launches, "clocks": clk,
            "form": (groups.get("fused") or {}).get("form", "grouped"),
            "forms": {k: {"value": n / r["seconds"], "unit": "solves/s", "seconds": r["seconds"],
                          "gpu_launches": r["launches"], "worst_rel_l2_vs_chosen": worst_vs_chosen(r)}
                      for k, r in forms.items()},
            "forms_what": "the same ensemble forced into each form (CUPSSGB_FUSE=1: one launch per kernel "
                          "over every grid size; =0: each grid size's own graphs on its own stream); the "
                          "line's value is the form prepare timed as faster",
            "accuracy": {"finite_members": int(sum(finite)), "members_compared": nplain,
                         "members_equal_to_plain": int(agree), "worst_rel_l2_vs_plain": worst,
                         "note": "members that diverge (large lambda^2 D / nu^3) do so identically in the plain "
                                 "solver: the semi-implicit scheme of the reference is unstable there"}}
    return line


def bench_served(args):
    """Served Poisson stream (EW, KPZ, CH 2D, CH 3D requests of mixed grids and step
    counts) through the continuous-batching server vs the same requests run one after
    another with the plain evolver (a FIFO single-solve server with the same arrival
    times).  Latency = completion - arrival.  Pools (batched) and update programs
    (both paths) are compiled before the stream starts."""
    import cupss_gb300 as c
    from cupss_gb300 import build as b
    from cupss_gb300.workloads import SYSTEMS, initial_fields, served_stream
    b.build()
    steps_range = getattr(args, "steps_range", (1e3, 1e5))
    reqs = served_stream(args.requests, args.rate, steps_range=steps_range)
    keys = sorted({(r["system"], r["shape"], r["dt"]) for r in reqs})
    srv = c.Server(hbm_budget=args.hbm_budget, max_slots=args.max_slots, max_chunk=args.max_chunk)
    sids = {k: srv.addSystem(SYSTEMS[k]) for k in ("ew", "kpz", "ch")}
    t0 = time.perf_counter()
    for sysname, shape, dt in keys:
        srv.warm(sids[sysname], shape, dt)
    warm_s = time.perf_counter() - t0

    def plain_solve(r, steps=None):
        sd = SYSTEMS[r["system"]]
        e = c.Evolver(True, *r["shape"], dt=r["dt"], write_every=10 ** 9)
        for nm, dyn in sd["fields"]:
            e.createField(nm, dyn)
        for k, v in sd["params"].items():
            e.addParameter(k, r["params"].get(k, v))
        for q in sd["eqs"]:
            e.addEquation(q)
        for f, a in sd["noise"]:
            e.addNoise(f, a)
        e.setNoiseSeed(r["seed"])
        for nm, arr in initial_fields(r).items():
            e.setReal(nm, arr)
        e.prepareProblem()
        t_adv = time.perf_counter()
        e.advanceTime(steps or r["steps"])
        out = e.getReal(sd["out"])
        t_adv = time.perf_counter() - t_adv
        e.close()
        return out, t_adv

    for sysname, shape, dt in keys:   # compile the plain path's programs
        plain_solve(dict(system=sysname, shape=shape, dt=dt, params={}, seed=0, init_seed=0), steps=1)


    clocks = Clocks(0)
    clocks.start()
    ids = []
    start = time.perf_counter()
    for r in reqs:
        delay = start + r["arrival"] - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        ids.append(srv.submit(sids[r["system"]], r["shape"], r["dt"], r["steps"], seed=r["seed"],
                              params=r["params"], init=initial_fields(r)))
    for rid in ids:
        srv.wait(rid)
    clk = clocks.stop()
    times = [srv.times(rid) for rid in ids]
    t_first = min(t[0] for t in times)
    makespan = max(t[2] for t in times) - t_first
    lat = np.array([t[2] - t[0] for t in times])
    served = [srv.result(rid) for rid in ids]
    stats = srv.stats()
    srv.close()

    # plain: service time of each request alone, FIFO in arrival order
    svc, adv = [], []
    agree = 0
    for r, got in zip(reqs, served):
        t1 = time.perf_counter()
        ref, t_adv = plain_solve(r)
        svc.append(time.perf_counter() - t1)
        adv.append(t_adv)
        fa, fb = bool(np.isfinite(ref).all()), bool(np.isfinite(got).all())
        if fa and fb:
            d = np.linalg.norm(got.astype(np.float64) - ref) / max(np.linalg.norm(ref), 1e-30)
            agree += d < 1e-6
        else:
            agree += fa == fb
    done, plat = 0.0, []
    for r, s_i in zip(reqs, svc):
        done = max(done, r["arrival"]) + s_i
        plat.append(done - r["arrival"])
    plat = np.array(plat)
    work = float(sum(np.prod(r["shape"]) * r["steps"] for r in reqs))
    line = {"metric": "served solves/s", "value": len(reqs) / makespan, "unit": "solves/s", "n_gpus": 1,
            "steps": None, "warmup": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic Poisson stream, seed 20261203",
            "config": {"workload": "served: %d requests, Poisson rate %.2f/s, {EW, KPZ, CH} 2D 64^2..1024^2 (incl. 96^2, 192^2), "
                                   "CH 3D 64^3..192^3, steps log-U[%g,%g]" % (len(reqs), args.rate, *steps_range),
                       "requests": len(reqs), "rate_per_s": args.rate, "hbm_budget": args.hbm_budget,
                       "max_slots": args.max_slots, "max_chunk": args.max_chunk, "pool_keys": len(keys),
                       "total_pt_steps": work},
            "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                          "max": float(lat.max())},
            "pt_steps_per_s": work / makespan, "makespan_s": makespan,
            "plain_sequential": {"value": len(reqs) / (done - reqs[0]["arrival"]), "unit": "solves/s",
                                 "latency_s": {"p50": float(np.percentile(plat, 50)),
                                               "p99": float(np.percentile(plat, 99))},
                                 "service_s_total": float(sum(svc)),
                                 "what": "each request alone: evolver create + prepare + advance + getReal, "
                                         "FIFO in arrival order (programs precompiled)"},
            "speedup_vs_plain": (done - reqs[0]["arrival"]) / makespan,
            # no schedule ends before a request's arrival plus its steps run alone (advance +
            # read-back with the GPU to itself): the ratio any server could reach on this stream
            "bound": {"latest_alone_end_s": max(r["arrival"] + a for r, a in zip(reqs, adv)),
                      "ratio_upper_bound": (done - reqs[0]["arrival"]) /
                                           max(r["arrival"] + a for r, a in zip(reqs, adv)),
                      "alone_s_total": float(sum(adv)),
                      # requests of >= 2^20 grid points keep the whole GPU busy alone: their
                      # alone times add up even when they share it
                      "large_alone_s_total": float(sum(a for r, a in zip(reqs, adv)
                                                       if np.prod(r["shape"]) >= (1 << 20))),
                      "what": "latest (arrival + alone advance time) over the requests; ratio_upper_bound = "
                              "plain FIFO time / that; large_alone_s_total: the alone advance time of the "
                              "requests of >= 2^20 grid points"},
            "accuracy": {"requests_equal_to_plain": int(agree), "tolerance": "rel L2 1e-6"},
            "server_stats": stats, "warm_s": warm_s, "clocks": clk}
    # the requests that finished last: (system, grid, steps, admitted after, latency) in s
    order = np.argsort([t[2] for t in times])[::-1][:6]
    line["last_finished"] = [[reqs[i]["system"], list(reqs[i]["shape"]), int(reqs[i]["steps"]),
                              round(times[i][1] - times[i][0], 3), round(float(lat[i]), 3)] for i in order]
    return line


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def reduce_max(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=None)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="ch3d-256", choices=sorted(WORKLOADS) + ["kpz-ensemble", "served"])
    ap.add_argument("--requests", type=int, default=64)
    ap.add_argument("--rate", type=float, default=2.0)
    ap.add_argument("--hbm-budget", type=float, default=150e9)
    ap.add_argument("--max-slots", type=int, default=32)
    ap.add_argument("--max-chunk", type=int, default=256)
    ap.add_argument("--members", type=int, default=512)
    ap.add_argument("--plain-members", type=int, default=None)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=50)
    ap.add_argument("--profile-steps", type=int, default=100)
    ap.add_argument("--no-cufft-ref", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the reduced ensemble and served lines")
    args = ap.parse_args()
    if args.workload == "kpz-ensemble":
        print(json.dumps(bench_ensemble(args)), flush=True)
        return
    if args.workload == "served":
        print(json.dumps(bench_served(args)), flush=True)
        return
    wl = WORKLOADS[args.workload]
    K = args.steps if args.steps is not None else wl["steps"]
    W = args.warmup if args.warmup is not None else wl["warmup"]
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    sx, sy, sz = wl["shape"]
    N = sx * sy * sz
    system = "model H (6 fields)" if "fields" in wl else "Cahn-Hilliard"
    noise = ""
    if wl["noise"]:
        noise = " + conserved noise T=0.01" if "q^2" in wl["noise"][0][1] else " + noise T=%g" % wl["params"]["T"]
    cfg = {"workload": "%s: %dx%dx%d %s%s, dt=%g, FP32" % (args.workload, sx, sy, sz, system, noise, wl["dt"]),
        "grid": [sx, sy, sz], "equation": wl["eqs"][0], "noise": wl["noise"][0][1] if wl["noise"] else None,
        "full_solve_steps": wl["solve_steps"], "l2": l2_note(device_bytes_estimate(wl)),
        "parallelism": "replicas" if ws > 1 else "single GPU"}

    if args.impl == "reference":
        if rank != 0:
            return
        cb = run_cpu_baseline(wl, steps_budget_s=max(10.0, min(150.0, 2.0 * (K + W))), max_steps=K + W)
        line = {"metric": "grid-pt-steps/s", "value": cb["value"], "unit": "pt-steps/s", "n_gpus": ws,
                "steps": K, "warmup": W, "ms_per_step": 1e3 * N / cb["value"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": cfg,
                "impl": "reference", "cpu_baseline": cb,
                "e2e": {"value": cb["value"], "unit": "pt-steps/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    import cupss_gb300 as c
    from cupss_gb300 import build as b
    b.build()
    c.api.set_device(local)
    e, init = make_evolver(wl)
    sv = _SolverView(c.load().cupssgb_evolver_solver(e.h), wl["shape"])
    cfg["tune"] = sv.tune_report()   # launch shapes chosen at prepare (timed or from the cache)
    # warmup
    sv.advance(W)
    sv.synchronize()
    barrier(ws)
    clocks = Clocks(local)
    clocks.start()
    l0 = sv.launch_count
    ms = sv.time_advance(K)
    launches = sv.launch_count - l0
    barrier(ws)
    clk = clocks.stop()
    ms_max = reduce_max(ms, ws)
    value = ws * N * K / (ms_max * 1e-3)

    # per-kernel timing pass (CUDA events around every launch on the solver's stream)
    sv.set_kernel_timing(True)
    sv.advance(args.profile_steps)
    rep = sv.kernel_report()
    sv.set_kernel_timing(False)
    peak, peak_kind = peak_hbm()
    per = {}
    for kind, v in rep.items():
        avg = v["ms"] / v["launches"]
        byts = kernel_bytes(kind, wl)
        per[kind] = {"launches": v["launches"], "avg_us": 1e3 * avg, "share": None,
                     "alg_bytes": byts, "GBps": None if byts is None else byts / (avg * 1e-3) / 1e9}
    tot = sum(v["ms"] for v in rep.values())
    for kind in per:
        per[kind]["share"] = rep[kind]["ms"] / tot
    dom = max(per, key=lambda k: rep[k]["ms"])
    d = per[dom]
    B_alg = wl.get("B_alg", 24.0)
    roof = {"bound": "hbm", "kernel": dom, "achieved": d["GBps"], "peak": peak, "unit": "GB/s",
            "frac": None if d["GBps"] is None else d["GBps"] / peak,
            "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
            "traffic": None, "alg_bytes_per_launch": d["alg_bytes"], "avg_launch_us": d["avg_us"],
            "kernels": per,
            "step_model": {"B_alg_per_pt_step": B_alg,
                           "achieved_GBps": B_alg * value / ws / 1e9,
                           "frac": B_alg * value / ws / 1e9 / peak}}
    prof_file = os.path.join(ROOT, "profiles", "ncu_traffic_%s.json" % args.workload)
    if os.path.exists(prof_file):
        try:
            with open(prof_file) as fh:
                tr = json.load(fh).get(dom)
            if tr:
                roof["traffic"] = tr
        except Exception:
            pass

    e2e = None
    if not args.no_e2e:
        # host-buffer path through the C-ABI, every step: the step's input field copied in
        # from page-locked host memory (cupssgb_solver_set_real: an input stream), one step,
        # and the result read out into page-locked host memory
        # (cupssgb_solver_snapshot_real: an output stream).  Inputs alternate between two
        # fields, outputs between two buffers, so the copy in of step k+1 and the copy out
        # of step k overlap each other and the steps; the timed region ends when the last
        # result is in host memory.
        init2 = c.splitmix64_uniform(N, 20261204, *wl["init"])
        pins = [c.api.PinnedBuffer(N) for _ in range(4)]
        pins[0].array[:] = init
        pins[1].array[:] = init2
        sv.synchronize()
        barrier(ws)
        t0 = time.perf_counter()
        for k in range(args.e2e_steps):
            sv.set_real_ptr(0, pins[k % 2].ptr)
            sv.advance(1)
            sv.snapshot_real_ptr(0, pins[2 + k % 2].ptr)
        sv.synchronize()
        el = reduce_max(time.perf_counter() - t0, ws)
        outs_ok = all(bool(np.isfinite(pins[j].array).all()) for j in (2, 3))
        # the same with each step's result read back (blocking) before the next input,
        # which is that result: nothing overlaps
        pin_in, pin_out = pins[0], pins[1]
        pin_in.array[:] = init
        sv.synchronize()
        barrier(ws)
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            sv.set_real_ptr(0, pin_in.ptr)
            sv.advance(1)
            sv.get_real_ptr(0, pin_out.ptr)
            pin_in, pin_out = pin_out, pin_in
        el_chain = reduce_max(time.perf_counter() - t0, ws)
        e2e = {"value": ws * N * args.e2e_steps / el, "unit": "pt-steps/s", "h2d_bytes_per_step": 4 * N,
               "d2h_bytes_per_step": 4 * N, "steps": args.e2e_steps, "finite": outs_ok,
               "path": "per step: cupssgb_solver_set_real (page-locked host input, copied on the input "
                       "stream) + cupssgb_solver_advance(1) + cupssgb_solver_snapshot_real (page-locked "
                       "host output, copied on the output stream); inputs alternate between two fields",
               "chained": {"value": ws * N * args.e2e_steps / el_chain, "unit": "pt-steps/s",
                           "path": "per step: set_real + advance(1) + get_real (blocking), the result being "
                                   "the next step's input"}}
        for pb in pins:
            pb.close()
        # a whole solve through the reference-facing evolver C-ABI, host in / host out
        t0 = time.perf_counter()
        e2 = make_evolver(wl)[0]
        e2.advanceTime(wl["solve_steps"])
        out = e2.getReal("phi")
        el2 = time.perf_counter() - t0
        e2e["full_solve"] = {"seconds": el2, "steps": wl["solve_steps"],
                             "value": N * wl["solve_steps"] / el2,
                             "path": "cupssgb_evolver_create .. prepare .. advance(%d) .. get_real" % wl["solve_steps"],
                             "finite": bool(np.isfinite(out).all())}
        e2.close()

    cufft_ref = None
    if not args.no_cufft_ref and wl["shape"][2] > 1:
        try:
            cufft_ref = cufft_reference_schedule(wl, steps=50, warmup=5)
        except Exception as ex:   # torch missing or out of memory: report why
            cufft_ref = {"unavailable": repr(ex)[:200]}

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        cpu = run_cpu_baseline(wl)

    # the batched and served forms, reduced so that the default run stays short: 64 KPZ
    # members for 200 steps against their plain solves, and 24 served requests of 1e2..1e4
    # steps (a hundredth of the full stream's) arriving at 64 requests/s, which saturates
    # both arms, against the plain FIFO
    extra = {}
    if rank == 0 and ws == 1 and not args.no_extra:
        for key, fn, over in (("ensemble_reduced", bench_ensemble,
                               dict(members=64, steps=200, plain_members=None)),
                              ("served_reduced", bench_served,
                               dict(requests=24, rate=64.0, steps_range=(1e2, 1e4)))):
            try:
                sub = argparse.Namespace(**vars(args))
                for k2, v2 in over.items():
                    setattr(sub, k2, v2)
                r = fn(sub)
                extra[key] = {k2: r.get(k2) for k2 in ("metric", "value", "unit", "speedup_vs_plain", "latency_s",
                                                        "plain_sequential", "accuracy", "config", "pt_steps_per_s",
                                                        "gpu_launches", "seconds", "makespan_s")
                              if k2 in r}
            except Exception as ex:   # report why, keep the headline line
                extra[key] = {"unavailable": repr(ex)[:300]}

    if rank == 0:
        line = {"metric": "grid-pt-steps/s", "value": value, "unit": "pt-steps/s", "n_gpus": ws, "steps": K,
                "warmup": W, "ms_per_step": ms_max / K, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic: SplitMix64 seed 20261203 uniform initial "
                "field, Fourier-space Philox noise seed 42", "config": cfg, "roofline": roof,
                "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": clk,
                "cufft_reference_schedule": cufft_ref, **extra}
        print(json.dumps(line), flush=True)
    e.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
