"""Oracle restatement of cuPSS's pseudospectral time step (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke`` and the CPU-baseline leg of ``bench.py``
may import this module.  It is the checker, never the thing measured or shipped.

It restates, with numpy full complex (C2C) FFTs in float64 or float32, the exact
sequence of operations of the reference GPU path:

* step driver ``evolver::advanceTime``             src/evolver.cpp:199-226
  (all non-dynamic updateTerms, then their setRHS, then the same for dynamic fields)
* ``field::updateTerms``                           src/field.cpp:15-23
* ``term::update`` (copyComp / computeProduct+FFT / applyPres_vector_pre)
                                                   src/term.cpp:12-25, term_kernels.cu:34-70,221-240
* ``term::precomputePrefactors`` (P(q) table, i-parity, sign)   src/term_init.cpp:135-200
* ``term::prepareDevice`` (needsaliasing, aliasing_order)       src/term_init.cpp:108-133
* ``field::setRHS``                                src/field.cpp:25-92
* ``setDynamic_k``                                 src/field_kernels.cu:199-227
* ``setNotDynamic_k``                              src/field_kernels.cu:130-197
* ``dealias_k``                                    src/field_kernels.cu:229-256
* ``normalize_k``                                  src/field_kernels.cu:115-128
* ``field::precalculateImplicit``                  src/field_init.cpp:237-284
* ``evolver::prepareProblem`` ordering (S1: dealiased copies stay zero until a
  field's first setRHS)                            src/evolver.cpp:81-126
* ``evolver::initializeDroplet``                   src/initializers.cpp:142-177

Noise: the reference draws real white N(0,1) with cuRAND (time-seeded) and
FFTs it.  The oracle instead takes the Fourier-space noise realisation from a
provider callable so that it can be fed exactly the field the CUDA engine
generates (see ``oracle/philox.py``); with ``noise=None`` it draws real white
noise and FFTs it like the reference.
"""
from __future__ import annotations

import numpy as np

from .ref_parser import System, Pres

PI_F = np.float32(3.1415926535)     # inc/cupss/defines.h:57


def q_axis(n: int, step: np.float32, dtype) -> np.ndarray:
    """q = (i < (n+1)/2 ? i : i - n) * stepq   (src/field_init.cpp:248-250)."""
    i = np.arange(n)
    m = np.where(i < (n + 1) // 2, i, i - n).astype(np.float32)
    return (m * np.float32(step)).astype(dtype)


class RefSolver:
    """State + step of a cuPSS system, restated.  Arrays are indexed [k][j][i]
    (z, y, x) so that the flat C order equals the reference index k*sx*sy+j*sx+i."""

    def __init__(self, system: System, sx, sy=1, sz=1, dx=1.0, dy=1.0, dz=1.0, dt=0.01,
                 precision="f64", noise=None, fft_workers=None):
        self.sys = system
        self.sx, self.sy, self.sz = int(sx), int(sy), int(sz)
        self.dt = np.float32(dt)
        self.rdt = np.float64 if precision == "f64" else np.float32
        self.cdt = np.complex128 if precision == "f64" else np.complex64
        self.shape = (self.sz, self.sy, self.sx)
        self.N = self.sx * self.sy * self.sz
        f32 = np.float32
        dx, dy, dz = f32(dx), f32(dy), f32(dz)
        # evolver::createField always uses the 3-size field constructor with dy=dz=1
        # for lower dimensions (src/evolver.cpp:184, src/field_init.cpp:207-213)
        self.stepq = (f32(2.0) * PI_F / (dx * f32(self.sx)),
                      f32(2.0) * PI_F / (dy * f32(self.sy)),
                      f32(2.0) * PI_F / (dz * f32(self.sz)))
        self.noise_provider = noise
        self.workers = fft_workers
        self.names = list(system.order)
        self.index = {n: i for i, n in enumerate(self.names)}
        F = len(self.names)
        self.real = [np.zeros(self.shape, self.rdt) for _ in range(F)]
        self.comp = [np.zeros(self.shape, self.cdt) for _ in range(F)]
        self.real_dealiased = [np.zeros(self.shape, self.rdt) for _ in range(F)]
        self.step_count = 0
        self.time = 0.0
        self.rng = np.random.default_rng(12345)
        self.callbacks = {}          # name -> fn(real ndarray) applied after normalize
        self.fourier_callbacks = {}  # name -> fn(complex ndarray) applied after the update
        self.prepared = False

    # ---- FFT helpers (unnormalised, like cuFFT C2C) ------------------------------------------
    def _fft(self, a):
        a = np.asarray(a, self.cdt)
        if self.workers:
            import scipy.fft as sf
            return sf.fftn(a, workers=self.workers).astype(self.cdt, copy=False)
        return np.fft.fftn(a).astype(self.cdt, copy=False)

    def _ifft_unnorm(self, a):
        if self.workers:
            import scipy.fft as sf
            return sf.ifftn(a, norm="forward", workers=self.workers).astype(self.cdt, copy=False)
        return np.fft.ifftn(a, norm="forward").astype(self.cdt, copy=False)

    # ---- tables ---------------------------------------------------------------------------------
    def _qgrids(self):
        qx = q_axis(self.sx, self.stepq[0], np.float32)
        qy = q_axis(self.sy, self.stepq[1], np.float32)
        qz = q_axis(self.sz, self.stepq[2], np.float32)
        QZ, QY, QX = np.meshgrid(qz, qy, qx, indexing="ij")
        q2 = (QX * QX + QY * QY + QZ * QZ).astype(np.float32)
        return QX, QY, QZ, q2

    def _term_table(self, pres):
        """precomputePrefactors (src/term_init.cpp:135-200): float table + i flag."""
        QX, QY, QZ, q2 = self._qgrids()
        total = np.zeros(self.shape, np.float32)
        s = (pres[0].iqx + pres[0].iqy + pres[0].iqz) % 2
        idx0 = np.zeros(self.shape, bool)
        idx0.flat[0] = True
        for p in pres:
            u = p.iqx + p.iqy + p.iqz
            half = int((u - s) / 2)                   # C truncating division
            negate = -2 * (half % 2 if half >= 0 else -((-half) % 2)) + 1
            v = np.full(self.shape, np.float32(p.pre) * np.float32(negate), np.float64)
            if p.q2n > 0:
                v = (v * np.power(q2.astype(np.float64), p.q2n)).astype(np.float32).astype(np.float64)
            if p.iqx > 0:
                v = (v * np.power(QX.astype(np.float64), p.iqx)).astype(np.float32).astype(np.float64)
            if p.iqy > 0:
                v = (v * np.power(QY.astype(np.float64), p.iqy)).astype(np.float32).astype(np.float64)
            if p.iqz > 0:
                v = (v * np.power(QZ.astype(np.float64), p.iqz)).astype(np.float32).astype(np.float64)
            if p.invq > 0:
                with np.errstate(divide="ignore"):
                    iq = np.where(idx0, np.float32(0), np.float32(1) / np.sqrt(q2)).astype(np.float32)
                v = (v * np.power(iq.astype(np.float64), p.invq)).astype(np.float32).astype(np.float64)
            total = (total + v.astype(np.float32)).astype(np.float32)
        return total, s

    def _implicit_tables(self, fld):
        """precalculateImplicit (src/field_init.cpp:237-284)."""
        QX, QY, QZ, q2 = self._qgrids()
        f32 = np.float32
        dt = self.dt
        sx, sy, sz = self.sx, self.sy, self.sz
        # dx recomputed from stepq in double, stored as float (field_init.cpp:239-241)
        ddx = f32(2.0 * float(PI_F) / float(self.stepq[0] * f32(sx)))
        ddy = f32(2.0 * float(PI_F) / float(self.stepq[1] * f32(sy)))
        ddz = f32(2.0 * float(PI_F) / float(self.stepq[2] * f32(sz)))
        kk, jj, ii = np.meshgrid(np.arange(sz), np.arange(sy), np.arange(sx), indexing="ij")
        imp = np.full(self.shape, f32(1.0) if fld.dynamic else f32(0.0), np.float32)
        for p in fld.implicit:
            v = np.full(self.shape, f32(p.pre), np.float32)
            if p.q2n != 0:
                v = (v.astype(np.float64) * np.power(q2.astype(np.float64), p.q2n)).astype(np.float32)
            if p.invq != 0:
                with np.errstate(divide="ignore"):
                    iq = np.where((ii > 0) | (jj > 0), f32(1.0) / np.sqrt(q2), f32(0.0)).astype(np.float32)
                v = (v.astype(np.float64) * np.power(iq.astype(np.float64), p.invq)).astype(np.float32)
            if fld.dynamic:
                imp = (imp - dt * v).astype(np.float32)
            else:
                imp = (imp + v).astype(np.float32)
        a = fld.noise
        base = f32(np.sqrt(float(f32(dt / (ddx * ddy * ddz) * f32(a.pre))))) if fld.noisy else f32(0.0)
        noise = np.full(self.shape, base, np.float32)
        if fld.noisy and a.q2n != 0:
            noise = (noise.astype(np.float64) * np.sqrt(np.power(q2.astype(np.float64), a.q2n))).astype(np.float32)
        if fld.noisy and a.invq != 0:
            idx = np.arange(self.N).reshape(self.shape)
            with np.errstate(divide="ignore"):
                iq = np.where(idx > 0, f32(1.0) / np.sqrt(q2), f32(0.0)).astype(np.float32)
            noise = (noise.astype(np.float64) * np.sqrt(np.power(iq.astype(np.float64), a.invq))).astype(np.float32)
        return imp, noise

    def _mask(self, order):
        """dealias_k (src/field_kernels.cu:229-256): cube mask, integer division."""
        sx, sy, sz = self.sx, self.sy, self.sz
        def n_of(i, n):
            return np.where(i > n // 2, i - n, i)
        kk, jj, ii = np.meshgrid(np.arange(sz), np.arange(sy), np.arange(sx), indexing="ij")
        out = ((np.abs(n_of(ii, sx)) > sx // (order + 1)) |
               (np.abs(n_of(jj, sy)) > sy // (order + 1)) |
               (np.abs(n_of(kk, sz)) > sz // (order + 1)))
        return ~out

    # ---- problem setup ------------------------------------------------------------------------
    def set_real(self, name, arr):
        self.real[self.index[name]][...] = np.asarray(arr, self.rdt).reshape(self.shape)

    def prepare(self):
        """prepareProblem (src/evolver.cpp:81-126)."""
        F = len(self.names)
        for f in range(F):
            self.comp[f] = self._fft(self.real[f])
        self.needs_alias = [False] * F
        self.alias_order = [1] * F
        self.term_tables = []
        for f, n in enumerate(self.names):
            fld = self.sys.fields[n]
            tabs = []
            for t in fld.terms:
                if len(t.product) >= 2:
                    for pn in t.product:
                        pi = self.index[pn]
                        self.needs_alias[pi] = True
                        if self.alias_order[pi] < len(t.product):
                            self.alias_order[pi] = len(t.product)
                tabs.append(self._term_table(t.pres))
            self.term_tables.append(tabs)
        self.imp = []
        self.noise_amp = []
        for n in self.names:
            a, b = self._implicit_tables(self.sys.fields[n])
            self.imp.append(a)
            self.noise_amp.append(b)
        self.masks = [self._mask(o) for o in self.alias_order]
        self.prepared = True

    def refresh_tables(self):
        """Re-derive tables after a parameter update (field::updateParameter)."""
        self.prepare_tables_only()

    def prepare_tables_only(self):
        comp = [c.copy() for c in self.comp]
        self.prepare()
        self.comp = comp

    # ---- step ---------------------------------------------------------------------------------------
    def _noise(self, f):
        if self.noise_provider is not None:
            return np.asarray(self.noise_provider(self.step_count, f), self.cdt).reshape(self.shape)
        w = self.rng.standard_normal(self.shape).astype(self.rdt)
        return self._fft(w)

    def _update_terms(self, f):
        fld = self.sys.fields[self.names[f]]
        noise = self._noise(f) if fld.noisy else None
        tcs = []
        for t, (tab, s) in zip(fld.terms, self.term_tables[f]):
            if len(t.product) == 1:
                tc = self.comp[self.index[t.product[0]]].copy()
            else:
                prod = np.ones(self.shape, self.rdt)
                for pn in t.product:
                    prod = (prod * self.real_dealiased[self.index[pn]]).astype(self.rdt)
                tc = self._fft(prod)
            tc = (tc * tab.astype(self.rdt)).astype(self.cdt)
            if s:
                tc = (1j * tc).astype(self.cdt)
            tcs.append(tc)
        return tcs, noise

    def _set_rhs(self, f, tcs, noise):
        fld = self.sys.fields[self.names[f]]
        dt = self.rdt(self.dt)
        c = self.comp[f]
        if fld.dynamic:
            for tc in tcs:
                c = (c + dt * tc).astype(self.cdt)
            if fld.noisy:
                c = (c + self.noise_amp[f].astype(self.rdt) * noise).astype(self.cdt)
            if fld.implicit:
                c = (c / self.imp[f].astype(self.rdt)).astype(self.cdt)
        else:
            if tcs:
                c = tcs[0].copy()
                for tc in tcs[1:]:
                    c = (c + tc).astype(self.cdt)
            if fld.noisy:
                sdt = self.rdt(1.0) / np.sqrt(dt)
                add = (sdt * self.noise_amp[f].astype(self.rdt) * noise).astype(self.cdt)
                c = add if not tcs else (c + add).astype(self.cdt)
            if fld.implicit:
                QX, QY, QZ, q2 = self._qgrids()
                fac = np.zeros(self.shape, np.float32)
                idx0 = np.zeros(self.shape, bool)
                idx0.flat[0] = True
                for p in fld.implicit:
                    v = np.full(self.shape, np.float32(p.pre), np.float32)
                    if p.q2n != 0:
                        v = (v * np.power(q2, np.float32(p.q2n))).astype(np.float32)
                    if p.invq != 0:
                        with np.errstate(divide="ignore"):
                            iq = np.where(idx0, np.float32(0), np.float32(1) / np.sqrt(q2)).astype(np.float32)
                        v = (v * np.power(iq, np.float32(p.invq))).astype(np.float32)
                    fac = (fac + v).astype(np.float32)
                fac.flat[0] = 1.0            # index 0 is skipped (field_kernels.cu:167)
                c = (c / fac.astype(self.rdt)).astype(self.cdt)
        fcb = self.fourier_callbacks.get(self.names[f])
        if fcb is not None:                 # callbackFourier (src/field.cpp:48-57)
            c = np.asarray(fcb(c), self.cdt)
        self.comp[f] = c
        if self.needs_alias[f]:
            cd = np.where(self.masks[f], c, 0).astype(self.cdt)
        invN = self.rdt(1.0) / self.rdt(self.N)
        r = (self._ifft_unnorm(c).real * invN).astype(self.rdt)
        if self.needs_alias[f]:
            rd = (self._ifft_unnorm(cd).real * invN).astype(self.rdt)
        cb = self.callbacks.get(self.names[f])
        if cb is not None:
            r = np.asarray(cb(r), self.rdt)
            if self.needs_alias[f]:
                rd = np.asarray(cb(rd), self.rdt)
        self.real[f] = r
        if self.needs_alias[f]:
            self.real_dealiased[f] = rd
        self.comp[f] = self._fft(r)

    def advance(self, n=1):
        assert self.prepared
        F = len(self.names)
        for _ in range(n):
            for dyn in (False, True):
                idx = [f for f in range(F) if self.sys.fields[self.names[f]].dynamic == dyn]
                pending = [self._update_terms(f) for f in idx]
                for f, (tcs, noise) in zip(idx, pending):
                    self._set_rhs(f, tcs, noise)
            self.step_count += 1
            self.time += float(self.dt)

    # ---- readout ------------------------------------------------------------------------------------
    def real_field(self, name):
        return self.real[self.index[name]]

    def fourier_field(self, name):
        return self.comp[self.index[name]]


def droplet(shape_xyz, val1, val2, radius, xi, px, py, pz):
    """evolver::initializeDroplet (src/initializers.cpp:142-177) in float."""
    sx, sy, sz = shape_xyz
    x_, y_, z_ = px % sx, py % sy, pz % sz
    kk, jj, ii = np.meshgrid(np.arange(sz), np.arange(sy), np.arange(sx), indexing="ij")
    xd = (ii - x_).astype(np.float32)
    yd = (jj - y_).astype(np.float32)
    zd = (kk - z_).astype(np.float32)
    rc = np.sqrt(xd * xd + yd * yd + zd * zd).astype(np.float32)
    dv = np.float64(np.float32(val2) - np.float32(val1))
    arg = (rc - np.float32(radius)).astype(np.float64) / (np.sqrt(2.0) * np.float64(np.float32(xi)))
    v = np.float64(np.float32(val1)) + dv * 0.5 * (1.0 + np.tanh(arg))
    return v.astype(np.float32)
