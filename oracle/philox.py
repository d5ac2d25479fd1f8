"""Oracle restatement of the Fourier-space noise stream (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke`` and the CPU-baseline leg of ``bench.py``
may import this module.

The reference (src/field.cpp:300-316, src/field_init.cpp:130-137) draws real
white N(0,1) noise with cuRAND's Philox4x32-10 generator seeded from
``time(NULL)`` and forward-FFTs it (unnormalised).  The DFT of i.i.d. N(0,1)
real noise is a Hermitian complex Gaussian field: each independent pair
(k, -k) has Re and Im ~ N(0, N/2); self-conjugate bins are real ~ N(0, N).
The GB300 engine generates that field directly in Fourier space with a
counter-based Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random
numbers: as easy as 1, 2, 3", SC'11) and the Box-Muller transform.  This module
restates the same definition in numpy so tests can feed the oracle the exact
realisation the GPU used:

  key      = (seed mod 2^32, seed >> 32),  counter = (c, step, field_id, 0)
  normals  = Box-Muller on a pair of words (a, b):
             u1 = ((a >> 8) + 1) 2^-24 in (0,1],  u2 = (b >> 8) 2^-24 in [0,1),
             g1 + i g2 = sqrt(-2 ln u1) exp(2 pi i (u2 - 1/2))
  modes 0 < kx < sx/2: the line-axis coordinate t (z in 3D, y in 2D, none in 1D)
             is folded to t mod Lt/2; c = (kz*sy + ky)*sx + kx with t folded; words
             (0,1) give the mode with t < Lt/2, words (2,3) the mode at t + Lt/2;
             value sqrt(N/2) (g1 + i g2);
  modes on the kx = 0 and kx = sx/2 planes: c = smaller linear index of the pair
             (k, -k), words (0,1); value sqrt(N/2)(g1 + i g2) at that member, the
             conjugate at the other; self-conjugate modes sqrt(N) g1;
  modes kx > sx/2: conjugate of the partner (sx - kx, -ky, -kz).
"""
from __future__ import annotations

import ctypes
import threading

import numpy as np

M0 = np.uint64(0xD2511F53)
M1 = np.uint64(0xCD9E8D57)
W0 = np.uint32(0x9E3779B9)
W1 = np.uint32(0xBB67AE85)
MASK32 = np.uint64(0xFFFFFFFF)


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Vectorised Philox4x32 with 10 rounds; all arguments uint32 arrays/scalars."""
    c0 = np.asarray(c0, np.uint32)
    c1 = np.asarray(c1, np.uint32)
    c2 = np.asarray(c2, np.uint32)
    c3 = np.asarray(c3, np.uint32)
    k0 = np.uint32(k0)
    k1 = np.uint32(k1)
    with np.errstate(over="ignore"):
        for r in range(10):
            p0 = c0.astype(np.uint64) * M0
            p1 = c2.astype(np.uint64) * M1
            hi0 = (p0 >> np.uint64(32)).astype(np.uint32)
            lo0 = (p0 & MASK32).astype(np.uint32)
            hi1 = (p1 >> np.uint64(32)).astype(np.uint32)
            lo1 = (p1 & MASK32).astype(np.uint32)
            c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
            k0 = np.uint32(k0 + W0)
            k1 = np.uint32(k1 + W1)
    return c0, c1, c2, c3


def normal_pair(x0, x1, dtype=np.float64):
    u1 = (((x0 >> np.uint32(8)).astype(np.float64) + 1.0) * 2.0 ** -24).astype(dtype)
    u2 = ((x1 >> np.uint32(8)).astype(np.float64) * 2.0 ** -24).astype(dtype)
    r = np.sqrt(-2.0 * np.log(u1))
    ang = 2.0 * np.pi * (u2 - 0.5)
    return r * np.cos(ang), r * np.sin(ang)


_C_LIB = None
_C_LOCK = threading.Lock()


def _c_lib():
    """The C restatement (oracle/noise.c), built on first use; None without a C compiler."""
    global _C_LIB
    with _C_LOCK:
        if _C_LIB is None:
            try:
                from . import build
                lib = ctypes.CDLL(build.build())
                lib.oracle_fourier_noise.restype = None
                lib.oracle_fourier_noise.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_ulonglong,
                                                     ctypes.c_uint, ctypes.c_uint, ctypes.c_void_p]
                _C_LIB = lib
            except Exception:
                _C_LIB = False
        return _C_LIB or None


def fourier_noise(sx, sy, sz, seed, step, field_id, dtype=np.complex128):
    """Full (reference-layout, [kz][ky][kx]) Hermitian noise field for one step, from the C
    restatement when it builds, else from the numpy one below (same values)."""
    lib = _c_lib()
    if lib is None:
        return fourier_noise_numpy(sx, sy, sz, seed, step, field_id, dtype)
    out = np.empty((sz, sy, sx), np.complex128)
    lib.oracle_fourier_noise(sx, sy, sz, int(seed) & 0xFFFFFFFFFFFFFFFF, int(step) & 0xFFFFFFFF,
                             int(field_id) & 0xFFFFFFFF, out.ctypes.data)
    return out.astype(dtype, copy=False)


def fourier_noise_numpy(sx, sy, sz, seed, step, field_id, dtype=np.complex128):
    """Full (reference-layout, [kz][ky][kx]) Hermitian noise field for one step (numpy)."""
    N = sx * sy * sz
    k0 = np.uint32(seed & 0xFFFFFFFF)
    k1 = np.uint32((seed >> 32) & 0xFFFFFFFF)
    kz, ky, kx = np.meshgrid(np.arange(sz), np.arange(sy), np.arange(sx), indexing="ij")
    out = np.zeros((sz, sy, sx), np.complex128)
    half = np.sqrt(N / 2.0)
    # modes 0 < kx < sx/2: folded line-axis counters, words (0,1) lower / (2,3) upper half
    Lt = sz if sz > 1 else (sy if sy > 1 else 1)
    sel = (kx > 0) & (2 * kx < sx)
    t = kz if sz > 1 else ky
    if Lt > 1:
        h = Lt // 2
        upper = t >= h
        tf = t - upper * h
    else:
        upper = np.zeros_like(t, bool)
        tf = t
    fkz = tf if sz > 1 else kz
    fky = ky if sz > 1 else tf
    lin_f = ((fkz * sy + fky) * sx + kx).astype(np.uint32)
    x0, x1, x2, x3 = philox4x32_10(lin_f, np.uint32(step), np.uint32(field_id), np.uint32(0), k0, k1)
    a1, a2 = normal_pair(x0, x1)
    b1, b2 = normal_pair(x2, x3)
    v = np.where(upper, b1 + 1j * b2, a1 + 1j * a2) * half
    out = np.where(sel, v, out)
    # kx = 0 and kx = sx/2 planes: canonical member of the Hermitian pair, words (0,1)
    edge = (kx == 0) | (2 * kx == sx)
    lin = (kz * sy + ky) * sx + kx
    plin = ((((-kz) % sz) * sy + ((-ky) % sy)) * sx + kx)
    canon = np.minimum(lin, plin).astype(np.uint32)
    y0, y1, _, _ = philox4x32_10(canon, np.uint32(step), np.uint32(field_id), np.uint32(0), k0, k1)
    c1, c2 = normal_pair(y0, y1)
    ev = half * (c1 + 1j * c2)
    ev = np.where(lin > plin, np.conj(ev), ev)
    ev = np.where(lin == plin, np.sqrt(float(N)) * c1 + 0j, ev)
    out = np.where(edge, ev, out)
    # kx > sx/2: conjugate of the partner (sx - kx, -ky, -kz)
    upper_x = 2 * kx > sx
    partner = np.conj(out[(-kz) % sz, (-ky) % sy, (-kx) % sx])
    out = np.where(upper_x, partner, out)
    return out.astype(dtype)


class NoiseProvider:
    """Callable for ``RefSolver(noise=...)``: (step, field_index) -> noise field."""

    def __init__(self, sx, sy, sz, seed, field_ids=None):
        self.sx, self.sy, self.sz, self.seed = sx, sy, sz, seed
        self.field_ids = field_ids

    def __call__(self, step, f):
        fid = f if self.field_ids is None else self.field_ids[f]
        return fourier_noise(self.sx, self.sy, self.sz, self.seed, step, fid)

