"""User callbacks (field::callback / callbackFourier, src/field.cpp:48-86) against the
oracle.  The reference calls the Fourier-space callback on comp_array after the
update and before dealiasing, and the real-space callback on real_array (and on the
dealiased copy when the field is in a product) after the inverse transform; the
oracle (oracle/ref_solver.py) applies the same functions at the same points.
Callbacks receive device pointers in GPU mode (wrapped here as torch tensors) and
host pointers in RUN_CPU mode (wrapped as numpy arrays)."""
import ctypes

import numpy as np
import pytest

from oracle.philox import NoiseProvider
from oracle.ref_parser import System
from oracle.ref_solver import RefSolver, droplet

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _in_tmp(tmp_path, monkeypatch, built_lib):
    monkeypatch.chdir(tmp_path)


class _CudaArray:
    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<f4", "data": (ptr, False), "version": 3,
                                         "strides": None}


def mirror_idx(n):
    i = np.arange(n)
    return np.where(i < n // 2, i, (n - i) % n)


def make_mirror(shape):
    sx, sy, sz = shape
    ii, jj = mirror_idx(sx), mirror_idx(sy)

    def np_fn(r):
        return r[:, jj][:, :, ii]

    def gpu_fn(ev, ptr, a, b, c):
        import torch
        t = torch.as_tensor(_CudaArray(ptr, 2 * sx * sy * sz), device="cuda").view(sz, sy, sx, 2)
        x = t[..., 0].clone()
        t[..., 0] = x[:, torch.as_tensor(jj, device="cuda")][:, :, torch.as_tensor(ii, device="cuda")]
        torch.cuda.synchronize()

    def host_fn(ev, ptr, a, b, c):
        arr = np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ctypes.c_float)), shape=(sz, sy, sx, 2))
        arr[..., 0] = np_fn(arr[..., 0].copy())

    return np_fn, gpu_fn, host_fn


def make_damping(shape, kcut):
    sx, sy, sz = shape
    n = lambda k, N: np.where(k > N // 2, k - N, k)
    kz, ky, kx = np.meshgrid(np.arange(sz), np.arange(sy), np.arange(sx), indexing="ij")
    fac = np.where(n(kx, sx) ** 2 + n(ky, sy) ** 2 + n(kz, sz) ** 2 > kcut ** 2, 0.5, 1.0).astype(np.float32)

    def np_fn(c):
        return c * fac

    def gpu_fn(ev, ptr, a, b, c):
        import torch
        t = torch.as_tensor(_CudaArray(ptr, 2 * sx * sy * sz), device="cuda").view(sz, sy, sx, 2)
        t *= torch.as_tensor(fac, device="cuda")[..., None]
        torch.cuda.synchronize()

    return np_fn, gpu_fn


def run(spec, shape, dt, nsteps, inits, real_cb=None, fourier_cb=None, seed=9, with_cuda=True):
    import cupss_gb300 as c
    fields, params, eqs, noises = spec
    sx, sy, sz = shape
    s = System()
    for nm, dyn in fields:
        s.create_field(nm, bool(dyn))
    for k, v in params.items():
        s.add_parameter(k, v)
    for q in eqs:
        s.add_equation(q)
    for f, a in noises:
        s.add_noise(f, a)
    r = RefSolver(s, sx, sy, sz, dt=dt, noise=NoiseProvider(sx, sy, sz, seed))
    e = c.Evolver(with_cuda, sx, sy, sz, dt=dt, write_every=10 ** 9)
    for nm, dyn in fields:
        e.createField(nm, bool(dyn))
    for k, v in params.items():
        e.addParameter(k, v)
    for q in eqs:
        e.addEquation(q)
    for f, a in noises:
        e.addNoise(f, a)
    e.setNoiseSeed(seed)
    for nm, (np_fn, dev_fn) in (real_cb or {}).items():
        r.callbacks[nm] = np_fn
        e.setCallback(nm, dev_fn, fourier=False)
    for nm, (np_fn, dev_fn) in (fourier_cb or {}).items():
        r.fourier_callbacks[nm] = np_fn
        e.setCallback(nm, dev_fn, fourier=True)
    for nm, arr in inits.items():
        r.set_real(nm, arr)
        e.setReal(nm, arr)
    r.prepare()
    e.prepareProblem()
    r.advance(nsteps)
    e.advanceTime(nsteps)
    return r, e, [nm for nm, _ in fields]


def rel(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


INHOM = ([("v", 1), ("iqxv", 0), ("x", 0)], {},
         ["dt v +0.5*q^2*v = iqx*x*iqxv + x*iqy^2*v", "iqxv = iqx*v"], [])


def test_real_space_callback_mirror_2d():
    """System and boundary trick of examples/07_inhomogeneous_diffusion (reduced)."""
    shape = (32, 32, 1)
    np_fn, gpu_fn, _ = make_mirror(shape)
    v0 = droplet(shape, 1.0, 0.0, 6.0, 2.0, 8, 8, 0)
    xx = np.broadcast_to(1.0 + 0.5 * np.tanh((np.arange(32) - 10) / 4.0), (1, 32, 32)).astype(np.float32)
    r, e, names = run(INHOM, shape, 0.01, 30, {"v": v0, "x": np.ascontiguousarray(xx)},
                      real_cb={"v": (np_fn, gpu_fn), "x": (np_fn, gpu_fn)})
    for nm in names:
        assert rel(e.getReal(nm), r.real_field(nm)) < 3e-5, nm


def test_fourier_callback_damping_2d():
    shape = (32, 32, 1)
    np_fn, gpu_fn = make_damping(shape, 6)
    spec = ([("phi", 1)], {"a": -1.0, "b": 1.0, "k": 1.0}, ["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3"], [])
    from cupss_gb300.workloads import splitmix64_uniform
    init = splitmix64_uniform(32 * 32, 3, -0.3, 0.3).reshape(1, 32, 32)
    r, e, _ = run(spec, shape, 0.05, 40, {"phi": init}, fourier_cb={"phi": (np_fn, gpu_fn)})
    assert rel(e.getReal("phi"), r.real_field("phi")) < 3e-5


def test_both_callbacks_noisy_3d():
    shape = (16, 8, 8)
    m_np, m_gpu, _ = make_mirror(shape)
    d_np, d_gpu = make_damping(shape, 3)
    spec = ([("phi", 1)], {"a": -1.0, "b": 1.0, "k": 1.0, "T": 0.01},
            ["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3"], [("phi", "2*T*q^2")])
    from cupss_gb300.workloads import splitmix64_uniform
    init = splitmix64_uniform(16 * 8 * 8, 5, -0.3, 0.3).reshape(8, 8, 16)
    r, e, _ = run(spec, shape, 0.02, 20, {"phi": init}, real_cb={"phi": (m_np, m_gpu)},
                  fourier_cb={"phi": (d_np, d_gpu)})
    assert rel(e.getReal("phi"), r.real_field("phi")) < 3e-5


def test_host_callback_in_cpu_mode():
    """RUN_CPU (examples/08_neumann_dirichlet_bc): callbacks get host pointers."""
    shape = (64, 1, 1)
    np_fn, _, host_fn = make_mirror(shape)
    spec = ([("phi_neu", 1)], {}, ["dt phi_neu + q^2*phi_neu = 0.0"], [])
    init = droplet(shape, 1.0, 0.0, 10.0, 3.0, 16, 0, 0)
    r, e, _ = run(spec, shape, 0.05, 25, {"phi_neu": init}, real_cb={"phi_neu": (np_fn, host_fn)},
                  with_cuda=False)
    assert rel(e.getReal("phi_neu"), r.real_field("phi_neu")) < 3e-5
