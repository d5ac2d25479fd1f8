"""Python mirror of the cuPSS API over the C-ABI.

``Evolver`` follows the reference's public C++ API (inc/cupss/evolver.h:14-86):
same method names, argument meaning and return codes; parse errors raise
``CupssError`` where the reference prints and exits.  ``Solver`` is the
IR-level handle (fields, implicit/explicit q-monomials, noise) used by the
batched and served forms and by tests.
"""
from __future__ import annotations

import ctypes as C
import json

import numpy as np

from . import capi


class Solver:
    """Owns one ``cupssgb_solver``: a system on an sx*sy*sz grid."""

    def __init__(self, sx, sy=1, sz=1, dx=1.0, dy=1.0, dz=1.0, dt=0.01):
        self.lib = capi.load()
        h = C.c_void_p()
        capi.check(self.lib.cupssgb_solver_create(sx, sy, sz, dx, dy, dz, dt, C.byref(h)))
        self.h = h
        self.shape = (sz, sy, sx)
        self.N = sx * sy * sz

    def close(self):
        if self.h:
            self.lib.cupssgb_solver_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_field(self, dynamic: bool) -> int:
        return capi.check(self.lib.cupssgb_solver_add_field(self.h, int(bool(dynamic))))

    def set_implicit(self, f, pres):
        arr, n = capi.pres_array(pres)
        capi.check(self.lib.cupssgb_solver_set_implicit(self.h, f, arr, n))

    def add_term(self, f, product, pres) -> int:
        prod = (C.c_int * max(len(product), 1))(*product)
        arr, n = capi.pres_array(pres)
        return capi.check(self.lib.cupssgb_solver_add_term(self.h, f, prod, len(product), arr, n))

    def set_term_pres(self, f, t, pres):
        arr, n = capi.pres_array(pres)
        capi.check(self.lib.cupssgb_solver_set_term_pres(self.h, f, t, arr, n))

    def set_noise(self, f, amp):
        if amp is None:
            capi.check(self.lib.cupssgb_solver_set_noise(self.h, f, None))
        else:
            arr, _ = capi.pres_array([amp])
            capi.check(self.lib.cupssgb_solver_set_noise(self.h, f, arr))

    def set_seed(self, seed: int):
        capi.check(self.lib.cupssgb_solver_set_seed(self.h, seed))

    def prepare(self):
        capi.check(self.lib.cupssgb_solver_prepare(self.h))

    def set_real(self, f, arr):
        a = np.ascontiguousarray(np.asarray(arr, np.float32).reshape(-1))
        assert a.size == self.N
        capi.check(self.lib.cupssgb_solver_set_real(self.h, f, capi.fptr(a)))

    def advance(self, n=1):
        capi.check(self.lib.cupssgb_solver_advance(self.h, n))

    def synchronize(self):
        capi.check(self.lib.cupssgb_solver_synchronize(self.h))

    def get_real(self, f):
        out = np.empty(self.N, np.float32)
        capi.check(self.lib.cupssgb_solver_get_real(self.h, f, capi.fptr(out)))
        return out.reshape(self.shape)

    def get_fourier(self, f):
        out = np.empty(2 * self.N, np.float32)
        capi.check(self.lib.cupssgb_solver_get_fourier(self.h, f, capi.fptr(out)))
        return (out[0::2] + 1j * out[1::2]).reshape(self.shape)

    def time_advance(self, n):
        ms = C.c_double()
        capi.check(self.lib.cupssgb_solver_time_advance(self.h, int(n), C.byref(ms)))
        return ms.value

    def set_stream_priority(self, level):
        capi.check(self.lib.cupssgb_solver_set_stream_priority(self.h, int(level)))

    def set_kernel_timing(self, on):
        capi.check(self.lib.cupssgb_solver_set_kernel_timing(self.h, int(bool(on))))

    def kernel_report(self):
        n = capi.check(self.lib.cupssgb_solver_kernel_report(self.h, None, 0))
        buf = C.create_string_buffer(n + 1)
        self.lib.cupssgb_solver_kernel_report(self.h, buf, n + 1)
        return json.loads(buf.value.decode())

    def generated_sources(self):
        out = []
        i = 0
        while True:
            n = self.lib.cupssgb_solver_generated_source(self.h, i, None, 0)
            if n < 0:
                break
            buf = C.create_string_buffer(n + 1)
            self.lib.cupssgb_solver_generated_source(self.h, i, buf, n + 1)
            out.append(buf.value.decode())
            i += 1
        return out

    def set_generated_programs(self, on):
        capi.check(self.lib.cupssgb_solver_set_generated_programs(self.h, int(bool(on))))

    def set_real_ptr(self, f, host_ptr):
        capi.check(self.lib.cupssgb_solver_set_real(self.h, f, C.cast(host_ptr, capi._FP)))

    def get_real_ptr(self, f, host_ptr):
        capi.check(self.lib.cupssgb_solver_get_real(self.h, f, C.cast(host_ptr, capi._FP)))

    def snapshot_real_ptr(self, f, host_ptr, done_event=None):
        """Asynchronous read-out of field f into host memory (complete after synchronize
        or once done_event, a cudaEvent_t handle, has been reached)."""
        capi.check(self.lib.cupssgb_solver_snapshot_real(self.h, f, C.cast(host_ptr, C.c_void_p), done_event))

    # ---- batches ----
    def set_members(self, n):
        capi.check(self.lib.cupssgb_solver_set_members(self.h, int(n)))

    def set_member_term_pres(self, m, f, t, pres):
        arr, n = capi.pres_array(pres)
        capi.check(self.lib.cupssgb_solver_set_member_term_pres(self.h, m, f, t, arr, n))

    def set_member_implicit(self, m, f, pres):
        arr, n = capi.pres_array(pres)
        capi.check(self.lib.cupssgb_solver_set_member_implicit(self.h, m, f, arr, n))

    def set_member_noise(self, m, f, amp):
        arr, _ = capi.pres_array([amp])
        capi.check(self.lib.cupssgb_solver_set_member_noise(self.h, m, f, arr))

    def set_member_seed(self, m, seed):
        capi.check(self.lib.cupssgb_solver_set_member_seed(self.h, m, int(seed)))

    def set_member_active(self, m, on):
        capi.check(self.lib.cupssgb_solver_set_member_active(self.h, m, int(bool(on))))

    def reset_member(self, m):
        capi.check(self.lib.cupssgb_solver_reset_member(self.h, m))

    def member_step(self, m):
        return capi.check(self.lib.cupssgb_solver_member_step(self.h, m))

    def set_real_member(self, f, m, arr):
        a = np.ascontiguousarray(np.asarray(arr, np.float32).reshape(-1))
        assert a.size == self.N
        capi.check(self.lib.cupssgb_solver_set_real_member(self.h, f, m, capi.fptr(a)))

    def get_real_member(self, f, m):
        out = np.empty(self.N, np.float32)
        capi.check(self.lib.cupssgb_solver_get_real_member(self.h, f, m, capi.fptr(out)))
        return out.reshape(self.shape)

    def estimate_bytes(self, members=1):
        return capi.check(self.lib.cupssgb_solver_estimate_bytes(self.h, int(members)))

    def tune_report(self):
        n = capi.check(self.lib.cupssgb_solver_tune_report(self.h, None, 0))
        buf = C.create_string_buffer(n + 1)
        self.lib.cupssgb_solver_tune_report(self.h, buf, n + 1)
        return json.loads(buf.value.decode())

    @property
    def step_count(self):
        return self.lib.cupssgb_solver_step_count(self.h)

    @property
    def launch_count(self):
        return self.lib.cupssgb_solver_launch_count(self.h)

    @property
    def device_bytes(self):
        return self.lib.cupssgb_solver_device_bytes(self.h)


class PinnedBuffer:
    """Page-locked host buffer (cupssgb_host_alloc) viewed as a float32 numpy array."""

    def __init__(self, nfloats):
        self.lib = capi.load()
        p = C.c_void_p()
        capi.check(self.lib.cupssgb_host_alloc(4 * nfloats, C.byref(p)))
        self.ptr = p
        self.array = np.ctypeslib.as_array(C.cast(p, capi._FP), shape=(nfloats,))

    def close(self):
        if self.ptr:
            self.lib.cupssgb_host_free(self.ptr)
            self.ptr = None


def jit_check(source):
    """Compiles a generated kernel source for sm_103a (no GPU needed); returns the
    cubin size or raises CupssError with the NVRTC log."""
    lib = capi.load()
    log = C.create_string_buffer(1 << 16)
    rc = lib.cupssgb_jit_check(source.encode(), log, len(log))
    if rc < 0:
        raise capi.CupssError(rc, log.value.decode())
    return rc


def set_device(dev):
    capi.check(capi.load().cupssgb_set_device(int(dev)))


def device_info():
    """(number of visible CUDA devices, one text line per device plus the versions)."""
    lib = capi.load()
    buf = C.create_string_buffer(8192)
    n = lib.cupssgb_device_info(buf, len(buf))
    if n < 0:
        capi.check(n)
    return n, buf.value.decode()


def write_field_csv(path, name, values, precision=6):
    """One field file in the reference's CSV format; values shaped (sz, sy, sx) or (sy, sx) or (sx,)."""
    a = np.ascontiguousarray(np.asarray(values, np.float32))
    shp = a.shape[::-1] + (1,) * (3 - a.ndim)
    return capi.check(capi.load().cupssgb_write_field_csv(str(path).encode(), name.encode(), capi.fptr(a.reshape(-1)),
                                                          shp[0], shp[1], shp[2], int(precision)))


class Evolver:
    """Mirror of the reference ``evolver`` (same method names as the C++ API)."""

    def __init__(self, with_cuda, sx, sy=1, sz=1, dx=1.0, dy=1.0, dz=1.0, dt=0.01, write_every=1):
        self.lib = capi.load()
        h = C.c_void_p()
        capi.check(self.lib.cupssgb_evolver_create(int(bool(with_cuda)), sx, sy, sz, dx, dy, dz, dt,
                                                   write_every, C.byref(h)))
        self.h = h
        self.shape = (sz, sy, sx)
        self.N = sx * sy * sz

    def close(self):
        if self.h:
            self.lib.cupssgb_evolver_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def createField(self, name, dynamic):
        return capi.check(self.lib.cupssgb_evolver_create_field(self.h, name.encode(), int(bool(dynamic))))

    def addParameter(self, name, value):
        return capi.check(self.lib.cupssgb_evolver_add_parameter(self.h, name.encode(), float(value)))

    def addEquation(self, eq):
        return capi.check(self.lib.cupssgb_evolver_add_equation(self.h, eq.encode()))

    def addNoise(self, name, amp):
        return capi.check(self.lib.cupssgb_evolver_add_noise(self.h, name.encode(), amp.encode()))

    def updateParameter(self, name, value):
        return capi.check(self.lib.cupssgb_evolver_update_parameter(self.h, name.encode(), float(value)))

    def getParameter(self, name):
        return self.lib.cupssgb_evolver_get_parameter(self.h, name.encode())

    def setOutputField(self, name, out):
        return capi.check(self.lib.cupssgb_evolver_set_output_field(self.h, name.encode(), int(out)))

    def setNoiseSeed(self, seed):
        return capi.check(self.lib.cupssgb_evolver_set_seed(self.h, int(seed)))

    def setReal(self, name, arr):
        a = np.ascontiguousarray(np.asarray(arr, np.float32).reshape(-1))
        assert a.size == self.N
        return capi.check(self.lib.cupssgb_evolver_set_real(self.h, name.encode(), capi.fptr(a)))

    def prepareProblem(self):
        return capi.check(self.lib.cupssgb_evolver_prepare(self.h))

    def advanceTime(self, n=1):
        return capi.check(self.lib.cupssgb_evolver_advance(self.h, int(n)))

    def writeOut(self):
        return capi.check(self.lib.cupssgb_evolver_write_out(self.h))

    def getReal(self, name):
        out = np.empty(self.N, np.float32)
        capi.check(self.lib.cupssgb_evolver_get_real(self.h, name.encode(), capi.fptr(out)))
        return out.reshape(self.shape)

    def getFourier(self, name):
        out = np.empty(2 * self.N, np.float32)
        capi.check(self.lib.cupssgb_evolver_get_fourier(self.h, name.encode(), capi.fptr(out)))
        return (out[0::2] + 1j * out[1::2]).reshape(self.shape)

    def getCurrentTimestep(self):
        return self.lib.cupssgb_evolver_current_step(self.h)

    def flushOutput(self):
        return capi.check(self.lib.cupssgb_evolver_flush_output(self.h))

    def createFromFile(self, path):
        return capi.check(self.lib.cupssgb_evolver_create_from_file(self.h, str(path).encode()))

    def initializeUniform(self, name, value):
        return capi.check(self.lib.cupssgb_evolver_initialize_uniform(self.h, name.encode(), float(value)))

    def initializeUniformNoise(self, name, amplitude):
        return capi.check(self.lib.cupssgb_evolver_initialize_uniform_noise(self.h, name.encode(), float(amplitude)))

    def initializeNormalNoise(self, name, mean, sigma):
        return capi.check(self.lib.cupssgb_evolver_initialize_normal_noise(self.h, name.encode(), float(mean),
                                                                           float(sigma)))

    def initializeHalfSystem(self, name, value1, value2, width, direction):
        return capi.check(self.lib.cupssgb_evolver_initialize_half_system(self.h, name.encode(), float(value1),
                                                                          float(value2), float(width), int(direction)))

    def initializeDroplet(self, name, value_out, value_in, radius, width, cx, cy, cz):
        return capi.check(self.lib.cupssgb_evolver_initialize_droplet(self.h, name.encode(), float(value_out),
                                                                      float(value_in), float(radius), float(width),
                                                                      int(cx), int(cy), int(cz)))

    def addDroplet(self, name, value, radius, width, cx, cy, cz):
        return capi.check(self.lib.cupssgb_evolver_add_droplet(self.h, name.encode(), float(value), float(radius),
                                                               float(width), int(cx), int(cy), int(cz)))

    def initializeFromFile(self, name, path, skiprows=0, delimiter=","):
        return capi.check(self.lib.cupssgb_evolver_initialize_from_file(self.h, name.encode(), str(path).encode(),
                                                                        int(skiprows), delimiter.encode()))

    def getHostReal(self, name):
        """The host array of a field (fieldsReal): what the initializers or setReal wrote."""
        out = np.empty(self.N, np.float32)
        capi.check(self.lib.cupssgb_evolver_get_host_real(self.h, name.encode(), capi.fptr(out)))
        return out.reshape(self.shape)

    def setCallback(self, name, fn, fourier=False):
        """fn(evolver_ptr, field_ptr, sx, sy, sz) -> None, or None to remove.  The ctypes
        wrapper is kept alive by this object."""
        cb = capi.CALLBACK(fn) if fn is not None else capi.CALLBACK()
        self._callbacks = getattr(self, "_callbacks", {})
        self._callbacks[(name, bool(fourier))] = cb
        return capi.check(self.lib.cupssgb_evolver_set_callback(self.h, name.encode(), int(bool(fourier)), cb))

    def describe(self):
        n = self.lib.cupssgb_evolver_describe(self.h, None, 0)
        buf = C.create_string_buffer(n + 1)
        self.lib.cupssgb_evolver_describe(self.h, buf, n + 1)
        return json.loads(buf.value.decode())


def multi_generated_sources(solvers):
    """Sources of the fused kernels (phases 0 and 1, "" for a phase without fields) that
    step these batched solvers together; no GPU needed."""
    lib = capi.load()
    arr = (C.c_void_p * len(solvers))(*[s.h for s in solvers])
    out = []
    for ph in (0, 1):
        n = capi.check(lib.cupssgb_multi_generated_source(arr, len(solvers), ph, None, 0))
        buf = C.create_string_buffer(n + 1)
        lib.cupssgb_multi_generated_source(arr, len(solvers), ph, buf, n + 1)
        out.append(buf.value.decode())
    return out


class Ensemble:
    """Mirror of the C++ ``ensemble`` (include/cupss/ensemble.h): one system declared
    with the evolver's calls, many members (grid, dt, seed, parameter values) advanced
    together in batch solvers."""

    def __init__(self):
        self.lib = capi.load()
        h = C.c_void_p()
        capi.check(self.lib.cupssgb_ensemble_create(C.byref(h)))
        self.h = h
        self.shapes = []

    def close(self):
        if self.h:
            self.lib.cupssgb_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def createField(self, name, dynamic):
        return capi.check(self.lib.cupssgb_ensemble_create_field(self.h, name.encode(), int(bool(dynamic))))

    def addParameter(self, name, value):
        return capi.check(self.lib.cupssgb_ensemble_add_parameter(self.h, name.encode(), float(value)))

    def addEquation(self, eq):
        return capi.check(self.lib.cupssgb_ensemble_add_equation(self.h, eq.encode()))

    def addNoise(self, name, amp):
        return capi.check(self.lib.cupssgb_ensemble_add_noise(self.h, name.encode(), amp.encode()))

    def addMember(self, sx, sy=1, sz=1, dx=1.0, dy=1.0, dz=1.0, dt=0.01, seed=0, **params):
        m = capi.check(self.lib.cupssgb_ensemble_add_member(self.h, sx, sy, sz, dx, dy, dz, dt, int(seed)))
        self.shapes.append((sz, sy, sx))
        for k, v in params.items():
            self.setMemberParameter(m, k, v)
        return m

    def setMemberParameter(self, m, name, value):
        return capi.check(self.lib.cupssgb_ensemble_set_member_parameter(self.h, m, name.encode(), float(value)))

    def prepare(self):
        return capi.check(self.lib.cupssgb_ensemble_prepare(self.h))

    def setReal(self, m, name, arr):
        a = np.ascontiguousarray(np.asarray(arr, np.float32).reshape(-1))
        assert a.size == int(np.prod(self.shapes[m]))
        return capi.check(self.lib.cupssgb_ensemble_set_real(self.h, m, name.encode(), capi.fptr(a)))

    def advance(self, n):
        return capi.check(self.lib.cupssgb_ensemble_advance(self.h, int(n)))

    def getReal(self, m, name):
        out = np.empty(int(np.prod(self.shapes[m])), np.float32)
        capi.check(self.lib.cupssgb_ensemble_get_real(self.h, m, name.encode(), capi.fptr(out)))
        return out.reshape(self.shapes[m])

    @property
    def groups(self):
        return self.lib.cupssgb_ensemble_groups(self.h)

    @property
    def device_bytes(self):
        return self.lib.cupssgb_ensemble_device_bytes(self.h)

    @property
    def launch_count(self):
        return self.lib.cupssgb_ensemble_launch_count(self.h)

    def describe(self):
        n = capi.check(self.lib.cupssgb_ensemble_describe(self.h, None, 0))
        buf = C.create_string_buffer(n + 1)
        self.lib.cupssgb_ensemble_describe(self.h, buf, n + 1)
        return json.loads(buf.value.decode())


class Server:
    """Mirror of the C++ ``server`` (include/cupss/server.h): continuous batching of
    independent solves within an HBM budget, scheduled by a native thread."""

    def __init__(self, hbm_budget=150e9, max_slots=32, max_chunk=256):
        self.lib = capi.load()
        h = C.c_void_p()
        capi.check(self.lib.cupssgb_server_create(float(hbm_budget), int(max_slots), int(max_chunk), C.byref(h)))
        self.h = h
        self.shapes = {}

    def close(self):
        if self.h:
            self.lib.cupssgb_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def addSystem(self, system=None):
        """New system id; `system` (a workloads.SYSTEMS entry) declares it at once."""
        sid = capi.check(self.lib.cupssgb_server_add_system(self.h))
        if system is not None:
            for nm, dyn in system["fields"]:
                self.createField(sid, nm, dyn)
            for k, v in system["params"].items():
                self.addParameter(sid, k, v)
            for q in system["eqs"]:
                self.addEquation(sid, q)
            for f, a in system["noise"]:
                self.addNoise(sid, f, a)
            if "out" in system:
                self.setOutputField(sid, system["out"])
        return sid

    def createField(self, sid, name, dynamic):
        return capi.check(self.lib.cupssgb_server_create_field(self.h, sid, name.encode(), int(bool(dynamic))))

    def addParameter(self, sid, name, value):
        return capi.check(self.lib.cupssgb_server_add_parameter(self.h, sid, name.encode(), float(value)))

    def addEquation(self, sid, eq):
        return capi.check(self.lib.cupssgb_server_add_equation(self.h, sid, eq.encode()))

    def addNoise(self, sid, name, amp):
        return capi.check(self.lib.cupssgb_server_add_noise(self.h, sid, name.encode(), amp.encode()))

    def setOutputField(self, sid, name):
        return capi.check(self.lib.cupssgb_server_set_output_field(self.h, sid, name.encode()))

    def submit(self, sid, shape, dt, nsteps, seed=0, params=None, init=None, cell=(1.0, 1.0, 1.0)):
        sx, sy, sz = shape
        params = params or {}
        init = init or {}
        names = (C.c_char_p * max(len(params), 1))(*[k.encode() for k in params])
        vals = (C.c_float * max(len(params), 1))(*[float(v) for v in params.values()])
        arrays = [np.ascontiguousarray(np.asarray(a, np.float32).reshape(-1)) for a in init.values()]
        for a in arrays:
            assert a.size == sx * sy * sz
        fields = (C.c_char_p * max(len(init), 1))(*[k.encode() for k in init])
        ptrs = (capi._FP * max(len(init), 1))(*[capi.fptr(a) for a in arrays])
        rid = capi.check(self.lib.cupssgb_server_submit(self.h, sid, sx, sy, sz, *cell, float(dt), int(nsteps),
                                                        int(seed), len(params), names, vals, len(init), fields,
                                                        ptrs))
        self.shapes[rid] = (sz, sy, sx)
        return rid

    def warm(self, sid, shape, dt, cell=(1.0, 1.0, 1.0)):
        return capi.check(self.lib.cupssgb_server_warm(self.h, sid, *shape, *cell, float(dt)))

    def wait(self, rid, timeout=-1.0):
        return bool(capi.check(self.lib.cupssgb_server_wait(self.h, rid, float(timeout))))

    def result(self, rid):
        out = np.empty(int(np.prod(self.shapes[rid])), np.float32)
        capi.check(self.lib.cupssgb_server_result(self.h, rid, capi.fptr(out)))
        return out.reshape(self.shapes[rid])

    def times(self, rid):
        t = (C.c_double * 3)()
        capi.check(self.lib.cupssgb_server_times(self.h, rid, t))
        return tuple(t)

    def stats(self):
        n = capi.check(self.lib.cupssgb_server_stats(self.h, None, 0))
        buf = C.create_string_buffer(n + 1)
        self.lib.cupssgb_server_stats(self.h, buf, n + 1)
        return json.loads(buf.value.decode())
