"""Host-memory paths of the solver C-ABI: page-locked inputs and outputs.

set_real from page-locked memory copies on an input stream into one of two staging
buffers; get_real into page-locked memory has the row pass store the field there
directly; snapshot_real copies out on an output stream.  These tests check that each
path gives the bytes of the plain path (pageable numpy arrays, copies on the solver's
stream), that a pipelined loop (input k+1 and output k in flight together) gives the
results of the blocking loop step by step, and that an unaligned page-locked address
falls back to the copy.
"""
import ctypes

import numpy as np
import pytest

from cupss_gb300.workloads import splitmix64_uniform

pytestmark = pytest.mark.gpu

CH_NOISELESS = ([("phi", 1)], {"a": -1.0, "b": 1.0, "k": 1.0},
                ["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3"], [])


def solver(shape):
    from tests.test_codegen import solver_from_ir
    from tests.test_parser_parity import build_lib
    s = solver_from_ir(build_lib(*CH_NOISELESS), shape)
    s.prepare()
    return s


@pytest.mark.parametrize("shape", [(64, 32, 16), (128, 128, 1), (96, 48, 24)])
def test_pinned_paths_equal_pageable(built_lib, monkeypatch, shape):
    from cupss_gb300.api import PinnedBuffer
    n = int(np.prod(shape))
    field = splitmix64_uniform(n, 3, -1, 1)
    a, b = solver(shape), solver(shape)
    pin = PinnedBuffer(n)
    pin.array[:] = field
    a.set_real_ptr(0, pin.ptr)            # input stream, staging buffer
    b.set_real(0, field.reshape(shape[::-1]))   # pageable: solver stream
    assert np.array_equal(a.get_fourier(0), b.get_fourier(0))
    a.advance(3)
    b.advance(3)
    out = PinnedBuffer(n)
    a.get_real_ptr(0, out.ptr)            # direct store into host memory
    want = b.get_real(0).ravel()
    assert np.array_equal(out.array, want)
    monkeypatch.setenv("CUPSSGB_HOST_DIRECT", "0")
    out.array[:] = 0
    a.get_real_ptr(0, out.ptr)            # the copy path
    assert np.array_equal(out.array, want)
    for x in (a, b):
        x.close()
    pin.close()
    out.close()


def test_pipelined_loop_equals_blocking_loop(built_lib):
    """Per step: input copied in from page-locked memory, one step, result copied out
    asynchronously; inputs alternate between two fields.  Every step's result equals
    the blocking loop's (set_real, advance, get_real) bit for bit."""
    from cupss_gb300.api import PinnedBuffer
    shape = (64, 64, 32)
    n = int(np.prod(shape))
    K = 7
    ins = [PinnedBuffer(n) for _ in range(2)]
    ins[0].array[:] = splitmix64_uniform(n, 1, -0.5, 0.5)
    ins[1].array[:] = splitmix64_uniform(n, 2, -0.5, 0.5)
    outs = [PinnedBuffer(n) for _ in range(K)]
    a = solver(shape)
    for k in range(K):
        a.set_real_ptr(0, ins[k % 2].ptr)
        a.advance(1)
        a.snapshot_real_ptr(0, outs[k].ptr)
    a.synchronize()
    b = solver(shape)
    for k in range(K):
        b.set_real(0, ins[k % 2].array.reshape(shape[::-1]).copy())
        b.advance(1)
        assert np.array_equal(outs[k].array, b.get_real(0).ravel()), k
    assert not np.array_equal(outs[0].array, outs[1].array)
    for x in [a, b] + ins + outs:
        x.close()


def test_unaligned_pinned_address_takes_the_copy(built_lib):
    from cupss_gb300.api import PinnedBuffer
    shape = (32, 16, 8)
    n = int(np.prod(shape))
    field = splitmix64_uniform(n, 9, -1, 1)
    pin = PinnedBuffer(n + 4)
    base = ctypes.cast(pin.ptr, ctypes.c_void_p).value
    view = np.ctypeslib.as_array(ctypes.cast(base + 4, ctypes.POINTER(ctypes.c_float)), shape=(n,))
    view[:] = field
    a, b = solver(shape), solver(shape)
    a.set_real_ptr(0, ctypes.c_void_p(base + 4))
    b.set_real(0, field.reshape(shape[::-1]))
    assert np.array_equal(a.get_fourier(0), b.get_fourier(0))
    view[:] = 0
    a.get_real_ptr(0, ctypes.c_void_p(base + 4))
    assert np.array_equal(view, b.get_real(0).ravel())
    for x in (a, b, pin):
        x.close()


def test_stream_priority(built_lib):
    """A solver whose work moves between streams of other priorities mid-run computes
    what one on the default stream does (each switch is ordered after the work before)."""
    import cupss_gb300 as c
    shape = (64, 32, 16)
    field = splitmix64_uniform(int(np.prod(shape)), 4, -1, 1).reshape(shape[::-1])
    out = []
    for level in (0, 9):
        from tests.test_codegen import solver_from_ir
        from tests.test_parser_parity import build_lib
        s = solver_from_ir(build_lib(*CH_NOISELESS), shape)
        s.set_stream_priority(level)   # 9: clamped to the device's highest
        s.prepare()
        s.set_real(0, field)
        for k in range(10):
            s.advance(3)
            s.set_stream_priority((k * 7 + level) % 4)   # switch with work in flight
        out.append(s.get_real(0))
        with pytest.raises(c.CupssError):
            s.set_stream_priority(-1)
        s.close()
    assert np.array_equal(out[0], out[1])
