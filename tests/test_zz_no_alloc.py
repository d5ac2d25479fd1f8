"""cupssgb_real_to_fourier_noalloc: the transform for callers that cannot allocate.

Callers that manage all device memory themselves (a fixed arena handed out by a host
application) cannot let the library call cudaMalloc; this entry point works from a
fixed device array inside the library instead.  The test drives it through the C-ABI
with caller-owned device buffers and checks it against the existing entry point
(cupssgb_solver_set_real + cupssgb_solver_get_fourier) on two calls in a row, with
different fields, so that nothing left in the shared working array from the first call
leaks into the second, and against numpy's FFT.  The shapes reach the size limit
(2048 x 1024 = 2^21 points: 1024-point rows and columns).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def reference_fourier(field, shape):
    import cupss_gb300 as c
    sx, sy, sz = shape
    s = c.Solver(sx, sy, sz, dt=0.01)
    f = s.add_field(True)
    s.prepare()
    s.set_real(f, field)
    out = s.get_fourier(f)
    s.close()
    return out


@pytest.mark.parametrize("shape", [(64, 32, 16), (256, 128, 1), (128, 1, 1), (2048, 1024, 1)])
def test_noalloc_matches_solver_path(built_lib, shape):
    import torch
    from cupss_gb300 import capi
    from cupss_gb300.workloads import splitmix64_uniform
    lib = capi.load()
    sx, sy, sz = shape
    n = sx * sy * sz
    outs = []
    for seed in (11, 12):
        field = splitmix64_uniform(n, seed, -1.0, 1.0)
        d_in = torch.from_numpy(field).cuda()
        d_out = torch.empty(2 * n, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        rc = lib.cupssgb_real_to_fourier_noalloc(ctypes.c_void_p(d_in.data_ptr()),
                                                 ctypes.c_void_p(d_out.data_ptr()), sx, sy, sz, None)
        assert rc == 0, lib.cupssgb_last_error()
        torch.cuda.synchronize()
        got = d_out.cpu().numpy()
        got = (got[0::2] + 1j * got[1::2]).reshape(sz, sy, sx)
        ref = reference_fourier(field, shape)
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert err < 1e-6, err
        # and against an FFT that shares no code with the library (double precision)
        exact = np.fft.fftn(field.astype(np.float64).reshape(sz, sy, sx))
        err2 = np.linalg.norm(got - exact) / np.linalg.norm(exact)
        assert err2 < 1e-5, err2
        outs.append(got)
    assert not np.allclose(outs[0], outs[1])


def test_noalloc_rejects_oversized_fields(built_lib):
    import torch
    from cupss_gb300 import capi
    lib = capi.load()
    d = torch.empty(8, dtype=torch.float32, device="cuda")
    rc = lib.cupssgb_real_to_fourier_noalloc(ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(d.data_ptr()),
                                             256, 256, 64, None)
    assert rc == capi.ERR_LIMIT
    assert b"exceeds" in lib.cupssgb_last_error()
