"""The allocation-free acceleration-factor entry point, through the C ABI.

Callers that cannot let the library allocate device memory while they run
(multi-stream acquisition pipelines, where cudaMalloc would synchronise the
device; processes that reserve GPU memory up front) use
cdx_accel_factor_device_noalloc, whose scratch is a fixed array in device
memory.  It must give the same results as cdx_accel_factor_device, call after
call, since every call reuses that array.

This file is collected last on purpose: it must pass both alone in a fresh
process and after the other tests."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_ELEMS = 4096 * 8192


def _bind(L):
    fn = L.cdx_accel_factor_device_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p,
                   ctypes.c_void_p, ctypes.c_void_p]
    return fn


def _call(torch, fn, d1, d2, n):
    out = torch.full((3,), -1.0, dtype=torch.float64, device="cuda")
    lam = torch.full((1,), -1.0, dtype=torch.float32, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ok = fn(ctypes.c_void_p(d1.data_ptr()), ctypes.c_void_p(d2.data_ptr()), n,
            ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(lam.data_ptr()), s)
    torch.cuda.synchronize()
    return ok, out.cpu().numpy(), float(lam.item())


def test_noalloc_matches_allocating_entry_point_two_calls(cdx, torch_cuda):
    torch = torch_cuda
    L = cdx.lib()
    noalloc = _bind(L)
    rng = np.random.default_rng(1234)
    # two calls in a row with different sizes: the fixed scratch and its
    # counter are reused from one call to the next
    for n in (19353600, 1000003):
        g1 = rng.standard_normal(n).astype(np.float32)
        g2 = (0.7 * g1 + 0.4 * rng.standard_normal(n)).astype(np.float32)
        d1 = torch.from_numpy(g1).cuda()
        d2 = torch.from_numpy(g2).cuda()
        ok_ref, ref, lam_ref = _call(torch, L.cdx_accel_factor_device, d1, d2, n)
        assert ok_ref == 1
        ok, got, lam = _call(torch, noalloc, d1, d2, n)
        assert ok == 1, L.cdx_last_error()
        np.testing.assert_allclose(got, ref, rtol=1e-12)
        assert abs(lam - lam_ref) <= 1e-7 * max(1.0, abs(lam_ref))


def test_noalloc_rejects_arrays_beyond_its_scratch(cdx, torch_cuda):
    torch = torch_cuda
    noalloc = _bind(cdx.lib())
    d = torch.zeros(1, dtype=torch.float32, device="cuda")
    ok, _, _ = _call(torch, noalloc, d, d, MAX_ELEMS + 1)
    assert ok == 0
    assert b"33554432" in cdx.lib().cdx_last_error()
