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
import subprocess
import sys
import textwrap

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


def test_noalloc_at_its_limit_against_float64_sums(cdx, torch_cuda):
    """n at the limit fills every partial slot of the fixed array; the result
    is checked against float products summed in float64 (the reference's
    innerProduct arithmetic, RLgpuImpl.cu:584-592), not only against the
    allocating entry point, which shares the block code."""
    torch = torch_cuda
    L = cdx.lib()
    noalloc = _bind(L)
    rng = np.random.default_rng(77)
    n = MAX_ELEMS
    g1 = rng.standard_normal(n, dtype=np.float32)
    g2 = (0.3 * g1 + rng.standard_normal(n, dtype=np.float32)).astype(np.float32)
    num = float(np.sum(g1 * g2, dtype=np.float64))
    den = float(np.sum(g2 * g2, dtype=np.float64))
    d1 = torch.from_numpy(g1).cuda()
    d2 = torch.from_numpy(g2).cuda()
    for _ in range(2):
        ok, got, lam = _call(torch, noalloc, d1, d2, n)
        assert ok == 1, L.cdx_last_error()
        np.testing.assert_allclose(got[:2], [num, den], rtol=1e-11)
        ref_lam = min(max(num / (den + 1.1920928955078125e-07), 0.0), 1.0)
        assert abs(lam - ref_lam) <= 1e-6


_RESET_SCRIPT = textwrap.dedent("""
    import ctypes, sys
    import numpy as np
    L = ctypes.CDLL(sys.argv[1])
    rt = ctypes.CDLL("libcudart.so.13")
    vp = ctypes.c_void_p
    for f in ("cdx_accel_factor_device", "cdx_accel_factor_device_noalloc"):
        getattr(L, f).restype = ctypes.c_int
        getattr(L, f).argtypes = [vp, vp, ctypes.c_longlong, vp, vp, vp]
    L.cdx_last_error.restype = ctypes.c_char_p
    n = 3000017
    rng = np.random.default_rng(5)
    g1 = rng.standard_normal(n).astype(np.float32)
    g2 = (0.5 * g1 + rng.standard_normal(n)).astype(np.float32)

    def dev_copy(a):
        p = vp()
        assert rt.cudaMalloc(ctypes.byref(p), ctypes.c_size_t(a.nbytes)) == 0
        assert rt.cudaMemcpy(p, a.ctypes.data_as(vp), ctypes.c_size_t(a.nbytes), 1) == 0
        return p

    def run(fn):
        d1, d2 = dev_copy(g1), dev_copy(g2)
        out = dev_copy(np.zeros(3, np.float64))
        lam = dev_copy(np.zeros(1, np.float32))
        assert getattr(L, fn)(d1, d2, n, out, lam, None) == 1, L.cdx_last_error()
        assert rt.cudaDeviceSynchronize() == 0
        h = np.zeros(3, np.float64)
        assert rt.cudaMemcpy(h.ctypes.data_as(vp), out, ctypes.c_size_t(24), 2) == 0
        for q in (d1, d2, out, lam):
            rt.cudaFree(q)
        return h

    ref = run("cdx_accel_factor_device")
    first = run("cdx_accel_factor_device_noalloc")
    L.cuda_reset()  # new primary context: the array may move
    second = run("cdx_accel_factor_device_noalloc")
    third = run("cdx_accel_factor_device_noalloc")
    for h in (first, second, third):
        assert np.allclose(h[:2], ref[:2], rtol=1e-12, atol=0), (h, ref)
    print("ok")
""")


def test_noalloc_after_cuda_reset_in_fresh_process(cdx, torch_cuda):
    """cuda_reset destroys the primary context; the next call must look the
    array's address up again in the new context.  Run in a child process so
    that the reset does not touch this process's CUDA state."""
    r = subprocess.run([sys.executable, "-c", _RESET_SCRIPT, str(cdx.lib_path())],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "ok" in r.stdout, r.stdout + r.stderr
