"""ORACLE — test infrastructure only.

ctypes access to oracle/_ref/libref_runner.so, which launches the
reference's own CUDA kernels (compiled from its sources to PTX) with cuFFT
in the order of the reference's host code.  Available only where the PTX
has been built (see oracle/build.py) and a GPU is present; `available()`
says whether it can be used.
"""

from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF = HERE / "_ref"
_L = None
_why = None

_fp = ctypes.POINTER(ctypes.c_float)
_up = ctypes.POINTER(ctypes.c_uint16)
_dp = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p


def _load():
    global _L, _why
    if _L is not None or _why is not None:
        return _L
    p = REF / "libref_runner.so"
    if not p.exists():
        _why = "reference kernels not built (oracle/_ref/libref_runner.so missing)"
        return None
    try:
        L = ctypes.CDLL(str(p))
    except OSError as e:
        _why = f"cannot load the reference runner: {e}"
        return None
    L.ref_last_error.restype = ctypes.c_char_p
    L.ref_load.argtypes = [ctypes.c_char_p]
    L.ref_deskew.argtypes = [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, _vp,
                             ctypes.c_int, ctypes.c_int, ctypes.c_float]
    L.ref_rotate.argtypes = [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _fp, _vp, ctypes.c_int,
                             ctypes.c_int]
    L.ref_affine.argtypes = [_fp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _fp, ctypes.c_int,
                             ctypes.c_float, ctypes.c_float, ctypes.c_float, _fp]
    L.ref_camcor.argtypes = [_up, ctypes.c_int, ctypes.c_int, ctypes.c_int, _fp, _up]
    L.ref_rl_iterations.argtypes = [_vp, _vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _fp,
                                    ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                    ctypes.c_float, ctypes.c_float, ctypes.c_int, _dp]
    if L.ref_load(str(REF).encode()) != 1:
        _why = "ref_load failed: " + L.ref_last_error().decode()
        return None
    _L = L
    return L


def available() -> tuple[bool, str]:
    L = _load()
    return (L is not None, _why or "")


def _check(ok, what):
    if ok != 1:
        raise RuntimeError(f"{what}: {_L.ref_last_error().decode()}")


def _torch():
    import torch
    return torch


def deskew(stack, deskew_factor, nx_out, extra_shift=0, pad_val=0.0):
    """deskew_GPU with the reference's kernel (host in, host out)."""
    torch = _torch()
    a = torch.from_numpy(np.ascontiguousarray(stack, np.float32)).cuda()
    nz, ny, nx = a.shape
    out = torch.empty((nz, ny, nx_out), dtype=torch.float32, device="cuda")
    _check(_load().ref_deskew(a.data_ptr(), nx, ny, nz, float(deskew_factor), out.data_ptr(),
                              int(nx_out), int(extra_shift), float(pad_val)), "ref_deskew")
    return out.cpu().numpy()


def rotate(stack, rot4, nx_out, nz_out):
    torch = _torch()
    a = torch.from_numpy(np.ascontiguousarray(stack, np.float32)).cuda()
    nz, ny, nx = a.shape
    r = np.ascontiguousarray(rot4, np.float32)
    out = torch.empty((nz_out, ny, nx_out), dtype=torch.float32, device="cuda")
    _check(_load().ref_rotate(a.data_ptr(), nx, ny, nz, r.ctypes.data_as(_fp), out.data_ptr(),
                              int(nx_out), int(nz_out)), "ref_rotate")
    return out.cpu().numpy()


def affine(stack, mat4x4, ra=False, dx=1.0, dy=1.0, dz=1.0):
    a = np.ascontiguousarray(stack, np.float32)
    m = np.ascontiguousarray(mat4x4, np.float32).reshape(16)
    nz, ny, nx = a.shape
    out = np.empty_like(a)
    _check(_load().ref_affine(a.ctypes.data_as(_fp), nx, ny, nz, m.ctypes.data_as(_fp), int(ra),
                              dx, dy, dz, out.ctypes.data_as(_fp)), "ref_affine")
    return out


def camcor(raw, camparam):
    a = np.ascontiguousarray(raw, np.uint16)
    p = np.ascontiguousarray(camparam, np.float32)
    nz, ny, nx = a.shape
    out = np.empty_like(a)
    _check(_load().ref_camcor(a.ctypes.data_as(_up), nx, ny, nz, p.ctypes.data_as(_fp),
                              out.ctypes.data_as(_up)), "ref_camcor")
    return out


def rl_iterations(X0, raw, otf_complex, kscales, n_iters):
    """The reference's RL loop (its kernels + cuFFT) from X0 with raw; otf_complex
    is the raw OTF as read from the file (radial table (nr, nzotf), or
    (nz_otf, ny_otf, nx_otf) for a 3D OTF).  Returns (X, lambdas)."""
    torch = _torch()
    X = torch.from_numpy(np.ascontiguousarray(X0, np.float32)).cuda()
    R = torch.from_numpy(np.ascontiguousarray(raw, np.float32)).cuda()
    nz, ny, nx = X.shape
    otf = np.ascontiguousarray(otf_complex, np.complex64)
    if otf.ndim == 2:
        nxo, nyo, nzo = otf.shape[0], 1, otf.shape[1]
    else:
        nzo, nyo, nxo = otf.shape
    flat = otf.view(np.float32).reshape(-1)
    lam = np.zeros(max(n_iters, 1), np.float64)
    _check(_load().ref_rl_iterations(X.data_ptr(), R.data_ptr(), nx, ny, nz, flat.ctypes.data_as(_fp),
                                     nxo, nyo, nzo, float(kscales[0]), float(kscales[1]),
                                     float(kscales[2]), int(n_iters), lam.ctypes.data_as(_dp)),
           "ref_rl_iterations")
    return X.cpu().numpy(), lam[:n_iters]
