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
    L.ref_session_open.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                   ctypes.c_int, _fp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_float, ctypes.c_float, ctypes.c_float, _fp,
                                   ctypes.c_int, ctypes.c_int]
    L.ref_session_step.argtypes = [ctypes.c_int, _vp, ctypes.c_float, ctypes.c_int, _vp]
    L.ref_session_close.argtypes = [ctypes.c_int]
    L.ref_session_close.restype = None
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


class Session:
    """One RL_interface call's device work with the reference's kernels and
    cuFFT (RichardsonLucy_GPU, src/RL-Biggs-Andrews.cpp:56-450): background
    subtraction, the bleach statistic, deskew, the RL loop with its
    per-iteration host round trip for lambda, rotation.  `state` is the
    oracle's restatement of RL_interface_init (oracle.rl_oracle.rl_init);
    buffers and cuFFT plans are made once here, as the plans are in
    RL_interface_init.  step() takes the cropped stack as a float32 device
    tensor (the reference converts u16 to float on the host) and writes the
    result into a device tensor of out_shape."""

    def __init__(self, state):
        from oracle import rl_oracle as O
        L = _load()
        if L is None:
            raise RuntimeError(_why)
        nz, ny, nx = state.output_nz, state.output_ny, state.output_nx
        desk = abs(state.deskewFactor) > 0.0
        gx = state.deskewedXdim if desk else nx
        kxs, kys, kzs = O.kscales(state, gx, ny, nz)
        otf = np.ascontiguousarray(state.otf, np.complex64)
        if otf.ndim == 2:
            nxo, nyo, nzo = otf.shape[0], 1, otf.shape[1]
        else:
            nzo, nyo, nxo = otf.shape
        self._otf = otf.view(np.float32).reshape(-1)
        rot = None
        nxr, nzr = gx, nz
        if state.rot is not None:
            rot = np.ascontiguousarray(state.rot, np.float32)
            nxr, nzr = O.rotated_dims(gx, nz, rot)
        self._rot = rot
        self.raw_shape = (nz, ny, nx)
        self.grid = (nz, ny, gx)
        self.out_shape = (nzr, ny, nxr)
        self.h = L.ref_session_open(nx, ny, nz, float(state.deskewFactor), int(gx),
                                    self._otf.ctypes.data_as(_fp), nxo, nyo, nzo, float(kxs),
                                    float(kys), float(kzs),
                                    rot.ctypes.data_as(_fp) if rot is not None else None,
                                    int(nxr), int(nzr))
        if self.h < 0:
            raise RuntimeError(f"ref_session_open: {L.ref_last_error().decode()}")

    def step(self, d_raw, background, n_iters, d_out):
        _check(_load().ref_session_step(self.h, d_raw.data_ptr(), float(background),
                                        int(n_iters), d_out.data_ptr()), "ref_session_step")

    def close(self):
        L = _load()
        if L is not None and self.h >= 0:
            L.ref_session_close(self.h)
            self.h = -1
