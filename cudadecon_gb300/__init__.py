"""cudadecon_gb300: GB300-native Richardson-Lucy deconvolution with the cudaDecon C ABI.

The product is the in-tree shared library ``lib/libcudaDecon.so`` (CUDA for
sm_103a plus C++ host code).  This module binds it with ctypes the way a
pycudadecon-style caller binds the reference library, and adds numpy helpers.
There is no CPU fallback: every function raises if the library is missing.

Reference ABI: scopetools/cudadecon src/linearDecon.h:243-317.
"""

from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_bool, c_char_p, c_double, c_float, c_int, c_longlong, c_size_t
from ctypes import c_uint, c_ushort, c_void_p
from pathlib import Path

import numpy as np

from . import _build
from . import synth

__all__ = [
    "lib",
    "build",
    "lib_path",
    "CudaDeconError",
    "rl_init",
    "rl_decon",
    "rl_cleanup",
    "set_dft_form",
    "dft_form",
    "output_shape",
    "deskew",
    "affine",
    "affine_ra",
    "camcor_init",
    "camcor",
    "load_image",
]

_LIB = None


class CudaDeconError(RuntimeError):
    """A library entry point returned failure (the message is cdx_last_error())."""


def lib_path() -> Path:
    return _build.lib_path()


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compile the CUDA library in-tree for sm_103a (nvcc required)."""
    global _LIB
    p = _build.build(verbose=verbose, force=force)
    return p


_F = POINTER(c_float)
_U16 = POINTER(c_ushort)


class BatchStack(ctypes.Structure):
    """struct cdx_batch_stack of include/cudadecon.h."""
    _fields_ = [("raw", c_void_p), ("nx", c_int), ("ny", c_int), ("nz", c_int),
                ("result", c_void_p), ("otf", _F), ("otf_w", c_int), ("otf_h", c_int),
                ("dr", c_float), ("dz", c_float), ("dr_psf", c_float), ("dz_psf", c_float),
                ("background", c_float)]


def _bind(L) -> None:
    sig = {
        # reference ABI (src/linearDecon.h:260-316)
        "RL_interface_init": (c_int, [c_int, c_int, c_int, c_float, c_float, c_float, c_float,
                                      c_float, c_float, c_int, c_bool, c_char_p]),
        "RL_interface": (c_int, [_U16, c_int, c_int, c_int, _F, _F, c_float, c_bool, c_bool,
                                 c_int, c_int, c_int, c_int, c_float, c_bool, c_bool]),
        "Deskew_interface": (c_int, [_F, c_int, c_int, c_int, c_float, c_float, c_float, _F,
                                     c_int, c_int, c_float]),
        "Affine_interface": (c_int, [_F, c_int, c_int, c_int, _F, _F]),
        "Affine_interface_RA": (c_int, [_F, c_int, c_int, c_int, c_float, c_float, c_float,
                                        _F, _F]),
        "camcor_interface_init": (c_int, [c_int, c_int, c_int, _F]),
        "camcor_interface": (c_int, [_U16, c_int, c_int, c_int, _U16]),
        "RL_cleanup": (None, []),
        "cuda_reset": (None, []),
        "get_output_nx": (c_uint, []),
        "get_output_ny": (c_uint, []),
        "get_output_nz": (c_uint, []),
        "get_version": (c_char_p, []),
        # extensions
        "cdx_last_error": (c_char_p, []),
        "cdx_RL_device": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p, c_float,
                                  c_bool, c_bool, c_int, c_int, c_int, c_int, c_float, c_bool,
                                  c_bool, c_void_p]),
        "cdx_last_launch_count": (c_longlong, []),
        "cdx_decon_grid": (c_int, [POINTER(c_int), POINTER(c_int), POINTER(c_int)]),
        "cdx_profile_enable": (c_int, [c_int]),
        "cdx_profile_read": (c_int, [POINTER(c_double), POINTER(c_longlong), c_int,
                                     POINTER(c_double), POINTER(c_longlong)]),
        "cdx_profile_pass_name": (c_char_p, [c_int]),
        "cdx_lambda_trace": (c_int, [c_int]),
        "cdx_set_dft_form": (c_int, [c_int]),
        "cdx_get_dft_form": (c_int, []),
        "cdx_tc_length_supported": (c_int, [c_int]),
        "cdx_tc_status": (c_int, []),
        "cdx_lambda_read": (c_int, [_F, c_int]),
        "cdx_change_trace": (c_int, [c_int]),
        "cdx_change_read": (c_int, [POINTER(c_double), c_int]),
        "cdx_deskew_device": (c_int, [c_void_p, c_int, c_int, c_int, c_double, c_void_p, c_int,
                                      c_int, c_float, c_void_p]),
        "cdx_rotate_device": (c_int, [c_void_p, c_int, c_int, c_int, _F, c_void_p, c_int, c_int,
                                      c_void_p]),
        "cdx_camcor_device": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p,
                                      c_void_p]),
        "cdx_rfft3d_device": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_void_p]),
        "cdx_conv3d_device": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_void_p]),
        "cdx_fft_length_supported": (c_int, [c_int]),
        "cdx_accel_factor_device": (c_int, [c_void_p, c_void_p, c_longlong, c_void_p, c_void_p,
                                            c_void_p]),
        "cdx_load_image": (c_int, [c_char_p, POINTER(c_int), POINTER(c_int), POINTER(c_int), _F,
                                   c_size_t]),
        "makeOTF": (c_int, [c_char_p, c_char_p, c_int, c_float, c_int, c_bool, c_float, c_float,
                            c_float, c_float, c_int, c_bool, c_bool]),
        "cdx_make_otf": (c_int, [_F, c_int, c_int, c_int, c_int, c_float, c_int, c_int, c_float,
                                 c_float, c_float, c_float, c_int, c_int, c_int, _F, c_size_t,
                                 POINTER(c_int), POINTER(c_int), POINTER(c_int)]),
        "cdx_save_image": (c_int, [c_char_p, c_int, c_int, c_int, _F]),
        "cdx_wiener_device": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_float, c_float,
                                      c_float, c_float, c_void_p]),
        "cdx_RL_tiled": (c_int, [_U16, c_int, c_int, c_int, _F, c_int, c_int, c_int, c_float,
                                 c_int, c_int, c_int, c_float]),
        "cdx_mip_device": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_void_p, c_void_p]),
        "cdx_batch_grid": (c_int, [c_int, c_int, c_int, POINTER(c_int), POINTER(c_int),
                                   POINTER(c_int)]),
        "cdx_RL_batch_device": (c_int, [POINTER(BatchStack), c_int, c_int, c_void_p]),
        "cdx_RL_batch_host": (c_int, [POINTER(BatchStack), c_int, c_int]),
        "cdx_batch_last_launch_count": (c_longlong, []),
        "cdx_batch_set_streams": (c_int, [c_int, c_int]),
        "cdx_batch_get_streams": (c_int, [POINTER(c_int), POINTER(c_int)]),
        "cdx_batch_release": (None, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args


def lib():
    """The loaded library (ctypes.CDLL); raises if it has not been built."""
    global _LIB
    if _LIB is None:
        p = lib_path()
        if not p.exists():
            raise CudaDeconError(
                f"{p} is missing: build it with cudadecon_gb300.build() "
                "(or __graft_entry__.build()); there is no CPU fallback")
        L = ctypes.CDLL(str(p), mode=os.RTLD_LOCAL if hasattr(os, "RTLD_LOCAL") else 0)
        _bind(L)
        _LIB = L
    return _LIB


def _err(what: str):
    msg = lib().cdx_last_error()
    raise CudaDeconError(f"{what} failed: {msg.decode() if msg else ''}")


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(_F)


def _u16ptr(a: np.ndarray):
    return a.ctypes.data_as(_U16)


# ---------------------------------------------------------------- RL
def rl_init(shape_zyx, otf_file, dr=0.104, dz=0.5, dr_psf=0.104, dz_psf=0.1, deskew_angle=0.0,
            rotation_angle=0.0, output_width=0, skewed_decon=False) -> None:
    """RL_interface_init for a raw stack of shape (nz, ny, nx)."""
    nz, ny, nx = (int(v) for v in shape_zyx)
    ok = lib().RL_interface_init(nx, ny, nz, dr, dz, dr_psf, dz_psf, deskew_angle,
                                 rotation_angle, int(output_width), bool(skewed_decon),
                                 str(otf_file).encode())
    if ok != 1:
        _err("RL_interface_init")


def decon_grid():
    """(nz, ny, nx) of the grid the RL iterations run on after the last rl_init."""
    x, y, z = c_int(0), c_int(0), c_int(0)
    if lib().cdx_decon_grid(ctypes.byref(x), ctypes.byref(y), ctypes.byref(z)) != 1:
        _err("cdx_decon_grid")
    return z.value, y.value, x.value


def output_shape():
    """(nz, ny, nx) of the RL_interface result after the last rl_init."""
    L = lib()
    return int(L.get_output_nz()), int(L.get_output_ny()), int(L.get_output_nx())


def rl_decon(raw: np.ndarray, background=100.0, n_iters=10, rescale=False, save_deskewed=False,
             extra_shift=0, napodize=0, nzblend=0, pad_val=0.0, dup_rev_stack=False,
             skewed_decon=False, deskewed_shape=None):
    """RL_interface on a (nz, ny, nx) uint16 stack; returns the float32 result
    (and the deskewed raw stack when save_deskewed)."""
    raw = np.ascontiguousarray(raw, dtype=np.uint16)
    nz, ny, nx = raw.shape
    out = np.zeros(output_shape(), dtype=np.float32)
    desk = None
    if save_deskewed:
        if deskewed_shape is None:
            raise ValueError("deskewed_shape is required with save_deskewed")
        desk = np.zeros(deskewed_shape, dtype=np.float32)
    ok = lib().RL_interface(_u16ptr(raw), nx, ny, nz, _fptr(out),
                            _fptr(desk) if desk is not None else None, background, bool(rescale),
                            bool(save_deskewed), int(n_iters), int(extra_shift), int(napodize),
                            int(nzblend), float(pad_val), bool(dup_rev_stack), bool(skewed_decon))
    if ok != 1:
        _err("RL_interface")
    return (out, desk) if save_deskewed else out


def rl_tiled(raw: np.ndarray, tile=128, tile_overlap=30, blend=False, background=100.0,
             n_iters=10, napodize=0, nzblend=0, pad_val=0.0):
    """cdx_RL_tiled on a (nz, ny, nx) uint16 stack (rl_init must have been
    called with the tile's ny); returns the stitched float32 result."""
    raw = np.ascontiguousarray(raw, dtype=np.uint16)
    nz, ny, nx = raw.shape
    L = lib()
    onz, _, onx = output_shape()
    out = np.zeros((onz, ny if tile else output_shape()[1], onx), dtype=np.float32)
    ok = L.cdx_RL_tiled(_u16ptr(raw), nx, ny, nz, _fptr(out), int(tile), int(tile_overlap),
                        int(bool(blend)), float(background), int(n_iters), int(napodize),
                        int(nzblend), float(pad_val))
    if ok != 1:
        _err("cdx_RL_tiled")
    return out


def mip(volume, axis):
    """cdx_mip_device on a (nz, ny, nx) float32 CUDA tensor; axis 0/1/2 = x/y/z."""
    import torch
    v = volume.contiguous().float()
    nz, ny, nx = v.shape
    shape = {0: (nz, ny), 1: (nz, nx), 2: (ny, nx)}[axis]
    out = torch.empty(shape, dtype=torch.float32, device=v.device)
    ok = lib().cdx_mip_device(c_void_p(v.data_ptr()), nx, ny, nz, int(axis), c_void_p(out.data_ptr()),
                              c_void_p(torch.cuda.current_stream().cuda_stream))
    if ok != 1:
        _err("cdx_mip_device")
    return out


def set_dft_form(form: str) -> None:
    """'plain' (FP32 CUDA-core FFT) or 'mixed' (tensor-core DFT stages in
    split TF32 for the x rows that have a tensor-core plan)."""
    code = {"plain": 0, "mixed": 1}[form]
    if lib().cdx_set_dft_form(code) != 1:
        _err("cdx_set_dft_form")


def dft_form() -> str:
    return "mixed" if lib().cdx_get_dft_form() == 1 else "plain"


def rl_cleanup() -> None:
    lib().RL_cleanup()


def wiener(stack, background=100.0, wiener=0.01, NA=1.2, wavelength=0.525, stream=None):
    """cdx_wiener_device on a (nz, ny, nx) float32 CUDA tensor (the decon grid
    of the last rl_init); returns the filtered CUDA tensor."""
    import torch
    x = stack.contiguous().float()
    nz, ny, nx = x.shape
    out = torch.empty_like(x)
    if stream is None:
        stream = torch.cuda.current_stream()
    ok = lib().cdx_wiener_device(c_void_p(x.data_ptr()), c_void_p(out.data_ptr()), nx, ny, nz,
                                 float(background), float(wiener), float(NA), float(wavelength),
                                 c_void_p(stream.cuda_stream))
    if ok != 1:
        _err("cdx_wiener_device")
    return out


# ---------------------------------------------------------------- OTF generation
_OTF_DEFAULTS = dict(lambdanm=520, dz=0.102, interpkr=10, background=None, NA=1.25, NIMM=1.3,
                     dr=0.102, krmax=0, cleanup=False, otf_3d=False)


def make_otf_file(psf_file, otf_file, **kw) -> None:
    """makeOTF: PSF file -> OTF file (the reference's libradialft entry point).
    background=None estimates it from the stack as the reference does."""
    a = dict(_OTF_DEFAULTS, **kw)
    rc = lib().makeOTF(str(psf_file).encode(), str(otf_file).encode(), int(a["lambdanm"]),
                       float(a["dz"]), int(a["interpkr"]), a["background"] is not None,
                       float(a["background"] or 0.0), float(a["NA"]), float(a["NIMM"]),
                       float(a["dr"]), int(a["krmax"]), bool(a["cleanup"]), bool(a["otf_3d"]))
    if rc != 0:
        _err("makeOTF")


def make_otf(psf: np.ndarray, **kw) -> np.ndarray:
    """cdx_make_otf on a (nz, ny, nx) PSF array.  Returns the OTF image as
    makeOTF writes it: (nx/2+1, 2*nz) float32 for the radial table (view it
    as complex64 for the (kr, kz) table), (nz, ny, 2*(nx/2+1)) for the 3D OTF."""
    a = dict(_OTF_DEFAULTS, **kw)
    p = np.ascontiguousarray(psf, dtype=np.float32)
    nz, ny, nx = p.shape
    L = lib()
    w, h, d = c_int(0), c_int(0), c_int(0)
    args = [int(a["lambdanm"]), float(a["dz"]), int(a["interpkr"]), int(a["background"] is not None),
            float(a["background"] or 0.0), float(a["NA"]), float(a["NIMM"]), float(a["dr"]),
            int(a["krmax"]), int(bool(a["cleanup"])), int(bool(a["otf_3d"]))]
    out = np.zeros((nz, ny, 2 * (nx // 2 + 1)) if a["otf_3d"] else (nx // 2 + 1, 2 * nz),
                   dtype=np.float32)
    ok = L.cdx_make_otf(_fptr(p), nx, ny, nz, *args, _fptr(out), out.size, ctypes.byref(w),
                        ctypes.byref(h), ctypes.byref(d))
    if ok != 1:
        _err("cdx_make_otf")
    return out


def save_image(path, img: np.ndarray) -> None:
    """cdx_save_image: write a float32 image ((depth,) height, width) as TIFF."""
    a = np.ascontiguousarray(img, dtype=np.float32)
    d, h, w = (1,) * (3 - a.ndim) + a.shape
    if lib().cdx_save_image(str(path).encode(), w, h, d, _fptr(a)) != 1:
        _err("cdx_save_image")


def batch_grid(shape_zyx):
    """(gz, gy, gx): the decon grid cdx_RL_batch_device uses for a stack."""
    nz, ny, nx = shape_zyx
    g = [c_int(0), c_int(0), c_int(0)]
    lib().cdx_batch_grid(nx, ny, nz, *(ctypes.byref(v) for v in g))
    return g[2].value, g[1].value, g[0].value


def rl_batch(stacks, n_iters=10, stream=None):
    """cdx_RL_batch_device on a list of stacks.  Each stack is a dict with
    `raw` (CUDA uint16 tensor, (nz, ny, nx)), `otf` ((nr, nz_otf) complex64
    radial table, host), `dr`, `dz`, `dr_psf`, `dz_psf` and `background`.
    Returns the float32 results (CUDA tensors on each stack's decon grid),
    complete when the work queued on `stream` (default: the current stream)
    after this call runs."""
    import torch
    L = lib()
    n = len(stacks)
    arr = (BatchStack * n)()
    keep, outs = [], []
    for i, d in enumerate(stacks):
        raw = d["raw"]
        nz, ny, nx = raw.shape
        gz, gy, gx = batch_grid((nz, ny, nx))
        out = torch.empty((gz, gy, gx), dtype=torch.float32, device=raw.device)
        img = np.ascontiguousarray(synth.otf_table_to_image(d["otf"]), dtype=np.float32)
        keep.append(img)
        outs.append(out)
        arr[i] = BatchStack(raw.data_ptr(), nx, ny, nz, out.data_ptr(), _fptr(img), img.shape[1],
                            img.shape[0], d.get("dr", 0.104), d.get("dz", 0.3),
                            d.get("dr_psf", 0.104), d.get("dz_psf", 0.1),
                            d.get("background", 100.0))
    if stream is None:
        stream = torch.cuda.current_stream()
    ok = L.cdx_RL_batch_device(arr, n, int(n_iters), c_void_p(stream.cuda_stream))
    if ok != 1:
        _err("cdx_RL_batch_device")
    return outs


def batch_streams(device=None, host=None):
    """Get, or set and get, the streams the batch spreads its stacks over
    (cdx_batch_set_streams): returns (device_streams, host_streams)."""
    L = lib()
    d, h = c_int(0), c_int(0)
    L.cdx_batch_get_streams(ctypes.byref(d), ctypes.byref(h))
    if device is not None or host is not None:
        nd = d.value if device is None else int(device)
        nh = h.value if host is None else int(host)
        if L.cdx_batch_set_streams(nd, nh) != 1:
            raise ValueError(L.cdx_last_error().decode())
        L.cdx_batch_get_streams(ctypes.byref(d), ctypes.byref(h))
    return d.value, h.value


def rl_batch_host(stacks, n_iters=10, results=None):
    """cdx_RL_batch_host: like rl_batch, but `raw` of each stack is a
    page-locked (pinned) CPU uint16 tensor and the results are written into
    pinned CPU float32 tensors (allocated here unless `results` gives them).
    Returns the results once they are complete."""
    import torch
    L = lib()
    n = len(stacks)
    arr = (BatchStack * n)()
    keep, outs = [], []
    for i, d in enumerate(stacks):
        raw = d["raw"]
        nz, ny, nx = raw.shape
        gz, gy, gx = batch_grid((nz, ny, nx))
        out = results[i] if results is not None else \
            torch.empty((gz, gy, gx), dtype=torch.float32).pin_memory()
        img = np.ascontiguousarray(synth.otf_table_to_image(d["otf"]), dtype=np.float32)
        keep.append(img)
        outs.append(out)
        arr[i] = BatchStack(raw.data_ptr(), nx, ny, nz, out.data_ptr(), _fptr(img), img.shape[1],
                            img.shape[0], d.get("dr", 0.104), d.get("dz", 0.3),
                            d.get("dr_psf", 0.104), d.get("dz_psf", 0.1),
                            d.get("background", 100.0))
    if L.cdx_RL_batch_host(arr, n, int(n_iters)) != 1:
        _err("cdx_RL_batch_host")
    return outs


# ---------------------------------------------------------------- geometry
def deskew(stack: np.ndarray, angle, dz, dr, output_width=0, extra_shift=0, pad_val=0.0,
           out_width=None):
    """Deskew_interface on a (nz, ny, nx) float32 stack.  The output width is
    output_width, or when 0 the reference's rule (see include/cudadecon.h);
    pass out_width to size the result buffer for that rule."""
    a = np.ascontiguousarray(stack, dtype=np.float32)
    nz, ny, nx = a.shape
    w = int(output_width) if output_width else int(out_width if out_width is not None else nx)
    out = np.zeros((nz, ny, w), dtype=np.float32)
    ok = lib().Deskew_interface(_fptr(a), nx, ny, nz, dz, dr, angle, _fptr(out),
                                int(output_width), int(extra_shift), float(pad_val))
    if ok != 1:
        _err("Deskew_interface")
    return out


def affine(stack: np.ndarray, mat4x4) -> np.ndarray:
    a = np.ascontiguousarray(stack, dtype=np.float32)
    m = np.ascontiguousarray(mat4x4, dtype=np.float32).reshape(16)
    nz, ny, nx = a.shape
    out = np.zeros_like(a)
    if lib().Affine_interface(_fptr(a), nx, ny, nz, _fptr(out), _fptr(m)) != 1:
        _err("Affine_interface")
    return out


def affine_ra(stack: np.ndarray, mat4x4, dx, dy, dz) -> np.ndarray:
    a = np.ascontiguousarray(stack, dtype=np.float32)
    m = np.ascontiguousarray(mat4x4, dtype=np.float32).reshape(16)
    nz, ny, nx = a.shape
    out = np.zeros_like(a)
    if lib().Affine_interface_RA(_fptr(a), nx, ny, nz, dx, dy, dz, _fptr(out), _fptr(m)) != 1:
        _err("Affine_interface_RA")
    return out


def camcor_init(shape_zyx, camparam: np.ndarray) -> None:
    """camcor_interface_init; camparam is (3, ny, nx) float32: a, b, offset."""
    nz, ny, nx = (int(v) for v in shape_zyx)
    p = np.ascontiguousarray(camparam, dtype=np.float32)
    if p.shape != (3, ny, nx):
        raise ValueError("camparam must have shape (3, ny, nx)")
    if lib().camcor_interface_init(nx, ny, nz, _fptr(p)) != 1:
        _err("camcor_interface_init")


def camcor(raw: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(raw, dtype=np.uint16)
    nz, ny, nx = a.shape
    out = np.zeros_like(a)
    if lib().camcor_interface(_u16ptr(a), nx, ny, nz, _u16ptr(out)) != 1:
        _err("camcor_interface")
    return out


def load_image(path) -> np.ndarray:
    """Read a TIFF / .cimg file as the library reads OTFs; returns (d, h, w) float32."""
    L = lib()
    w, h, d = c_int(0), c_int(0), c_int(0)
    if L.cdx_load_image(str(path).encode(), ctypes.byref(w), ctypes.byref(h), ctypes.byref(d),
                        None, 0) != 1:
        _err("cdx_load_image")
    out = np.zeros((d.value, h.value, w.value), dtype=np.float32)
    if L.cdx_load_image(str(path).encode(), None, None, None, _fptr(out), out.size) != 1:
        _err("cdx_load_image")
    return out
