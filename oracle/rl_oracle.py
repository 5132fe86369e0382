"""ORACLE — test infrastructure only.

CPU restatement of the reference's Richardson-Lucy path (scopetools/cudadecon).
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
import this module; the product never does.

Every function follows the reference code it names, in the same order of
operations and with C's float/double evaluation rules written out (np.float32
for C `float`, Python floats for C `double`).  The geometry kernels (deskew,
rotate, camcor) come from geom_oracle.c, built by oracle/build.py.  FFTs use
scipy.fft (pocketfft): FFTW, which the reference uses on the CPU, is not
available here, and cuFFT is what the reference uses on the GPU; both compute
the same unnormalised DFT, so only rounding differs.

dtype=np.float32 reproduces the reference's single-precision iteration;
dtype=np.float64 is the FP64 oracle the precision targets are measured against.

Parity status: pinned.  The reference ships no golden vectors, so its own
CUDA kernels (compiled from its sources by oracle/build.py) were run with
cuFFT on a GB300 through oracle/ref_runner.cu: deskew, rotate, camcor and
affine outputs and two RL runs (64x256x256 plain; 100x256x756 deskewed stage
scan) are committed as fixtures in tests/golden/ (tests/golden/make_golden.py),
and tests/test_golden_cpu.py checks this restatement against them.
tests/test_ref_pin.py repeats the comparison live when that build is present.
"""

from __future__ import annotations

import ctypes
import math
import os
from dataclasses import dataclass, field

import numpy as np
import scipy.fft as sfft

from . import build as _obuild

F32 = np.float32
FLT_EPS = float(np.finfo(np.float32).eps)

_libm = ctypes.CDLL("libm.so.6")
_libm.cosf.restype = ctypes.c_float
_libm.cosf.argtypes = [ctypes.c_float]
_libm.sinf.restype = ctypes.c_float
_libm.sinf.argtypes = [ctypes.c_float]

_GEOM = None


def geom_lib():
    """ctypes handle of the C geometry oracle (built on first use)."""
    global _GEOM
    if _GEOM is None:
        p = _obuild.build_geom()
        L = ctypes.CDLL(str(p))
        fp = ctypes.POINTER(ctypes.c_float)
        up = ctypes.POINTER(ctypes.c_uint16)
        L.oracle_deskew.argtypes = [fp, ctypes.c_int, ctypes.c_int, ctypes.c_int, fp, ctypes.c_int,
                                    ctypes.c_int, ctypes.c_double, ctypes.c_float, ctypes.c_int]
        L.oracle_rotate.argtypes = [fp, ctypes.c_int, ctypes.c_int, ctypes.c_int, fp, ctypes.c_int,
                                    ctypes.c_int, fp, ctypes.c_int]
        L.oracle_camcor.argtypes = [up, ctypes.c_int, ctypes.c_int, ctypes.c_int, fp, up,
                                    ctypes.c_int]
        _GEOM = L
    return _GEOM


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


# ---------------------------------------------------------------- sizes
def not_good_dimension(num: int) -> bool:
    """RL-Biggs-Andrews.cpp:18-31 (sizes below 2 are treated as not good)."""
    if num in (2, 3, 5, 7):
        return False
    if num < 2:
        return True
    for p in (2, 3, 5, 7):
        if num % p == 0:
            return not_good_dimension(num // p)
    return True


def find_optimal_dimension(n: int, step: int = -1) -> int:
    """RL-Biggs-Andrews.cpp:33-43; returns 0 when no good size >= 2 exists."""
    out = n
    while out >= 2 and not_good_dimension(out):
        out += step
    return out if out >= 2 else 0


# ---------------------------------------------------------------- geometry oracles
def deskew(stack, deskew_factor, nx_out, extra_shift=0, pad_val=0.0, contract=1):
    """deskew_kernel (geometryTransform.cu:4-31) on a (nz, ny, nx) float32 stack."""
    a = np.ascontiguousarray(stack, dtype=np.float32)
    nz, ny, nx = a.shape
    out = np.empty((nz, ny, nx_out), dtype=np.float32)
    geom_lib().oracle_deskew(_fp(a), nx, ny, nz, _fp(out), int(nx_out), int(extra_shift),
                             float(deskew_factor), float(pad_val), int(contract))
    return out


def rotate(stack, rot4, nx_out, nz_out, contract=1):
    """rotate_kernel (geometryTransform.cu:50-88)."""
    a = np.ascontiguousarray(stack, dtype=np.float32)
    nz, ny, nx = a.shape
    r = np.ascontiguousarray(rot4, dtype=np.float32)
    out = np.empty((nz_out, ny, nx_out), dtype=np.float32)
    geom_lib().oracle_rotate(_fp(a), nx, ny, nz, _fp(out), int(nx_out), int(nz_out), _fp(r),
                             int(contract))
    return out


def camcor(raw, camparam, contract=1):
    """camcor_kernel (camcor.cu:80-108); camparam is (3, ny, nx): a, b, offset."""
    a = np.ascontiguousarray(raw, dtype=np.uint16)
    nz, ny, nx = a.shape
    p = np.ascontiguousarray(camparam, dtype=np.float32)
    out = np.empty_like(a)
    up = ctypes.POINTER(ctypes.c_uint16)
    geom_lib().oracle_camcor(a.ctypes.data_as(up), nx, ny, nz, _fp(p), out.ctypes.data_as(up),
                             int(contract))
    return out


def rotated_dims(nx, nz, rot4):
    """Output sizes of the rotation (RL-Biggs-Andrews.cpp:410-411)."""
    p = [F32(v) for v in rot4]
    nz_r = int(F32(F32(nz) * p[3]) / p[0])
    nx_r = int(F32(F32(nx) * p[3]) + F32(F32(F32(F32(nz) * p[2]) * p[2]) / F32(abs(p[1]))))
    return nx_r, nz_r


def reported_dims(state):
    """get_output_nx/nz (RL-Biggs-Andrews.cpp:474-503), with the signed p[1]."""
    if state.rot is None:
        return state.deskewedXdim, state.output_nz
    p = [F32(v) for v in state.rot]
    nx_r = int(F32(F32(state.deskewedXdim) * p[3]) +
               F32(F32(F32(F32(state.output_nz) * p[2]) * p[2]) / p[1]))
    nz_r = int(F32(F32(state.output_nz) * p[3]) / p[0])
    return nx_r, nz_r


# ---------------------------------------------------------------- init
@dataclass
class InitState:
    output_nx: int
    output_ny: int
    output_nz: int
    bCrop: bool
    deskewFactor: float
    deskewedXdim: int
    rot: np.ndarray | None
    dr: np.float32
    dz: np.float32
    dkx_otf: np.float32
    dky_otf: np.float32
    dkz_otf: np.float32
    nx_otf: int
    ny_otf: int
    nz_otf: int
    otf: np.ndarray  # complex64: (nr, nzotf) radial table or (nz_otf, ny_otf, nx_otf) 3D
    skewed: bool
    bleach: dict = field(default_factory=lambda: {"i0": 0.0, "first": True})


def rl_init(nx, ny, nz, dr, dz, dr_psf, dz_psf, deskewAngle, rotationAngle, outputWidth,
            bSkewedDecon, otf_img) -> InitState:
    """RL_interface_init (RL-Biggs-Andrews.cpp:531-655).

    otf_img is the OTF file content as a (depth, height, width) float32
    array, i.e. in CImg order."""
    dr, dz, dr_psf, dz_psf = F32(dr), F32(dz), F32(dr_psf), F32(dz_psf)
    deskewAngle, rotationAngle = F32(deskewAngle), F32(rotationAngle)
    bCrop = False
    out_ny = find_optimal_dimension(ny)
    bCrop |= out_ny != ny
    out_nz = find_optimal_dimension(nz)
    bCrop |= out_nz != nz
    out_nx = nx
    if not abs(float(deskewAngle)) > 0.0:
        out_nx = find_optimal_dimension(nx)
        bCrop |= out_nx != nx
    img = np.asarray(otf_img, dtype=np.float32)
    if img.ndim == 2:
        img = img[None]
    d, h, w = img.shape
    if bSkewedDecon:
        dz_psf = F32(float(dz_psf) * abs(math.sin(float(deskewAngle) * math.pi / 180.)))
    # determine_OTF_dimensions (RL-Biggs-Andrews.cpp:506-529)
    if d > 1:
        nx_otf, ny_otf, nz_otf = w // 2, h, d
        otf = img.reshape(d, h, w).view(np.complex64)  # (nz_otf, ny_otf, nx_otf)
    else:
        nx_otf, ny_otf, nz_otf = h, 1, w // 2
        otf = img.reshape(h, w).view(np.complex64)  # (nr, nzotf)
    dkx_otf = F32(1) / F32(F32((nx_otf - 1) * 2) * dr_psf)
    dky_otf = F32(1) / F32(F32(ny_otf) * dr_psf) if ny_otf > 1 else dkx_otf
    dkz_otf = F32(1) / F32(F32(nz_otf) * dz_psf)
    deskewFactor = 0.0
    deskewedXdim = out_nx
    if abs(float(deskewAngle)) > 0.0:
        if deskewAngle < 0:
            deskewAngle = F32(float(deskewAngle) + 180.)
        ang = float(deskewAngle) * math.pi / 180.
        deskewFactor = math.cos(ang) * float(dz) / float(dr)
        if outputWidth == 0:
            t = float(F32(F32(out_nz) * dz)) * abs(math.cos(ang)) / float(dr)
            deskewedXdim = int(deskewedXdim + math.floor(t))
        else:
            deskewedXdim = int(outputWidth)
        deskewedXdim = find_optimal_dimension(deskewedXdim)
        dz = F32(float(dz) * abs(math.sin(ang)))
    rot = None
    if abs(float(rotationAngle)) > 0.0:
        ra = F32(float(rotationAngle) * (math.pi / 180))
        stretch = F32(dr / dz)
        rot = np.array([F32(_libm.cosf(ra)) * stretch, F32(_libm.sinf(ra)) * stretch,
                        -F32(_libm.sinf(ra)), F32(_libm.cosf(ra))], dtype=np.float32)
    return InitState(out_nx, out_ny, out_nz, bCrop, deskewFactor, deskewedXdim, rot, dr, dz,
                     dkx_otf, dky_otf, dkz_otf, nx_otf, ny_otf, nz_otf, otf, bool(bSkewedDecon))


def kscales(state: InitState, gx, gy, gz):
    """transferConstants' k-scales for a decon grid (RL-Biggs-Andrews.cpp:634-642)."""
    dkx = F32(1.0 / float(F32(state.dr * F32(gx))))
    dky = F32(1.0 / float(F32(state.dr * F32(gy))))
    dkz = F32(1.0 / float(F32(state.dz * F32(gz))))
    return dkx / state.dkx_otf, dky / state.dky_otf, dkz / state.dkz_otf


def otf_on_grid(state: InitState, gx, gy, gz, dtype=np.float32):
    """makeOTFarray_kernel + dev_otfinterpolate (RLgpuImpl.cu:228-366): the
    OTF at every bin of the (gz, gy, gx//2+1) half spectrum."""
    ft = np.dtype(dtype).type
    kxs, kys, kzs = (ft(v) for v in kscales(state, gx, gy, gz))
    nxh = gx // 2 + 1
    kx = np.arange(nxh, dtype=ft) * kxs
    yy = np.arange(gy)
    ky = np.where(yy > gy >> 1, yy - gy, yy).astype(ft) * kys
    zz = np.arange(gz)
    kz = np.where(zz > gz >> 1, zz - gz, zz).astype(ft) * kzs
    otf = state.otf.astype(np.complex128 if ft is np.float64 else np.complex64)
    nzotf = ft(state.nz_otf)
    kzi = np.where(kz < 0, kz + nzotf, kz)
    if state.ny_otf == 1:
        nr = state.nx_otf
        kr = np.sqrt(kx[None, :] ** 2 + ky[:, None] ** 2).astype(ft)  # (gy, nxh)
        KR = np.broadcast_to(kr[None], (gz, gy, nxh))
        KZ = np.broadcast_to(kzi[:, None, None], (gz, gy, nxh))
        valid = (KR < ft(nr - 1)) & (KZ < nzotf) & (KZ >= 0)
        ir = np.where(valid, np.floor(KR), 0).astype(np.int64)
        iz = np.where(valid, np.floor(KZ), 0).astype(np.int64)
        ar = (KR - ir.astype(ft)).astype(ft)
        az = (KZ - iz.astype(ft)).astype(ft)
        iz1 = np.where(iz == state.nz_otf - 1, 0, iz + 1)
        ir1 = np.minimum(ir + 1, nr - 1)
        one = ft(1)
        v = (one - ar) * (otf[ir, iz] * (one - az) + otf[ir, iz1] * az) + \
            ar * (otf[ir1, iz] * (one - az) + otf[ir1, iz1] * az)
        return np.where(valid, v, 0)
    # non radially averaged OTF: trilinear with y/z wrap
    nxo, nyo = state.nx_otf, state.ny_otf
    kyi = np.where(ky < 0, ky + ft(nyo), ky)
    KX = np.broadcast_to(kx[None, None, :], (gz, gy, nxh))
    KY = np.broadcast_to(kyi[None, :, None], (gz, gy, nxh))
    KZ = np.broadcast_to(kzi[:, None, None], (gz, gy, nxh))
    valid = (KX < ft(nxo - 1)) & (KY < ft(nyo)) & (KZ < nzotf) & (KY >= 0) & (KZ >= 0)
    ix = np.where(valid, np.floor(KX), 0).astype(np.int64)
    iy = np.where(valid, np.floor(KY), 0).astype(np.int64)
    iz = np.where(valid, np.floor(KZ), 0).astype(np.int64)
    ax, ay, az = (KX - ix).astype(ft), (KY - iy).astype(ft), (KZ - iz).astype(ft)
    iy1, iz1 = (iy + 1) % nyo, (iz + 1) % state.nz_otf
    ix1 = np.minimum(ix + 1, nxo - 1)
    o = otf  # (nz_otf, ny_otf, nx_otf)
    one = ft(1)
    v = (one - az) * (o[iz, iy, ix] * (one - ay) * (one - ax) + o[iz, iy, ix1] * (one - ay) * ax +
                      o[iz, iy1, ix] * ay * (one - ax) + o[iz, iy1, ix1] * ay * ax) + \
        az * (o[iz1, iy, ix] * (one - ay) * (one - ax) + o[iz1, iy, ix1] * (one - ay) * ax +
              o[iz1, iy1, ix] * ay * (one - ax) + o[iz1, iy1, ix1] * ay * ax)
    return np.where(valid, v, 0)


# ---------------------------------------------------------------- conditioning
def apodize(img, napodize):
    """apodize_x_kernel then apodize_y_kernel (RLgpuImpl.cu:848-894), in place."""
    if napodize <= 0:
        return img
    nz, ny, nx = img.shape
    for z in range(nz):
        diff = ((img[z, ny - 1, :] - img[z, 0, :]).astype(np.float64) / 2.0).astype(np.float32)
        for l in range(napodize):
            w = 1.0 - math.sin(((float(F32(l)) + 0.5) / float(F32(napodize))) * math.pi * 0.5)
            fact = (diff.astype(np.float64) * w).astype(np.float32)
            img[z, l, :] += fact
            img[z, ny - 1 - l, :] -= fact
    for z in range(nz):
        diff = ((img[z, :, nx - 1] - img[z, :, 0]).astype(np.float64) / 2.0).astype(np.float32)
        for k in range(napodize):
            w = 1.0 - math.sin(((k + 0.5) / float(F32(napodize))) * math.pi * 0.5)
            fact = (diff.astype(np.float64) * w).astype(np.float32)
            img[z, :, k] += fact
            img[z, :, nx - 1 - k] -= fact
    return img


def bgsub(img, background):
    """bgsubtr_kernel (RLgpuImpl.cu:124-132)."""
    v = img - F32(background)
    return np.where(v > 0, v, F32(0)).astype(np.float32)


def mean_above_background(img):
    """meanAboveBackground_GPU (RLgpuImpl.cu:668-718)."""
    n = img.size
    s = float(np.sum(img, dtype=np.float64))
    mean = F32(s / n)
    m = img > mean
    s2 = float(np.sum(img[m], dtype=np.float64))
    return s2 / int(np.count_nonzero(m))


def zblend(img, nZblend):
    """zBlend_kernel (RLgpuImpl.cu:908-925) as the reference launches it: the
    slice index is blockDim.z == 1, so slices 1 and nz-2 are updated nZblend
    times (applied here one after the other)."""
    nz = img.shape[0]
    if nZblend <= 0 or nz < 3:
        return img
    w = 1.0 - math.sin(((1 + 0.5) / float(F32(nZblend))) * math.pi * 0.5)
    for _ in range(nZblend):
        diff = img[nz - 1] - img[0]
        fact = (diff.astype(np.float64) * w).astype(np.float32)
        img[1] += fact
        img[nz - 2] -= fact
    return img


# ---------------------------------------------------------------- RL
def rl_iterations(X0, raw, H, n_iters, dtype=np.float32, workers=None, lambdas=None,
                  norms=None):
    """The hot loop of RichardsonLucy_GPU (RL-Biggs-Andrews.cpp:282-367).

    X0, raw: (nz, ny, nx) arrays; H: the OTF on the half-spectrum grid.
    Returns the final estimate.  When lambdas is a list, the acceleration
    factor of each iteration k > 1 is appended to it.  When norms is a list,
    the relative change of each iteration, ||X_{k+1} - X_k|| / ||X_k||
    (float64 sums; the reference computes none), is appended to it."""
    ft = np.dtype(dtype).type
    workers = workers or os.cpu_count()
    shape = X0.shape
    X = np.array(X0, dtype=dtype)
    rawb = np.array(raw, dtype=dtype)
    Hc = H.astype(np.complex128 if ft is np.float64 else np.complex64)
    eps = ft(FLT_EPS)
    Xm1 = np.zeros_like(X)
    G1 = np.zeros_like(X)
    G2 = np.zeros_like(X)

    def conv(a, conj):
        F = sfft.rfftn(a, workers=workers)
        F *= np.conj(Hc) if conj else Hc
        return sfft.irfftn(F, s=shape, workers=workers).astype(dtype, copy=False)

    for k in range(n_iters):
        if k > 1:
            # calcAccelFactor (RLgpuImpl.cu:510-569): products in the working
            # precision, sums in double; lambda clamped to [0,1] and used as float
            num = float(np.sum((G1 * G2).astype(dtype), dtype=np.float64))
            den = float(np.sum((G2 * G2).astype(dtype), dtype=np.float64))
            lam = num / (den + FLT_EPS)
            lam = 1.0 if 1.0 < lam else lam
            lam = 0.0 if lam < 0.0 else lam
            if lambdas is not None:
                lambdas.append(lam)
            lamf = ft(F32(lam)) if ft is np.float32 else ft(lam)
            Y = X + lamf * (X - Xm1)
            Y = np.where(Y > 0, Y, ft(0)).astype(dtype)
        else:
            Y = X.copy()
        Xm1 = X
        if k > 0:
            G2 = G1
        CC = conv(Y, False)
        CC = np.where(np.abs(CC) > 0, CC, eps)
        CC = (rawb / CC + eps).astype(dtype)
        CC = np.clip(CC, ft(-10), ft(10))
        CC = conv(CC, True)
        X = (CC * Y).astype(dtype)
        X = np.where(X > 0, X, ft(0)).astype(dtype)
        G1 = (X - Y).astype(dtype)
        if norms is not None:
            d = X.astype(np.float64) - Xm1.astype(np.float64)
            o = float(np.sum(Xm1.astype(np.float64) ** 2))
            norms.append(float(np.sqrt(np.sum(d * d) / o)) if o > 0 else 0.0)
    return X


def rl_interface(state: InitState, raw_u16, background=100.0, bDoRescale=False,
                 bSaveDeskewedRaw=False, nIters=10, extraShift=0, napodize=0, nZblend=0,
                 padVal=0.0, bDupRevStack=False, bSkewedDecon=False, dtype=np.float32,
                 workers=None, lambdas=None):
    """RL_interface + RichardsonLucy_GPU (RL-Biggs-Andrews.cpp:56-450, 657-705).

    Returns (result, deskewed_raw_or_None) as (nz, ny, nx) float arrays with
    the sizes the library writes (the rotated result is cut to the
    get_output_n* sizes when those are smaller)."""
    s = state
    nx0, ny, nz0 = s.output_nx, s.output_ny, s.output_nz
    X = np.asarray(raw_u16)[:nz0, :ny, :nx0].astype(np.float32)
    save_desk = bSaveDeskewedRaw and abs(s.deskewFactor) > 0.0
    desk_out = None
    pre = nIters > 0 or save_desk or s.rot is not None
    nx, nz = nx0, nz0
    if pre:
        X = apodize(X, napodize)
        X = bgsub(X, background)
        if bDoRescale:
            inten = mean_above_background(X)
            if s.bleach["first"]:
                s.bleach["i0"] = inten
                s.bleach["first"] = False
            else:
                ratio = F32(s.bleach["i0"] / inten)
                X = (X.astype(np.float64) * float(ratio)).astype(np.float32)
        deskew_now = (not bSkewedDecon or (save_desk and nIters == 0)) and abs(s.deskewFactor) > 0
        if deskew_now:
            nx = s.deskewedXdim
            X = deskew(X, s.deskewFactor, nx, extraShift, padVal)
            if save_desk:
                desk_out = X.copy()
                if nIters == 0:
                    return X, desk_out
        X = zblend(X, nZblend)
        if bDupRevStack:
            X = np.concatenate([X, X[::-1]], axis=0)
            nz *= 2
    if nIters > 0:
        if bSkewedDecon and abs(s.deskewFactor) > 0:
            gx = nx  # decon on the skewed grid
        else:
            gx = nx
        H = otf_on_grid(s, gx, ny, nz, dtype=dtype)
        X = rl_iterations(X, X, H, nIters, dtype=dtype, workers=workers, lambdas=lambdas)
        X = np.asarray(X, dtype=np.float32) if dtype == np.float32 else X
    if bDupRevStack and pre:
        nz //= 2
        X = X[:nz]
    if bSkewedDecon and abs(s.deskewFactor) > 0.0:
        X = deskew(np.asarray(X, np.float32), s.deskewFactor, s.deskewedXdim, extraShift, 0.0)
        nx = s.deskewedXdim
    if s.rot is not None:
        nxr, nzr = rotated_dims(nx, nz, s.rot)
        X = rotate(np.asarray(X, np.float32), s.rot, nxr, nzr)
        rnx, rnz = reported_dims(s)
        if nxr * ny * nzr > rnx * ny * rnz:
            X = X.reshape(-1)[: rnx * ny * rnz].reshape(rnz, ny, rnx)
    return X, desk_out


# ---------------------------------------------------------------- affine
def affine(stack, mat4x4, ra=False, dx=1.0, dy=1.0, dz=1.0):
    """transformKernel / transformKernelRA (geometryTransform.cu:183-253):
    trilinear texture fetch with zero border at M*(x, y, z, 1) (+0.5 in the
    non-RA form; world coordinates with voxel size (dx, dy, dz) in the RA
    form).  The texture unit's interpolation weights have 8 fractional bits
    (CUDA Programming Guide, texture fetching); they are rounded to that
    grid here, which reproduces the hardware to within about 5e-3 of the
    data range, not bit for bit."""
    a = np.asarray(stack, dtype=np.float64)
    nz, ny, nx = a.shape
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    m = np.asarray(mat4x4, dtype=np.float32).reshape(16)
    u, v, w = (c.astype(np.float32) for c in (x, y, z))
    if ra:
        u, v, w = ((0.5 + (c.astype(np.float64) - 0.5) * float(F32(d))).astype(np.float32)
                   for c, d in ((u, dx), (v, dy), (w, dz)))
    t = []
    for r in range(3):
        s = (F32(m[4 * r]) * u + F32(m[4 * r + 1]) * v + F32(m[4 * r + 2]) * w + F32(m[4 * r + 3]))
        t.append((s + F32(0.5)).astype(np.float32) if not ra else s.astype(np.float32))
    if ra:
        t = [(0.5 + (c.astype(np.float64) - 0.5) / float(F32(d))).astype(np.float32)
             for c, d in zip(t, (dx, dy, dz))]
    xb, yb, zb = (c.astype(np.float64) - 0.5 for c in t)
    i, j, k = (np.floor(c).astype(np.int64) for c in (xb, yb, zb))
    ax, ay, az = (np.round((c - f) * 256) / 256 for c, f in ((xb, i), (yb, j), (zb, k)))

    def T(kk, jj, ii):
        ok = (ii >= 0) & (ii < nx) & (jj >= 0) & (jj < ny) & (kk >= 0) & (kk < nz)
        return np.where(ok, a[np.clip(kk, 0, nz - 1), np.clip(jj, 0, ny - 1), np.clip(ii, 0, nx - 1)], 0)

    out = ((1 - az) * ((1 - ay) * ((1 - ax) * T(k, j, i) + ax * T(k, j, i + 1)) +
                       ay * ((1 - ax) * T(k, j + 1, i) + ax * T(k, j + 1, i + 1))) +
           az * ((1 - ay) * ((1 - ax) * T(k + 1, j, i) + ax * T(k + 1, j, i + 1)) +
                 ay * ((1 - ax) * T(k + 1, j + 1, i) + ax * T(k + 1, j + 1, i + 1))))
    return out.astype(np.float32)


def otfinterpolate(otf, kx, ky, kz):
    """otfinterpolate (linearDecon.cpp:78-114), vectorised: bilinear
    interpolation of the radial table otf (nr, nzotf) at the (sub-pixel)
    OTF coordinates (kx, ky, kz), kz wrapping; 0 outside the table."""
    nr, nzotf = otf.shape
    kx, ky, kz = (np.asarray(a, dtype=F32) for a in (kx, ky, kz))
    krindex = np.sqrt((kx * kx + ky * ky).astype(F32)).astype(F32)
    kzindex = np.where(kz < 0, (kz + F32(nzotf)).astype(F32), kz)
    inside = (krindex < nr - 1) & (kzindex < nzotf)
    ir = np.where(inside, np.floor(krindex), 0).astype(np.int64)
    iz = np.where(inside, np.floor(kzindex), 0).astype(np.int64)
    ar = (krindex - ir).astype(np.float64)
    az = (kzindex - iz).astype(np.float64)
    iz1 = np.where(iz == nzotf - 1, 0, iz + 1)
    o = otf.astype(np.complex128)
    v = (1 - ar) * (o[ir, iz] * (1 - az) + o[ir, iz1] * az) + ar * (o[ir + 1, iz] * (1 - az)
                                                                  + o[ir + 1, iz1] * az)
    return np.where(inside, v, 0)


def wiener(state: InitState, img, background, wiener_const, NA, wavelength):
    """One-step Wiener filter of the reference's CLI (wienerfilter,
    linearDecon.cpp:116-168, applied at 1116-1127) on a float32 (nz, ny, nx)
    volume on the decon grid, with the OTF and pixel sizes of `state`."""
    x = np.asarray(img, dtype=F32) - F32(background)
    nz, ny, nx = x.shape
    dkx = F32(1.0 / (float(state.dr) * nx))
    dky = F32(1.0 / (float(state.dr) * ny))
    dkz = F32(1.0 / (float(state.dz) * nz))
    kxscale = F32(dkx / state.dkx_otf)
    kyscale = F32(dky / state.dkx_otf)
    kzscale = F32(dkz / state.dkz_otf)
    rcutoff = F32(2 * F32(NA) / F32(wavelength))
    w = F32(wiener_const) * F32(wiener_const)
    kz = np.arange(nz)
    kz = np.where(kz > nz // 2, kz - nz, kz).astype(F32)[:, None, None]
    ky = np.arange(ny)
    ky = np.where(ky > ny // 2, ky - ny, ky).astype(F32)[None, :, None]
    kx = np.arange(nx // 2 + 1).astype(F32)[None, None, :]
    kr = np.sqrt((kx * kx * dkx * dkx + ky * ky * dky * dky).astype(F32)).astype(F32)
    kr = np.broadcast_to(kr, (nz, ny, nx // 2 + 1))
    o = otfinterpolate(state.otf, np.broadcast_to(kx * kxscale, kr.shape),
                       np.broadcast_to(ky * kyscale, kr.shape), np.broadcast_to(kz * kzscale, kr.shape))
    amp2 = np.abs(o) ** 2
    rho = kr.astype(np.float64) / float(rcutoff)
    H = np.where(kr <= rcutoff, np.conj(o) * (1 - rho) / (amp2 + float(w)), 0)
    G = np.fft.rfftn(x.astype(np.float64))
    return np.fft.irfftn(G * H, s=x.shape, axes=tuple(range(x.ndim))).astype(np.float32)


def tiling(ny, tile_requested, tile_overlap_requested):
    """Tiling setup of the CLI (linearDecon.cpp:498-519): (tile_size, number
    of tiles, overlap (double), y offsets)."""
    if tile_requested == 0:
        return ny, 1, 0.0, [0]
    tile = min(128, ny) if tile_requested < 0 else min(tile_requested, ny)
    n = math.ceil(ny / (tile - tile_overlap_requested))
    overlap = math.floor((tile * n - ny) / (n - 1)) if n > 1 else 0.0
    offs = [math.floor(t * (tile - overlap)) for t in range(n)]
    return tile, n, float(overlap), offs


def tile_crop(raw, y0, tile):
    """Rows y0 .. y0+tile-1 of a (nz, ny, nx) stack; rows past the stack repeat
    its last row (CImg get_crop with boundary conditions)."""
    ny = raw.shape[1]
    idx = np.clip(np.arange(y0, y0 + tile), 0, ny - 1)
    return np.ascontiguousarray(raw[:, idx, :])


def stitch_tiles(tiles, offs, ny_out, overlap, blend_on):
    """Stitching of the CLI (linearDecon.cpp:1175-1245) of processed tiles
    (each (nz, tny, nx) float32) at y offsets offs into (nz, ny_out, nx)."""
    if len(tiles) == 1:
        return tiles[0].copy()
    nz, tny, nx = tiles[0].shape
    out = np.zeros((nz, ny_out, nx), dtype=np.float32)
    w = np.zeros((nz, ny_out, nx), dtype=bool)
    no_zone = math.ceil((overlap - 4) / 2.0)
    blend_zone = int(overlap - no_zone - no_zone)
    n = len(tiles)
    for t, (img, yoff) in enumerate(zip(tiles, offs)):
        first, last = t == 0, t + 1 >= n
        for y in range(tny):
            if first and y <= overlap:
                b = F32(1)
            elif last and y >= tny - overlap:
                b = F32(1)
            elif y <= no_zone:
                b = F32(0)
            elif no_zone < y <= no_zone + blend_zone:
                b = F32((y - no_zone) / blend_zone)
            elif y >= tny - no_zone:
                b = F32(0)
            else:
                b = F32(1)
            yo = y + yoff
            if yo >= ny_out:
                continue
            v = img[:, y, :]
            if blend_on:
                cur, ww = out[:, yo, :], w[:, yo, :]
                if 0 < b < 1:
                    mixed = ((v * b).astype(np.float64) + cur.astype(np.float64) * (1.0 - float(b))).astype(F32)
                    out[:, yo, :] = np.where(ww, mixed, v)
                elif b == 1:
                    out[:, yo, :] = v
                if b > 0:
                    w[:, yo, :] = True
            else:
                past_front = y >= math.floor(float(F32(overlap)) / 2.0) or first
                before_end = y < math.floor(tny - float(F32(overlap)) / 2.0) or last
                if past_front and before_end:
                    out[:, yo, :] = v
    return out
