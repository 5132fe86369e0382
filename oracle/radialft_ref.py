"""ORACLE — test infrastructure only.

The reference's own makeOTF (src/radialft_interface.cpp:95-197 of
scopetools/cudadecon), compiled from its source where it lies by
oracle/build.py (build_radialft_ref) into oracle/_ref/libradialft_ref.so,
with stand-ins for the two libraries it needs that this image lacks:
oracle/shim/fftw3.h (its in-place 3D real-to-complex FFT, computed as direct
DFTs in double precision) and oracle/shim/tiffio.h (CImg's TIFF writer;
makeOTF's output is captured in memory instead of written).  The PSF is
handed to makeOTF as a .cimg file.  Only where the reference checkout is
present (the fixture generator tests/golden/make_otf_golden.py uses it);
`available()` says whether it can be used.
"""

from __future__ import annotations

import ctypes
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_ref" / "libradialft_ref.so"
_L = None


def available() -> bool:
    return LIB.exists()


def _lib():
    global _L
    if _L is None:
        L = ctypes.CDLL(str(LIB))
        L.makeOTF.restype = ctypes.c_int
        L.makeOTF.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_float,
                              ctypes.c_int, ctypes.c_bool, ctypes.c_float, ctypes.c_float,
                              ctypes.c_float, ctypes.c_float, ctypes.c_int, ctypes.c_bool,
                              ctypes.c_bool]
        L.cdx_tiff_captured.restype = ctypes.c_int
        L.cdx_tiff_captured.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                        ctypes.POINTER(ctypes.c_int),
                                        ctypes.POINTER(ctypes.c_float), ctypes.c_long]
        _L = L
    return _L


def make_otf(psf, lambdanm=520, dz=0.102, interpkr=10, user_background=None, NA=1.25,
             NIMM=1.3, dr=0.102, krmax=0, do_cleanup=False, out_3d=False):
    """makeOTF on a (nz, ny, nx) PSF with the reference's defaults
    (radialft_interface.cpp:52-58).  Returns the complex table (nx/2+1, nz),
    or with out_3d the half spectrum (nz, ny, nx/2+1)."""
    from cudadecon_gb300 import synth
    L = _lib()
    psf = np.ascontiguousarray(psf, np.float32)
    with tempfile.TemporaryDirectory() as td:
        src = Path(td) / "psf.cimg"
        synth.write_cimg(src, psf)
        rc = L.makeOTF(str(src).encode(), str(Path(td) / "otf.tif").encode(), int(lambdanm),
                       float(dz), int(interpkr), user_background is not None,
                       float(user_background if user_background is not None else 90.0),
                       float(NA), float(NIMM), float(dr), int(krmax), bool(do_cleanup),
                       bool(out_3d))
    if rc != 0:
        raise RuntimeError(f"makeOTF returned {rc}")
    w, h = ctypes.c_int(), ctypes.c_int()
    n = L.cdx_tiff_captured(-1, ctypes.byref(w), ctypes.byref(h), None, 0)
    planes = []
    for i in range(n):
        L.cdx_tiff_captured(i, ctypes.byref(w), ctypes.byref(h), None, 0)
        buf = np.empty(w.value * h.value, np.float32)
        L.cdx_tiff_captured(i, ctypes.byref(w), ctypes.byref(h),
                            buf.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), buf.size)
        planes.append(buf.reshape(h.value, w.value))
    img = np.stack(planes)
    cplx = img.view(np.complex64)
    return cplx if out_3d else cplx[0]
