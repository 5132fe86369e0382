"""ORACLE -- test infrastructure only.

CPU restatement of the reference's OTF generation, `makeOTF` of libradialft
(src/radialft_interface.cpp:95-197): PSF stack -> background-subtracted,
re-centred 3D FFT -> radially averaged (nx/2+1) x nz complex table, or the
3D OTF.  Only tests/ may import this module; the product never does.

Each function follows the reference function it names, with C's float /
double evaluation written out (np.float32 for `float`, Python floats for
`double`).  The FFT is numpy's (float64); the reference calls FFTW in float
(absent here), so results agree to FFT rounding, not bit for bit.

Parity status: pinned.  No golden OTF ships with the reference, so its own
makeOTF was run here (src/radialft_interface.cpp compiled from its source
with stand-ins for FFTW and libtiff, oracle/radialft_ref.py) on seeded PSFs
with the argument sets the tests use; its outputs are the fixtures in
tests/golden/golden_otf.npz (tests/golden/make_otf_golden.py), and this
restatement agrees with them to relative L2 below 1e-6
(tests/test_otf_cpu.py).  The tests also check it against analytic OTFs of
Gaussian beads.
"""

from __future__ import annotations

import math

import numpy as np

F32 = np.float32


def fitparabola(a1, a2, a3):
    """fitparabola (radialft_interface.cpp:270-284): vertex of the parabola
    through (-1, a1), (0, a2), (1, a3); 0 when flat or farther than 1.5."""
    a1, a2, a3 = F32(a1), F32(a2), F32(a3)
    slope = F32(0.5 * float(F32(a3 - a1)))
    curve = F32(F32(a3 + a1) - F32(2) * a2)
    if curve == 0:
        return F32(0)
    peak = F32(-slope / curve)
    if peak > 1.5 or peak < -1.5:
        return F32(0)
    return peak


def determine_center_and_background(stack):
    """determine_center_and_background (radialft_interface.cpp:199-262) on a
    (nz, ny, nx) float32 stack: peak pixel (first strict maximum above 0 in
    scan order), parabola-refined centre with the reference's +0.6 in z, and
    the mean of rows y < yc - 20 of the in-focus slice (divided by
    (yc - 20) * nx, as the reference does)."""
    st = np.asarray(stack, dtype=F32)
    nz, ny, nx = st.shape
    flat = st.ravel()
    m = int(np.argmax(flat))
    if not flat[m] > 0:
        maxk = maxi = maxj = 0
        maxval = F32(0)
    else:
        maxk, rem = divmod(m, ny * nx)
        maxi, maxj = divmod(rem, nx)
        maxval = flat[m]
    im, ip = (maxi - 1) % ny, (maxi + 1) % ny
    jm, jp = (maxj - 1) % nx, (maxj + 1) % nx
    km, kp = (maxk - 1) % nz, (maxk + 1) % nz
    zc = F32(F32(maxk) + fitparabola(st[km, maxi, maxj], maxval, st[kp, maxi, maxj]))
    zc = F32(float(zc) + 0.6)
    yc = F32(F32(maxi) + fitparabola(st[maxk, im, maxj], maxval, st[maxk, ip, maxj]))
    xc = F32(F32(maxj) + fitparabola(st[maxk, maxi, jm], maxval, st[maxk, maxi, jp]))
    s = 0.0
    zs = int(math.floor(float(zc)))
    i = 0
    while F32(i) < F32(yc - F32(20)):
        s += float(np.sum(st[zs, i, :].astype(np.float64)))
        i += 1
    den = F32(F32(yc - F32(20)) * F32(nx))
    with np.errstate(divide="ignore", invalid="ignore"):
        bg = F32(np.float64(s) / np.float64(den))
    return xc, yc, zc, bg


def shift_center(bands, nx, ny, nz, xc, yc, zc):
    """shift_center (radialft_interface.cpp:286-319): multiply the half
    spectrum (nz, ny, nx/2+1) by exp(i phi), phi = (2 pi zc/nz) kz +
    (2 pi yc/ny) ky + (2 pi xc/nx) kx in float, frequencies wrapped."""
    dphiz = F32(2 * math.pi * float(zc) / nz)
    dphiy = F32(2 * math.pi * float(yc) / ny)
    dphix = F32(2 * math.pi * float(xc) / nx)
    kz = np.arange(nz)
    kz = np.where(kz > nz // 2, kz - nz, kz).astype(F32)
    ky = np.arange(ny)
    ky = np.where(ky > ny // 2, ky - ny, ky).astype(F32)
    kx = np.arange(nx // 2 + 1).astype(F32)
    phi = ((dphiz * kz)[:, None, None] + (dphiy * ky)[None, :, None]).astype(F32)
    phi = (phi + (dphix * kx)[None, None, :]).astype(F32)
    e = np.cos(phi).astype(np.float64) + 1j * np.sin(phi).astype(np.float64)
    return bands * e


def radial_bins(nx, ny):
    """Radial bin of each (ky, kx) of the half spectrum (-1: not averaged), as
    radialft computes it (radialft_interface.cpp:343-349): rint of the float
    distance, kept when below nx/2+1."""
    ky = np.arange(ny)
    ky = np.where(ky > ny // 2, ky - ny, ky)
    kx = np.arange(nx // 2 + 1)
    r2 = ky[:, None] ** 2 + kx[None, :] ** 2
    rdist = np.sqrt(r2.astype(np.float64)).astype(F32)
    keep = rdist < (nx // 2 + 1)
    return np.where(keep, np.rint(rdist).astype(np.int64), -1)


def radialft(bands, nx, ny, nz):
    """radialft (radialft_interface.cpp:321-381): average the half spectrum
    over rings of equal rint(kr) for every kz, then make each kr row
    Hermitian in kz.  Returns the (nx/2+1, nz) complex table."""
    nxh = nx // 2 + 1
    bins = radial_bins(nx, ny)
    avg = np.zeros((nxh, nz), dtype=np.complex128)
    cnt = np.zeros(nxh, dtype=np.int64)
    for r in range(nxh):
        sel = bins == r
        c = int(sel.sum())
        cnt[r] = c
        if c:
            avg[r, :] = bands[:, sel].sum(axis=1) / c
    out = avg.copy()
    out[:, 0] = out[:, 0].real
    for kz in range(1, nz // 2 + 1):
        a = (out[:, kz] + np.conj(out[:, nz - kz])) / 2
        out[:, kz] = a
        out[:, nz - kz] = np.conj(a)
    return out


def cleanup(otf, nx, nz, dkr, dkz, lambdanm, krmax_user, NA, NIMM):
    """cleanup (radialft_interface.cpp:383-417): zero the table outside the
    OTF support of a widefield objective."""
    otf = otf.copy()
    lam = lambdanm * 0.001
    sinalpha = NA / NIMM
    cosalpha = math.cos(math.asin(sinalpha))
    krmax = 2 * NA / lam
    if krmax_user * dkr < krmax and krmax_user != 0:
        krmax = krmax_user * dkr
    for ix in range(nx // 2 + 1):
        kr = ix * dkr
        if kr <= krmax:
            beta = math.asin((NA - kr * lam) / NIMM)
            kzedge = (NIMM / lam) * (math.cos(beta) - cosalpha)
            kzstart = int(np.rint(kzedge / dkz + 1))
            kzend = nz - kzstart
            if kzstart <= kzend:
                otf[ix, max(kzstart, 0):kzend + 1] = 0
        else:
            otf[ix, :] = 0
    return otf


def fixorigin(otf, kx2):
    """fixorigin (radialft_interface.cpp:419-443): replace the kr = 0 row by
    the intercept of a straight-line fit over kr = 1..kx2 (double).  Returns
    (table, ok); ok is False when |kr=0| <= |kr=1| at kz = 0."""
    otf = otf.copy()
    nz = otf.shape[1]
    x = np.arange(1, kx2 + 1, dtype=np.float64)
    mean_kx = (kx2 + 1) / 2.0
    for z in range(nz):
        vals = otf[1:kx2 + 1, z].astype(np.complex128)
        mean_val = vals.sum() / kx2
        num = ((x - mean_kx) * (vals - mean_val)).sum()
        den = ((x - mean_kx) ** 2).sum()
        otf[0, z] = mean_val - (num / den) * mean_kx
        if z == 0 and abs(otf[0, 0]) <= abs(otf[1, 0]):
            return otf, False
    return otf, True


def rescale(otf):
    """rescale (radialft_interface.cpp:488-504): divide by the largest magnitude."""
    return otf / np.abs(otf).max()


def make_otf(psf, dr=0.102, dz=0.102, lambdanm=520, interpkr=10, user_background=None,
             NA=1.25, NIMM=1.3, krmax=0, do_cleanup=False):
    """makeOTF (radialft_interface.cpp:95-197), radial form: (nz, ny, nx)
    PSF -> (nx/2+1, nz) complex table (the file holds it as a float image of
    width 2 nz and height nx/2+1).  Raises on the reference's fixorigin
    failure (fewer than 4 points left)."""
    st = np.asarray(psf, dtype=F32)
    nz, ny, nx = st.shape
    dkr = 1 / (ny * dr)
    dkz = 1 / (nz * dz)
    xc, yc, zc, bg = determine_center_and_background(st)
    if user_background is not None:
        bg = F32(user_background)
    img = (st - bg).astype(F32)
    bands = np.fft.rfftn(img.astype(np.float64))
    bands = shift_center(bands, nx, ny, nz, xc, yc, zc)
    otf = radialft(bands, nx, ny, nz)
    if do_cleanup:
        otf = cleanup(otf, nx, nz, dkr, dkz, lambdanm, krmax, NA, NIMM)
    if interpkr > 0:
        while True:
            fixed, ok = fixorigin(otf, interpkr)
            if ok:
                otf = fixed
                break
            otf = fixed
            interpkr -= 1
            if interpkr < 4:
                raise RuntimeError("#pixels < 4 used in kr=0 extrapolation")
    return rescale(otf)


def make_otf_3d(psf, interpkr=10, user_background=None):
    """makeOTF with b3Dout (radialft_interface.cpp:150-154): the re-centred
    half spectrum (nz, ny, nx/2+1), its origin replaced by the fit over the
    +/-45 degree lines (fixorigin of radialft_interface.cpp:445-486) when
    interpkr > 1, divided by its largest magnitude."""
    st = np.asarray(psf, dtype=F32)
    nz, ny, nx = st.shape
    xc, yc, zc, bg = determine_center_and_background(st)
    if user_background is not None:
        bg = F32(user_background)
    bands = np.fft.rfftn((st - bg).astype(F32).astype(np.float64))
    bands = shift_center(bands, nx, ny, nz, xc, yc, zc)
    if interpkr > 1:
        nxh = nx // 2 + 1
        proj = np.zeros(nxh, dtype=np.complex128)
        for x in range(1, nxh):
            proj[x] = bands[:, x, x].sum() + bands[:, ny - x, x].sum()
        xs = np.arange(1, interpkr + 1, dtype=np.float64)
        mean_val = proj[1:interpkr + 1].sum() / interpkr
        mean_kx = (interpkr + 1) / 2.0
        slope = ((xs - mean_kx) * (proj[1:interpkr + 1] - mean_val)).sum() / ((xs - mean_kx) ** 2).sum()
        bands[0, 0, 0] = mean_val - slope * mean_kx
    return bands / np.abs(bands).max()
