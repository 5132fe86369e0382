"""Seeded synthetic light-sheet data for tests and benchmarks.

Nothing here is measured: these generators build the inputs (bead and
filament stacks, Gaussian PSFs, radially averaged OTF tables in the file
layout the reference reads, sCMOS camera parameters).  The OTF file layout
is the one radialft writes (scopetools/cudadecon src/radialft_interface.cpp:
160-193): a float32 image of width 2*nz_otf and height nr holding complex
values interleaved, kz fastest.
"""

from __future__ import annotations

import struct
from pathlib import Path

import numpy as np


# ---------------------------------------------------------------- OTF
def gaussian_otf_table(nr: int, nzotf: int, sigma_xy: float, sigma_z: float) -> np.ndarray:
    """Radially averaged OTF of a Gaussian PSF as a (nr, nzotf) complex64 table.

    sigma_xy / sigma_z are in PSF pixels; radial sample ir is at
    ir / (2 (nr - 1)) cycles per pixel (dkr_otf = 1/((nr-1) 2 dr_psf)) and kz
    sample iz at kz/nzotf cycles per z pixel with kz wrapped to
    [-nzotf/2, nzotf/2).  Normalised so that OTF(0, 0) = 1.
    """
    fr = np.arange(nr, dtype=np.float64) / (2.0 * (nr - 1))
    kz = np.arange(nzotf, dtype=np.float64)
    kz = np.where(kz > nzotf // 2, kz - nzotf, kz) / nzotf
    val = np.exp(-2.0 * np.pi ** 2 * (sigma_xy ** 2 * fr[:, None] ** 2 + sigma_z ** 2 * kz[None, :] ** 2))
    return val.astype(np.complex64)


def otf_table_to_image(table: np.ndarray) -> np.ndarray:
    """(nr, nzotf) complex -> (nr, 2*nzotf) float32 image (height nr, width 2 nzotf)."""
    t = np.ascontiguousarray(table, dtype=np.complex64)
    return t.view(np.float32).reshape(t.shape[0], 2 * t.shape[1])


def write_tiff(path, img: np.ndarray) -> None:
    """Minimal baseline TIFF (little endian, uncompressed, one strip per page).

    img is (h, w) or (d, h, w); float32, uint16 or uint8."""
    a = np.ascontiguousarray(img)
    if a.ndim == 2:
        a = a[None]
    if a.dtype == np.float32:
        bits, fmt = 32, 3
    elif a.dtype == np.uint16:
        bits, fmt = 16, 1
    elif a.dtype == np.uint8:
        bits, fmt = 8, 1
    else:
        a = a.astype(np.float32)
        bits, fmt = 32, 3
    a = a.astype(a.dtype.newbyteorder("<"), copy=False)
    d, h, w = a.shape
    out = bytearray(b"II*\x00")
    out += struct.pack("<I", 0)  # first IFD offset, patched below
    page_bytes = w * h * bits // 8
    ifd_pos_slot = 4
    for z in range(d):
        data_off = len(out)
        out += a[z].tobytes()
        if len(out) % 2:
            out += b"\x00"
        ifd_off = len(out)
        struct.pack_into("<I", out, ifd_pos_slot, ifd_off)
        tags = [
            (256, 4, 1, w), (257, 4, 1, h), (258, 3, 1, bits), (259, 3, 1, 1), (262, 3, 1, 1),
            (273, 4, 1, data_off), (277, 3, 1, 1), (278, 4, 1, h), (279, 4, 1, page_bytes),
            (284, 3, 1, 1), (339, 3, 1, fmt),
        ]
        out += struct.pack("<H", len(tags))
        for tag, typ, cnt, val in tags:
            if typ == 3:
                out += struct.pack("<HHIHH", tag, typ, cnt, val, 0)
            else:
                out += struct.pack("<HHII", tag, typ, cnt, val)
        ifd_pos_slot = len(out)
        out += struct.pack("<I", 0)
    Path(path).write_bytes(bytes(out))


def write_cimg(path, img: np.ndarray) -> None:
    """CImg .cimg file (uncompressed float, little endian) of a (h, w) or (d, h, w) array."""
    a = np.ascontiguousarray(img, dtype="<f4")
    if a.ndim == 2:
        a = a[None]
    d, h, w = a.shape
    hdr = f"1 float little_endian\n{w} {h} {d} 1\n".encode()
    Path(path).write_bytes(hdr + a.tobytes())


def write_otf(path, table: np.ndarray) -> None:
    """Write a radial OTF table in the reference layout; format from the suffix."""
    img = otf_table_to_image(table)
    if str(path).lower().endswith(".cimg"):
        write_cimg(path, img)
    else:
        write_tiff(path, img)


# ---------------------------------------------------------------- stacks
def _gauss_otf_grid(shape, sigma_z, sigma_y, sigma_x):
    nz, ny, nx = shape
    fz = np.fft.fftfreq(nz)[:, None, None]
    fy = np.fft.fftfreq(ny)[None, :, None]
    fx = np.fft.rfftfreq(nx)[None, None, :]
    return np.exp(-2 * np.pi ** 2 * ((sigma_z * fz) ** 2 + (sigma_y * fy) ** 2 + (sigma_x * fx) ** 2))


def _splat_points(shape, pts, amps):
    """Deposit point intensities with trilinear weights."""
    vol = np.zeros(shape, dtype=np.float64)
    nz, ny, nx = shape
    p0 = np.floor(pts).astype(np.int64)
    f = pts - p0
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                w = (f[:, 0] if dz else 1 - f[:, 0]) * (f[:, 1] if dy else 1 - f[:, 1]) * \
                    (f[:, 2] if dx else 1 - f[:, 2])
                iz, iy, ix = p0[:, 0] + dz, p0[:, 1] + dy, p0[:, 2] + dx
                ok = (iz >= 0) & (iz < nz) & (iy >= 0) & (iy < ny) & (ix >= 0) & (ix < nx)
                np.add.at(vol, (iz[ok], iy[ok], ix[ok]), (amps * w)[ok])
    return vol


def bead_stack(shape, n_beads=200, sigma_range=(0.5, 2.0), amp_range=(500.0, 5000.0),
               psf_sigma_xy=1.5, psf_sigma_z=4.0, background=100.0, n_filaments=0,
               filament_intensity=(200.0, 3000.0), seed=1001, poisson=True) -> np.ndarray:
    """(nz, ny, nx) uint16 stack: Gaussian beads (and optional random 3D
    polylines) blurred by a Gaussian PSF, plus background and Poisson noise."""
    rng = np.random.default_rng(seed)
    shape = tuple(int(s) for s in shape)
    nz, ny, nx = shape
    obj = np.zeros(shape, dtype=np.float64)
    # beads: each bead's own Gaussian width is combined with the PSF below by
    # grouping beads into a few width bins (blur per bin)
    sig = rng.uniform(*sigma_range, size=n_beads)
    amp = rng.uniform(*amp_range, size=n_beads)
    pos = rng.uniform([0, 0, 0], [nz - 1, ny - 1, nx - 1], size=(n_beads, 3))
    bins = np.linspace(sigma_range[0], sigma_range[1], 5)
    idx = np.clip(np.digitize(sig, bins) - 1, 0, 3)
    spec = np.zeros((nz, ny, nx // 2 + 1), dtype=np.complex128)
    for b in range(4):
        m = idx == b
        if not m.any():
            continue
        s = 0.5 * (bins[b] + bins[b + 1])
        # peak amplitude A of a Gaussian bead of width s carries A (2 pi)^1.5 s^3
        pts = _splat_points(shape, pos[m], amp[m] * (2 * np.pi) ** 1.5 * s ** 3)
        spec += np.fft.rfftn(pts) * _gauss_otf_grid(shape, s, s, s)
    if n_filaments:
        for _ in range(n_filaments):
            nseg = rng.integers(2, 6)
            verts = rng.uniform([0, 0, 0], [nz - 1, ny - 1, nx - 1], size=(nseg + 1, 3))
            inten = rng.uniform(*filament_intensity)
            pts = []
            for a, b in zip(verts[:-1], verts[1:]):
                n = int(np.ceil(np.linalg.norm(b - a) * 2)) + 1
                t = np.linspace(0, 1, n)[:, None]
                pts.append(a + t * (b - a))
            pts = np.concatenate(pts)
            spec += np.fft.rfftn(_splat_points(shape, pts, np.full(len(pts), inten * 0.5)))
    spec *= _gauss_otf_grid(shape, psf_sigma_z, psf_sigma_xy, psf_sigma_xy)
    img = np.fft.irfftn(spec, s=shape, axes=(0, 1, 2))
    img = np.maximum(img, 0) + background
    if poisson:
        img = rng.poisson(img).astype(np.float64)
    return np.clip(np.rint(img), 0, 65535).astype(np.uint16)


def bead_stack_gpu(shape, n_beads=2000, amp_range=(500.0, 5000.0), psf_sigma_xy=1.5,
                   psf_sigma_z=4.0, background=100.0, seed=1001, device="cuda"):
    """Large stacks generated on the GPU (seeded torch generator): point
    beads of uniform amplitude, blurred by the Gaussian PSF (FFT on the
    device), plus background and Poisson noise.  Returns a (nz, ny, nx)
    uint16 tensor on `device`."""
    import torch
    gen = torch.Generator(device=device)
    gen.manual_seed(int(seed))
    nz, ny, nx = (int(v) for v in shape)
    obj = torch.zeros((nz, ny, nx), dtype=torch.float32, device=device)
    idx = torch.randint(0, nz * ny * nx, (n_beads,), generator=gen, device=device)
    amp = amp_range[0] + (amp_range[1] - amp_range[0]) * torch.rand(
        n_beads, generator=gen, device=device)
    obj.view(-1).index_add_(0, idx, amp * (2 * np.pi) ** 1.5 * psf_sigma_xy ** 2 * psf_sigma_z)
    fz = torch.fft.fftfreq(nz, device=device)[:, None, None]
    fy = torch.fft.fftfreq(ny, device=device)[None, :, None]
    fx = torch.fft.rfftfreq(nx, device=device)[None, None, :]
    otf = torch.exp(-2 * np.pi ** 2 * ((psf_sigma_z * fz) ** 2 + (psf_sigma_xy * fy) ** 2 +
                                       (psf_sigma_xy * fx) ** 2))
    img = torch.fft.irfftn(torch.fft.rfftn(obj) * otf, s=(nz, ny, nx))
    del obj, otf
    img = img.clamp_(min=0.0).add_(background)
    img = torch.poisson(img, generator=gen)
    return img.clamp_(0, 65535).to(torch.int32).to(torch.uint16)


def camcor_params(ny, nx, seed=1005, offset=(90.0, 110.0), coeff=(0.0, 0.02)) -> np.ndarray:
    """(3, ny, nx) float32 sCMOS parameters: planes a, b, offset."""
    rng = np.random.default_rng(seed)
    a = rng.uniform(*coeff, size=(ny, nx))
    b = rng.uniform(*coeff, size=(ny, nx))
    off = rng.uniform(*offset, size=(ny, nx))
    return np.stack([a, b, off]).astype(np.float32)


def smooth_sizes(lo, hi):
    """All 2,3,5,7-smooth integers in [lo, hi]."""
    out = []
    for n in range(max(lo, 2), hi + 1):
        m = n
        for p in (2, 3, 5, 7):
            while m % p == 0:
                m //= p
        if m == 1:
            out.append(n)
    return out
