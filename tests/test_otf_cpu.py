"""CPU checks of OTF generation: the oracle's restatement of makeOTF against
known answers (a Gaussian bead's OTF is a Gaussian), the parabola fit, and
the library's TIFF writer read back by its TIFF reader (no GPU needed)."""

import math

from pathlib import Path

import numpy as np
import pytest

from oracle import otf_oracle as OO

ROOT_GOLDEN = Path(__file__).resolve().parent / "golden"


def gaussian_bead(shape, center, sxy, sz, amp=1000.0, bg=100.0):
    nz, ny, nx = shape
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    cz, cy, cx = center
    g = amp * np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2 * sxy ** 2) - (z - cz) ** 2 / (2 * sz ** 2))
    return (g + bg).astype(np.float32)


def test_fitparabola_known_answers():
    assert OO.fitparabola(1.0, 2.0, 1.0) == 0.0          # symmetric peak
    assert abs(OO.fitparabola(0.0, 1.0, 0.5) - 0.1666667) < 1e-6
    assert OO.fitparabola(1.0, 1.0, 1.0) == 0.0          # flat: no peak
    assert OO.fitparabola(0.0, 0.0, 10.0) == -0.5
    assert OO.fitparabola(0.0, 1.0, 1.9) == 0.0          # vertex at 9.5: beyond 1.5


def test_center_and_background_of_a_bead():
    psf = gaussian_bead((32, 64, 64), (15.0, 33.0, 30.0), 1.5, 2.5)
    xc, yc, zc, bg = OO.determine_center_and_background(psf)
    assert abs(xc - 30.0) < 0.05 and abs(yc - 33.0) < 0.05
    assert abs(zc - 15.6) < 0.05                         # the reference adds 0.6 in z
    assert abs(bg - 100.0) < 0.5


def test_radial_otf_of_a_gaussian_bead_is_gaussian():
    shape = (32, 64, 64)
    sxy, sz = 1.5, 2.5
    psf = gaussian_bead(shape, (16.0, 32.0, 32.0), sxy, sz)
    otf = OO.make_otf(psf, interpkr=0, user_background=100.0)
    nz, ny, nx = shape
    kr = np.arange(nx // 2 + 1)[:, None] / nx
    kz = np.arange(nz)
    kz = np.where(kz > nz // 2, kz - nz, kz)[None, :] / nz
    want = np.exp(-2 * math.pi ** 2 * (sxy ** 2 * kr ** 2 + sz ** 2 * kz ** 2))
    assert abs(otf[0, 0] - 1) < 1e-12
    # ring averages of a Gaussian over integer-rounded radii, and the +0.6
    # z offset of the centre estimate turns into a kz phase ramp: compare
    # magnitudes at low frequencies
    low = (kr[:, 0] < 0.15)[:, None] & (np.abs(kz) < 0.15)
    assert np.max(np.abs(np.abs(otf) - want)[low]) < 0.03
    assert np.allclose(otf[:, 1:], np.conj(otf[:, :0:-1]))  # Hermitian in kz


def test_fixorigin_restores_a_linear_profile():
    nz = 8
    t = np.tile((1.0 - 0.05 * np.arange(12))[:, None], (1, nz)).astype(np.complex128)
    t[0, :] = 0
    fixed, ok = OO.fixorigin(t, 10)
    assert ok and np.allclose(fixed[0], 1.0)


def test_float_tiff_writer_roundtrip(cdx, tmp_path):
    rng = np.random.default_rng(7)
    for shape in [(3, 5), (2, 4, 6)]:
        a = rng.standard_normal(shape).astype(np.float32)
        p = tmp_path / f"img{len(shape)}.tif"
        cdx.save_image(p, a)
        b = cdx.load_image(p)
        assert np.array_equal(b.reshape(a.shape), a)


def test_make_otf_missing_file_returns_one(cdx, tmp_path):
    assert cdx.lib().makeOTF(str(tmp_path / "nope.tif").encode(), str(tmp_path / "o.tif").encode(),
                             520, 0.1, 10, False, 90.0, 1.25, 1.3, 0.1, 0, False, False) == 1


def _golden_otf_cases():
    from golden.make_otf_golden import CASES
    return CASES


@pytest.mark.parametrize("case", [c[0] for c in _golden_otf_cases()])
def test_otf_oracle_matches_reference_makeotf_fixtures(case):
    """The oracle's restatement of makeOTF against the reference's own
    makeOTF (its source compiled with stand-ins for FFTW and libtiff;
    tests/golden/make_otf_golden.py)."""
    from conftest import rel_l2
    from golden.make_otf_golden import CASES, psf
    name, shape, center, sxy, sz, seed, kw = next(c for c in CASES if c[0] == case)
    want = np.load(ROOT_GOLDEN / "golden_otf.npz")[name]
    p = psf(shape, center, sxy, sz, seed)
    if kw.get("out_3d"):
        got = OO.make_otf_3d(p)
    else:
        got = OO.make_otf(p, dr=kw.get("dr", 0.102), dz=kw.get("dz", 0.102),
                          lambdanm=kw.get("lambdanm", 520), interpkr=kw.get("interpkr", 10),
                          user_background=kw.get("user_background"), NA=kw.get("NA", 1.25),
                          do_cleanup=kw.get("do_cleanup", False))
    assert got.shape == want.shape
    assert rel_l2(got, want) < 1e-6
