"""GPU OTF generation (makeOTF / cdx_make_otf) against the oracle's
restatement of the reference's makeOTF (radialft_interface.cpp:95-197).

The transform is float32 on the GPU and float64 in the oracle, so the
tables agree to FFT rounding: relative L2 <= 1e-5 (tables are normalised to
a peak of 1)."""

import numpy as np
import pytest

from conftest import rel_l2
from oracle import otf_oracle as OO
from test_otf_cpu import gaussian_bead

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _psf(shape=(32, 64, 64), center=(14.3, 35.6, 29.2), seed=3):
    psf = gaussian_bead(shape, center, 1.6, 2.8)
    rng = np.random.default_rng(seed)
    return (psf + rng.normal(0, 0.5, psf.shape)).astype(np.float32)


@pytest.mark.parametrize("kw", [dict(), dict(interpkr=6), dict(background=95.0),
                                dict(cleanup=True, NA=1.1, lambdanm=510, dr=0.1, dz=0.2)])
def test_make_otf_matches_oracle(cdx, torch_cuda, kw):
    psf = _psf()
    got = cdx.make_otf(psf, **kw)
    ref = OO.make_otf(psf, dr=kw.get("dr", 0.102), dz=kw.get("dz", 0.102),
                      lambdanm=kw.get("lambdanm", 520), interpkr=kw.get("interpkr", 10),
                      user_background=kw.get("background"), NA=kw.get("NA", 1.25),
                      do_cleanup=kw.get("cleanup", False))
    g = got.view(np.complex64)
    assert g.shape == ref.shape
    assert rel_l2(g, ref) < TOL


def test_make_otf_3d_matches_oracle(cdx, torch_cuda):
    psf = _psf(shape=(16, 32, 48), center=(7.2, 15.5, 22.8))
    got = cdx.make_otf(psf, otf_3d=True).view(np.complex64)
    ref = OO.make_otf_3d(psf)
    assert got.shape == ref.shape
    assert rel_l2(got, ref) < TOL


def test_make_otf_file_feeds_rl_init(cdx, torch_cuda, tmp_path):
    """PSF file -> makeOTF -> OTF file -> RL_interface_init, as a pycudadecon
    user does (the OTF file layout is the one the reference reads)."""
    from cudadecon_gb300 import synth
    psf = _psf()
    pfile, ofile = tmp_path / "psf.tif", tmp_path / "otf.tif"
    cdx.save_image(pfile, psf)
    cdx.make_otf_file(pfile, ofile)
    img = cdx.load_image(ofile)
    assert img.shape == (1, 33, 64)
    ref = OO.make_otf(psf)
    assert rel_l2(img[0].view(np.complex64), ref) < TOL
    raw = synth.bead_stack((32, 64, 64), n_beads=20, seed=5)
    cdx.rl_init(raw.shape, ofile, dr=0.102, dz=0.102, dr_psf=0.102, dz_psf=0.102)
    out = cdx.rl_decon(raw, background=100.0, n_iters=3)
    assert np.isfinite(out).all() and out.shape == (32, 64, 64)
    cdx.rl_cleanup()


def test_make_otf_rejects_unsupported_sizes(cdx, torch_cuda):
    psf = _psf(shape=(11, 64, 64), center=(5.0, 32.0, 32.0))
    with pytest.raises(cdx.CudaDeconError):
        cdx.make_otf(psf)


@pytest.mark.parametrize("case", ["default", "interpkr6", "user_background", "cleanup", "wide",
                                  "out_3d"])
def test_make_otf_matches_reference_makeotf_fixtures(cdx, torch_cuda, case):
    """cdx_make_otf against the reference's own makeOTF output
    (tests/golden/golden_otf.npz, tests/golden/make_otf_golden.py)."""
    from pathlib import Path
    from golden.make_otf_golden import CASES, psf
    name, shape, center, sxy, sz, seed, kw = next(c for c in CASES if c[0] == case)
    want = np.load(Path(__file__).resolve().parent / "golden" / "golden_otf.npz")[name]
    p = psf(shape, center, sxy, sz, seed)
    args = {k: v for k, v in dict(dr=kw.get("dr"), dz=kw.get("dz"), lambdanm=kw.get("lambdanm"),
                                  interpkr=kw.get("interpkr"), background=kw.get("user_background"),
                                  NA=kw.get("NA"), cleanup=kw.get("do_cleanup")).items()
            if v is not None}
    if kw.get("out_3d"):
        args["otf_3d"] = True
    got = cdx.make_otf(p, **args).view(np.complex64)
    assert got.shape == want.shape
    assert rel_l2(got, want) < TOL
