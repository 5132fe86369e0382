"""GPU Wiener filter (cdx_wiener_device) against the oracle's restatement of
the reference's wienerfilter + otfinterpolate (linearDecon.cpp:78-168).
Float32 FFTs on the GPU, float64 in the oracle: relative L2 <= 1e-5."""

import numpy as np
import pytest

from conftest import rel_l2
from cudadecon_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape,kw", [((32, 64, 64), dict(wiener=0.01, NA=1.2, wavelength=0.525)),
                                      ((21, 50, 64), dict(wiener=0.05, NA=0.8, wavelength=0.6)),
                                      ((100, 256, 756), dict(wiener=0.01, NA=1.1, wavelength=0.51))])
def test_wiener_matches_oracle(cdx, oracle, torch_cuda, tmp_path, shape, kw):
    torch = torch_cuda
    tab = synth.gaussian_otf_table(65, 32, 1.3, 2.5)
    p = tmp_path / "otf.tif"
    synth.write_otf(p, tab)
    nz, ny, nx = shape
    cdx.rl_init(shape, p, dr=0.104, dz=0.3, dr_psf=0.104, dz_psf=0.2, deskew_angle=0.0,
                rotation_angle=0.0)
    assert cdx.decon_grid() == shape
    rng = np.random.default_rng(9)
    img = (100 + rng.gamma(2.0, 40.0, shape)).astype(np.float32)
    out = cdx.wiener(torch.from_numpy(img).cuda(), background=100.0, **kw).cpu().numpy()
    st = oracle.rl_init(nx, ny, nz, 0.104, 0.3, 0.104, 0.2, 0.0, 0.0, 0, False,
                        synth.otf_table_to_image(tab))
    ref = oracle.wiener(st, img, 100.0, kw["wiener"], kw["NA"], kw["wavelength"])
    assert rel_l2(out, ref) < 1e-5
    cdx.rl_cleanup()


def test_wiener_without_init_fails(cdx, torch_cuda):
    torch = torch_cuda
    cdx.rl_cleanup()
    with pytest.raises(cdx.CudaDeconError):
        cdx.wiener(torch.zeros((8, 8, 8), device="cuda"))
