"""Full-size checks where the oracle would take too long: size-independent
properties of the RL pipeline on the large time-lapse stack's grid
(256x1024x1024 u16 raw, deskewed to 256x1024x1620).

With a unit OTF the blur is the identity, so the RL ratio is raw / X and a
run started from the conditioned stack stays there: the result must equal the
deskewed, background-subtracted stack to float rounding, whatever the size."""

import numpy as np
import pytest

from conftest import rel_l2
from cudadecon_gb300 import synth

pytestmark = pytest.mark.gpu


def test_unit_otf_is_a_fixed_point_at_256x1024x1620(cdx, oracle, torch_cuda, tmp_path):
    torch = torch_cuda
    shape = (256, 1024, 1024)
    nz, ny, nx = shape
    # OTF = 1 at every (kr, kz).  The table is in physical frequency units and
    # zero beyond its last radial sample, so the PSF pixel is half the image
    # pixel: the table then reaches past the grid's corner frequencies
    # (sqrt(2) times the Nyquist radius) and the blur is the identity.
    tab = np.ones((65, 32), dtype=np.complex64)
    p = tmp_path / "otf.tif"
    synth.write_otf(p, tab)
    cdx.rl_init(shape, p, dr=0.104, dz=0.3, dr_psf=0.052, dz_psf=0.3, deskew_angle=31.5,
                rotation_angle=0.0)
    gz, gy, gx = cdx.decon_grid()
    assert (gz, gy, gx) == (256, 1024, 1620)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(1005)
    lam = 200.0 + 800.0 * torch.rand(shape, generator=gen, device="cuda")
    raw = torch.poisson(lam, generator=gen).to(torch.int32).to(torch.uint16)
    L = cdx.lib()
    import ctypes
    import math
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    # the conditioned stack, built independently: background subtraction, then
    # the (bit-exact) deskew with RL_interface_init's factor
    bg = (raw.float() - 100.0).clamp_min_(0.0)
    factor = math.cos(31.5 * math.pi / 180.0) * float(np.float32(0.3)) / float(np.float32(0.104))
    want = torch.empty((gz, gy, gx), dtype=torch.float32, device="cuda")
    assert L.cdx_deskew_device(ctypes.c_void_p(bg.data_ptr()), nx, ny, nz, factor,
                               ctypes.c_void_p(want.data_ptr()), gx, 0, 0.0, st) == 1
    del bg
    for n in (1, 3):
        o = torch.empty((gz, gy, gx), dtype=torch.float32, device="cuda")
        ok = L.cdx_RL_device(ctypes.c_void_p(raw.data_ptr()), nx, ny, nz, ctypes.c_void_p(o.data_ptr()),
                             None, 100.0, False, False, n, 0, 0, 0, 0.0, False, False, st)
        assert ok == 1, L.cdx_last_error()
        torch.cuda.synchronize()
        inside = want > 1.0
        assert inside.float().mean().item() > 0.5
        err = (o[inside] - want[inside]).abs().max().item() / want.abs().max().item()
        assert err < 1e-5, (n, err)
        assert torch.isfinite(o).all()
        del o
    cdx.rl_cleanup()
