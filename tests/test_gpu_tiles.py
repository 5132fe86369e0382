"""Y-tiled deconvolution (cdx_RL_tiled) and maximum-intensity projections
(cdx_mip_device), the CLI's tiling (linearDecon.cpp:497-566, 1175-1245) and
MaxIntProj (1434-1473).

Each tile is processed by the same pipeline as RL_interface, so the tiled
result must equal, bit for bit, the oracle's restatement of the CLI's tiling
and stitching applied to tiles deconvolved one RL_interface call at a time."""

import numpy as np
import pytest

from cudadecon_gb300 import synth

pytestmark = pytest.mark.gpu


def _init(cdx, tmp_path, shape, **kw):
    tab = synth.gaussian_otf_table(33, 16, 1.2, 2.0)
    p = tmp_path / "otf.tif"
    synth.write_otf(p, tab)
    a = dict(dr=0.104, dz=0.3, dr_psf=0.104, dz_psf=0.3, deskew_angle=0.0, rotation_angle=0.0)
    a.update(kw)
    cdx.rl_init(shape, p, **a)


@pytest.mark.parametrize("blend", [False, True])
@pytest.mark.parametrize("geom", ["plain", "deskew_rotate"])
def test_tiled_matches_per_tile_stitching(cdx, oracle, torch_cuda, tmp_path, blend, geom):
    raw = synth.bead_stack((20, 100, 64), n_beads=40, seed=31)
    tile, want_overlap = 48, 16
    kw = dict(deskew_angle=31.5, rotation_angle=31.5) if geom == "deskew_rotate" else {}
    tsize, n, overlap, offs = oracle.tiling(raw.shape[1], tile, want_overlap)
    assert (tsize, n, overlap, offs) == (48, 4, 30.0, [0, 18, 36, 54])  # last tile runs past y
    _init(cdx, tmp_path, (20, tile, 64), **kw)
    got = cdx.rl_tiled(raw, tile=tile, tile_overlap=want_overlap, blend=blend, n_iters=4)
    tiles = [cdx.rl_decon(oracle.tile_crop(raw, y0, tile), background=100.0, n_iters=4)
             for y0 in offs]
    want = oracle.stitch_tiles(tiles, offs, raw.shape[1], overlap, blend)
    cdx.rl_cleanup()
    assert got.shape == want.shape
    bad = np.argwhere(got != want)
    assert bad.size == 0, (len(bad), bad[:5], np.abs(got - want).max())


def test_untiled_equals_rl_interface(cdx, oracle, torch_cuda, tmp_path):
    raw = synth.bead_stack((16, 40, 48), n_beads=20, seed=32)
    _init(cdx, tmp_path, raw.shape)
    got = cdx.rl_tiled(raw, tile=0, n_iters=3)
    want = cdx.rl_decon(raw, background=100.0, n_iters=3)
    cdx.rl_cleanup()
    assert np.array_equal(got, want)


@pytest.mark.parametrize("axis", [0, 1, 2])
def test_mip_matches_max(cdx, torch_cuda, axis):
    torch = torch_cuda
    v = torch.randn((21, 33, 45), device="cuda")
    got = cdx.mip(v, axis)
    dim = {0: 2, 1: 1, 2: 0}[axis]
    want = torch.clamp_min(v.max(dim=dim).values, -1e10)
    assert torch.equal(got, want)


def test_tiled_repeat_calls_reuse_buffers(cdx, torch_cuda, tmp_path):
    """The tiling buffers stay in the session between calls: a second call
    (and one on a different stack) must not see the first call's stitch
    weights or output."""
    a = synth.bead_stack((12, 90, 40), n_beads=20, seed=51)
    b = synth.bead_stack((12, 90, 40), n_beads=25, seed=52)
    _init(cdx, tmp_path, (12, 40, 40))
    ra1 = cdx.rl_tiled(a, tile=40, tile_overlap=12, blend=True, n_iters=3)
    rb = cdx.rl_tiled(b, tile=40, tile_overlap=12, blend=True, n_iters=3)
    ra2 = cdx.rl_tiled(a, tile=40, tile_overlap=12, blend=True, n_iters=3)
    cdx.rl_cleanup()
    assert np.array_equal(ra1, ra2)
    assert not np.array_equal(ra1, rb)
