"""Oracle restatement of the CLI's Y tiling (linearDecon.cpp:497-519) and
stitching (1175-1245): known answers of the tiling arithmetic and the
properties the stitch rules must have."""

import numpy as np
import pytest

from oracle import rl_oracle as ro


@pytest.mark.parametrize("ny,tile,overlap,want", [
    (100, 48, 16, (48, 4, 30.0, [0, 18, 36, 54])),
    (300, -1, 30, (128, 4, 70.0, [0, 58, 116, 174])),   # -tile default: 128 rows
    (1024, 128, 30, (128, 11, 38.0, [90 * t for t in range(11)])),
    (60, 128, 30, (60, 2, 60.0, [0, 0])),                # tile clipped to the stack
    (77, 0, 30, (77, 1, 0.0, [0])),                      # no tiling
])
def test_tiling_known_answers(ny, tile, overlap, want):
    assert ro.tiling(ny, tile, overlap) == want


def test_tile_crop_repeats_last_row():
    raw = np.arange(2 * 10 * 3, dtype=np.uint16).reshape(2, 10, 3)
    t = ro.tile_crop(raw, 6, 8)
    assert t.shape == (2, 8, 3)
    assert np.array_equal(t[:, :4], raw[:, 6:10])
    assert np.array_equal(t[:, 4:], np.repeat(raw[:, 9:10], 4, axis=1))


@pytest.mark.parametrize("ny,tile,ov", [(100, 48, 16), (300, 128, 30), (257, 64, 20)])
def test_stitching_tiles_of_one_volume_gives_it_back(ny, tile, ov):
    rng = np.random.default_rng(ny)
    vol = rng.uniform(1, 2, size=(3, ny, 5)).astype(np.float32)
    tsize, n, overlap, offs = ro.tiling(ny, tile, ov)
    tiles = [ro.tile_crop(vol, y0, tsize) for y0 in offs]
    plain = ro.stitch_tiles(tiles, offs, ny, overlap, False)
    assert np.array_equal(plain, vol)           # every row written, each from a tile holding it
    blended = ro.stitch_tiles(tiles, offs, ny, overlap, True)
    np.testing.assert_allclose(blended, vol, rtol=1e-6)


def test_stitch_zones_of_constant_tiles():
    """Tile t holds the value t+1: the plain mode switches tiles at the middle
    of each overlap; the blend mode ramps over blend_zone rows after no_zone
    rows of each later tile."""
    ny, tsize, n, overlap, offs = 100, 48, 4, 30.0, [0, 18, 36, 54]
    tiles = [np.full((1, tsize, 1), t + 1, np.float32) for t in range(n)]
    plain = ro.stitch_tiles(tiles, offs, ny, overlap, False)[0, :, 0]
    # tile t >= 1 writes from its row 15 = floor(30/2) on; tile t < n-1 stops before row 33
    assert plain[17] == 1 and plain[18 + 15] == 2 and plain[36 + 15] == 3 and plain[54 + 15] == 4
    assert plain[32] == 1 and plain[50] == 2
    blended = ro.stitch_tiles(tiles, offs, ny, overlap, True)[0, :, 0]
    no_zone, blend_zone = 13, 4                  # ceil((30-4)/2), 30-2*13
    for k in range(1, blend_zone + 1):           # rows no_zone+k of tile 1 mix 2 over 1
        b = np.float32(k / blend_zone)
        assert blended[18 + no_zone + k] == np.float32(np.float32(2 * b) + 1.0 * (1.0 - float(b)))
    assert blended[18 + no_zone] == 1            # tile 1's no-zone leaves tile 0's rows
