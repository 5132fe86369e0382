"""Generate tests/golden/golden_otf.npz: the reference's own makeOTF
(src/radialft_interface.cpp:95-197, compiled here from its source by
oracle/build.py with stand-ins for FFTW and libtiff, oracle/radialft_ref.py)
on seeded synthetic PSFs, with the argument sets the tests use.

Run where the reference checkout is present:

    python -c "from oracle import build; build.build_all()"
    python tests/golden/make_otf_golden.py
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

OUT = Path(__file__).resolve().parent / "golden_otf.npz"

# (name, PSF shape, bead centre, sigma xy, sigma z, noise seed, makeOTF arguments)
CASES = [
    ("default", (32, 64, 64), (14.3, 35.6, 29.2), 1.6, 2.8, 3, {}),
    ("interpkr6", (32, 64, 64), (14.3, 35.6, 29.2), 1.6, 2.8, 3, {"interpkr": 6}),
    ("user_background", (32, 64, 64), (14.3, 35.6, 29.2), 1.6, 2.8, 3, {"user_background": 95.0}),
    ("cleanup", (32, 64, 64), (14.3, 35.6, 29.2), 1.6, 2.8, 3,
     {"do_cleanup": True, "NA": 1.1, "lambdanm": 510, "dr": 0.1, "dz": 0.2}),
    ("wide", (48, 96, 80), (22.7, 47.2, 41.9), 2.1, 3.6, 7, {"dr": 0.104, "dz": 0.2}),
    ("out_3d", (16, 32, 48), (7.2, 15.5, 22.8), 1.6, 2.8, 3, {"out_3d": True}),
]


def psf(shape, center, sxy, sz, seed):
    """Seeded Gaussian bead on a background of 100 with Gaussian noise."""
    nz, ny, nx = shape
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    cz, cy, cx = center
    g = 1000.0 * np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2 * sxy ** 2) -
                        (z - cz) ** 2 / (2 * sz ** 2)) + 100.0
    return (g + np.random.default_rng(seed).normal(0, 0.5, g.shape)).astype(np.float32)


def main() -> None:
    from oracle import radialft_ref as R
    if not R.available():
        raise SystemExit("oracle/_ref/libradialft_ref.so is not built (needs the reference)")
    out = {}
    for name, shape, center, sxy, sz, seed, kw in CASES:
        out[name] = R.make_otf(psf(shape, center, sxy, sz, seed), **kw)
    np.savez_compressed(OUT, **out)
    print(OUT, {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
