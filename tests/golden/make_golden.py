"""Generate the golden fixtures of tests/golden/ from the reference's own CUDA
kernels (compiled from its sources, launched by oracle/ref_runner.cu with
cuFFT in the order of the reference's host code).  Needs a GPU and
oracle/_ref/ built; run on the GPU machine:

    python tests/golden/make_golden.py --out <dir>

and copy the .npz files into tests/golden/.  Inputs are seeded and stored in
the fixtures with the outputs.
"""

from __future__ import annotations

import argparse
import math
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from cudadecon_gb300 import synth  # noqa: E402
from oracle import ref_kernels as RK  # noqa: E402
from oracle import rl_oracle as O  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=str(Path(__file__).resolve().parent))
    args = ap.parse_args()
    out = Path(args.out)
    out.mkdir(parents=True, exist_ok=True)
    ok, why = RK.available()
    if not ok:
        raise SystemExit(why)
    rng = np.random.default_rng(20261203)

    # deskew (geometryTransform.cu:4-48): stage-scan factor, and a negative one
    a = (rng.random((12, 6, 80)) * 1000).astype(np.float32)
    f1 = math.cos(float(np.float32(31.5)) * math.pi / 180.) * float(np.float32(0.3)) / float(np.float32(0.104))
    np.savez_compressed(out / "golden_deskew.npz", input=a,
                        factor=np.array([f1, -1.3]), nxo=np.array([120, 96]),
                        shift=np.array([0, 2]), pad=np.array([0.0, 7.5], np.float32),
                        out0=RK.deskew(a, f1, 120, 0, 0.0), out1=RK.deskew(a, -1.3, 96, 2, 7.5))

    # rotate (geometryTransform.cu:50-106) with the stage-scan rotation matrix
    st = O.rl_init(512, 256, 101, 0.104, 0.3, 0.104, 0.2, 31.5, 31.5, 0, False,
                   synth.otf_table_to_image(synth.gaussian_otf_table(129, 64, 1.3, 3.0)))
    b = (rng.random((30, 5, 90)) * 1000).astype(np.float32)
    nxr, nzr = O.rotated_dims(90, 30, st.rot)
    np.savez_compressed(out / "golden_rotate.npz", input=b, rot=st.rot, nxr=nxr, nzr=nzr,
                        out=RK.rotate(b, st.rot, nxr, nzr))

    # camcor (camcor.cu:80-108), including voxels below the offset
    raw = rng.integers(60, 4000, size=(5, 24, 32)).astype(np.uint16)
    p = synth.camcor_params(24, 32, seed=77)
    p[0] *= 500.0
    np.savez_compressed(out / "golden_camcor.npz", raw=raw, camparam=p, out=RK.camcor(raw, p))

    # affine (geometryTransform.cu:183-349), texture filtering
    c = rng.random((10, 14, 18)).astype(np.float32)
    M = np.eye(4, dtype=np.float32)
    M[:3, :3] = [[0.95, 0.08, 0.0], [-0.07, 0.97, 0.03], [0.0, 0.02, 1.01]]
    M[:3, 3] = [1.3, -0.7, 0.4]
    np.savez_compressed(out / "golden_affine.npz", input=c, mat=M, out=RK.affine(c, M),
                        out_ra=RK.affine(c, M, ra=True, dx=0.1, dy=0.1, dz=0.3))

    # RL loop (RL-Biggs-Andrews.cpp:282-367): small stack, radially averaged OTF
    shape = (12, 40, 36)
    raw = synth.bead_stack(shape, n_beads=25, psf_sigma_xy=1.2, psf_sigma_z=2.0, seed=31)
    tab = synth.gaussian_otf_table(19, 12, 1.2, 2.0)
    # a complex OTF that is still Hermitian in kz (the OTF of a real,
    # asymmetric PSF): odd phase, zero at kz = 0 and at the Nyquist bin.  A
    # non-Hermitian spectrum would make the inverse real FFT's result
    # depend on the FFT implementation.
    kz = np.arange(12)
    tab = (tab * np.exp(0.2j * np.sin(2 * np.pi * kz / 12))[None, :]).astype(np.complex64)
    st = O.rl_init(36, 40, 12, 0.1, 0.1, 0.1, 0.1, 0.0, 0.0, 0, False, synth.otf_table_to_image(tab))
    X0 = O.bgsub(raw.astype(np.float32), 100.0)
    ks = O.kscales(st, 36, 40, 12)
    Xr, lam = RK.rl_iterations(X0, X0, tab, ks, 8)
    np.savez_compressed(out / "golden_rl.npz", raw=raw, background=np.float32(100.0), otf=tab,
                        kscales=np.array(ks, np.float32), n_iters=8, out=Xr, lambdas=lam)
    print("wrote", sorted(p.name for p in out.glob("golden_*.npz")))


if __name__ == "__main__":
    main()
