"""The oracle against golden fixtures produced by the reference's own CUDA
kernels (tests/golden/make_golden.py: the reference sources compiled to PTX,
launched with cuFFT in the order of its host code, on a GB300).  These pin
the CPU restatement to the reference itself."""

from pathlib import Path

import numpy as np
import pytest

from conftest import rel_l2

G = Path(__file__).resolve().parent / "golden"


def _load(name):
    p = G / name
    if not p.exists():
        pytest.skip(f"{name} not generated")
    return np.load(p)


def test_deskew_oracle_bit_exact_to_reference(oracle):
    d = _load("golden_deskew.npz")
    for i in (0, 1):
        out = oracle.deskew(d["input"], float(d["factor"][i]), int(d["nxo"][i]), int(d["shift"][i]),
                            float(d["pad"][i]))
        np.testing.assert_array_equal(out.view(np.uint32), d[f"out{i}"].view(np.uint32))


def test_rotate_oracle_bit_exact_to_reference(oracle):
    d = _load("golden_rotate.npz")
    out = oracle.rotate(d["input"], d["rot"], int(d["nxr"]), int(d["nzr"]))
    np.testing.assert_array_equal(out.view(np.uint32), d["out"].view(np.uint32))


def test_rotate_sizes_match_reference_matrix(oracle):
    d = _load("golden_rotate.npz")
    nz, ny, nx = d["input"].shape
    assert oracle.rotated_dims(nx, nz, d["rot"]) == (int(d["nxr"]), int(d["nzr"]))


def test_camcor_oracle_to_reference(oracle):
    d = _load("golden_camcor.npz")
    out = oracle.camcor(d["raw"], d["camparam"])
    diff = np.abs(out.astype(np.int32) - d["out"].astype(np.int32))
    # the C library's expf may differ from CUDA's in the last bit
    assert diff.max() <= 1 and np.count_nonzero(diff) <= d["raw"].size // 1000
    assert np.any(d["out"] == 0)  # negative corrections saturate at 0


def test_affine_oracle_to_reference(oracle):
    d = _load("golden_affine.npz")
    assert np.max(np.abs(oracle.affine(d["input"], d["mat"]) - d["out"])) < 5e-3
    assert np.max(np.abs(oracle.affine(d["input"], d["mat"], ra=True, dx=0.1, dy=0.1, dz=0.3)
                         - d["out_ra"])) < 5e-3


def test_rl_oracle_to_reference(oracle):
    d = _load("golden_rl.npz")
    X0 = oracle.bgsub(d["raw"].astype(np.float32), float(d["background"]))
    st = oracle.rl_init(X0.shape[2], X0.shape[1], X0.shape[0], 0.1, 0.1, 0.1, 0.1, 0.0, 0.0, 0, False,
                        d["otf"].view(np.float32).reshape(d["otf"].shape[0], -1))
    assert np.allclose(oracle.kscales(st, X0.shape[2], X0.shape[1], X0.shape[0]), d["kscales"])
    H = oracle.otf_on_grid(st, X0.shape[2], X0.shape[1], X0.shape[0])
    lam = []
    out = oracle.rl_iterations(X0, X0, H, int(d["n_iters"]), lambdas=lam)
    assert rel_l2(out, d["out"]) < 1e-5
    np.testing.assert_allclose(lam, d["lambdas"][2:], atol=1e-5)
