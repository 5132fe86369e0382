"""CPU checks of the oracle: known answers derived from the reference's code
(src/RL-Biggs-Andrews.cpp, src/RLgpuImpl.cu, src/geometryTransform.cu,
src/camcor.cu) and self-consistency between its float32 and float64 forms."""

import math

import numpy as np
import pytest

from conftest import rel_l2
from cudadecon_gb300 import synth


def _state(O, shape_zyx, otf_table, **kw):
    nz, ny, nx = shape_zyx
    args = dict(dr=0.1, dz=0.1, dr_psf=0.1, dz_psf=0.1, deskewAngle=0.0, rotationAngle=0.0,
                outputWidth=0, bSkewedDecon=False)
    args.update(kw)
    return O.rl_init(nx, ny, nz, args["dr"], args["dz"], args["dr_psf"], args["dz_psf"],
                     args["deskewAngle"], args["rotationAngle"], args["outputWidth"],
                     args["bSkewedDecon"], synth.otf_table_to_image(otf_table))


def test_find_optimal_dimension_known_values(oracle):
    # RL-Biggs-Andrews.cpp:18-43: round down to a 2,3,5,7-smooth size
    f = oracle.find_optimal_dimension
    assert f(101) == 100
    assert f(757) == 756
    assert f(1653) == 1620
    assert f(256) == 256
    assert f(613) == 600
    assert f(186) == 180
    assert f(11) == 10
    assert f(13) == 12
    assert f(1) == 0  # no smooth size >= 2 (the reference recurses forever)
    assert f(97, step=+1) == 98
    for n in range(2, 2000):
        m = f(n)
        assert m <= n and not oracle.not_good_dimension(m)
        assert all(oracle.not_good_dimension(k) for k in range(m + 1, n + 1))


def test_stage_scan_geometry_known_answers(oracle):
    # 101x256x512 raw at 31.5 deg, dz 0.3, dxy 0.104 -> decon 100x256x756, rotated 150x256x723
    tab = synth.gaussian_otf_table(129, 64, 1.3, 3.0)
    st = _state(oracle, (101, 256, 512), tab, dr=0.104, dz=0.3, dr_psf=0.104, dz_psf=0.2,
                deskewAngle=31.5, rotationAngle=31.5)
    assert (st.output_nz, st.output_ny, st.output_nx) == (100, 256, 512)
    assert st.deskewedXdim == 756
    assert abs(st.deskewFactor - math.cos(math.radians(31.5)) * 0.3 / 0.104) < 1e-6
    assert abs(float(st.dz) - 0.3 * math.sin(math.radians(31.5))) < 1e-6
    assert oracle.rotated_dims(756, 100, st.rot) == (723, 150)
    np.testing.assert_allclose(st.rot, [0.5657, 0.3467, -0.5225, 0.8526], atol=1e-4)


def test_negative_rotation_reported_width_quirk(oracle):
    # get_output_nx uses p[1] without fabs (RL-Biggs-Andrews.cpp:479 vs 411):
    # for a negative rotation angle it reports less than the rotated width
    tab = synth.gaussian_otf_table(129, 64, 1.3, 3.0)
    st = _state(oracle, (101, 256, 512), tab, dr=0.104, dz=0.4, dr_psf=0.104, dz_psf=0.1,
                deskewAngle=-32.8, rotationAngle=-32.8)
    nxr, nzr = oracle.rotated_dims(st.deskewedXdim, st.output_nz, st.rot)
    rnx, rnz = oracle.reported_dims(st)
    assert rnz == nzr and rnx < nxr


def test_rl_float32_close_to_float64(oracle):
    raw = synth.bead_stack((32, 64, 64), n_beads=20, seed=7)
    st = _state(oracle, raw.shape, synth.gaussian_otf_table(33, 32, 1.5, 4.0))
    r32, _ = oracle.rl_interface(st, raw, nIters=10, dtype=np.float32)
    r64, _ = oracle.rl_interface(st, raw, nIters=10, dtype=np.float64)
    assert rel_l2(r32, r64) < 1e-5


def test_rl_constant_image_fixed_point(oracle):
    # conv of a constant by a normalised OTF is the constant: ratio = 1 + eps
    # in the first iteration, then X stays at (raw - bg)(1 + eps)
    st = _state(oracle, (16, 32, 32), synth.gaussian_otf_table(17, 16, 1.0, 2.0))
    raw = np.full((16, 32, 32), 600, np.uint16)
    r, _ = oracle.rl_interface(st, raw, background=100, nIters=6, dtype=np.float64)
    np.testing.assert_allclose(r, 500.0 * (1 + oracle.FLT_EPS), rtol=1e-12)


def test_rl_unit_otf_returns_raw(oracle):
    # OTF == 1 everywhere: conv is the identity and one iteration gives
    # X = (raw/X0 + eps) X0 = raw + eps X0
    tab = np.ones((17, 16), np.complex64)
    st = _state(oracle, (16, 32, 32), tab)
    raw = synth.bead_stack((16, 32, 32), n_beads=5, seed=9)
    r, _ = oracle.rl_interface(st, raw, background=0, nIters=1, dtype=np.float64)
    x0 = raw.astype(np.float64)
    # the radial table only covers kr < nr-1: corners of the xy spectrum are cut
    assert rel_l2(r, x0 * (1 + oracle.FLT_EPS)) < 0.05


def test_otf_interpolation_radial_known_values(oracle):
    # unit k-scales: the OTF at integer (kr, kz) equals the table entry
    tab = synth.gaussian_otf_table(33, 16, 1.2, 2.0)
    st = _state(oracle, (16, 64, 64), tab)
    H = oracle.otf_on_grid(st, 64, 64, 16, dtype=np.float64)
    assert H.shape == (16, 64, 33)
    for kx in (0, 3, 10):
        for kz in (0, 2, 15):
            np.testing.assert_allclose(H[kz, 0, kx], tab[kx, kz], rtol=1e-6)
    # outside kr >= nr - 1 the OTF is zero
    assert H[0, 0, 32] == 0 and H[0, 32, 32] == 0


def test_deskew_oracle_zero_factor_is_shift(oracle):
    a = np.random.default_rng(0).random((4, 3, 20)).astype(np.float32)
    # deskewFactor 0, nxOut == nx: xin = xout exactly; the last column is padVal
    out = oracle.deskew(a, 0.0, 20, 0, pad_val=-1.0)
    np.testing.assert_array_equal(out[..., :19], a[..., :19])
    assert np.all(out[..., 19] == -1.0)


def test_rotate_oracle_zero_angle_flips_z(oracle):
    a = np.random.default_rng(1).random((6, 3, 10)).astype(np.float32)
    rot = np.array([1, 0, 0, 1], np.float32)
    out = oracle.rotate(a, rot, 10, 6)
    # zin = zout - 3 + 3 (centred), output z flipped; last row/col is outside
    np.testing.assert_array_equal(out[::-1][:5, :, :9], a[:5, :, :9])


def test_camcor_oracle_previous_slice_wraps(oracle):
    rng = np.random.default_rng(2)
    raw = rng.integers(100, 2000, size=(3, 4, 5)).astype(np.uint16)
    p = np.zeros((3, 4, 5), np.float32)
    p[0] = 10.0   # a
    p[1] = 0.001  # b
    p[2] = 100.0  # offset
    out = oracle.camcor(raw, p)
    for z in range(3):
        prev = raw[z - 1 if z else 2].astype(np.float64)
        ref = raw[z] - 100.0 - 0.9 * 10.0 * (1 - np.exp(-0.001 * (prev - 100.0)))
        assert np.max(np.abs(out[z].astype(np.float64) - np.floor(np.maximum(ref, 0)))) <= 1


def test_camcor_oracle_negative_saturates_to_zero(oracle):
    raw = np.full((2, 2, 2), 50, np.uint16)
    p = np.zeros((3, 2, 2), np.float32)
    p[2] = 100.0
    assert np.all(oracle.camcor(raw, p) == 0)


def test_zblend_oracle_reference_slice_bug(oracle):
    img = np.zeros((6, 2, 2), np.float32)
    img[-1] = 10.0
    out = oracle.zblend(img.copy(), 3)
    w = 1.0 - math.sin((1.5 / 3.0) * math.pi * 0.5)
    # only slices 1 and nz-2 change, three times each
    assert np.all(out[[0, 2, 3]] == 0)
    np.testing.assert_allclose(out[1], 3 * np.float32(10.0 * w), rtol=1e-6)


def test_torch_fp64_oracle_matches_numpy_fp64(oracle):
    """The torch restatement of the FP64 oracle (used on the GPU for the
    full-size grids) against the numpy one, on the CPU: OTF grid, estimates
    and acceleration factors agree to float64 rounding."""
    torch = pytest.importorskip("torch")
    from oracle import rl_oracle_torch as OT
    shape = (12, 20, 30)
    tab = synth.gaussian_otf_table(17, 10, 1.3, 2.0)
    st = _state(oracle, shape, tab, dr=0.104, dz=0.3, dr_psf=0.09, dz_psf=0.2)
    H = oracle.otf_on_grid(st, 30, 20, 12, dtype=np.float64)
    Ht = OT.otf_on_grid(st, 30, 20, 12, device="cpu")
    assert rel_l2(Ht.numpy(), H) < 1e-14
    rng = np.random.default_rng(9)
    raw = (rng.gamma(2.0, 50.0, shape) + 1.0).astype(np.float32)
    la, lb = [], []
    a = oracle.rl_iterations(raw, raw, H, 8, dtype=np.float64, lambdas=la)
    b = OT.rl_iterations(raw, raw, Ht, 8, lambdas=lb, device="cpu").numpy()
    assert rel_l2(b, a) < 1e-12
    assert np.allclose(la, lb, rtol=0, atol=1e-12)


def test_convergence_norms_are_relative_changes_of_the_estimate():
    """rl_iterations(norms=...) records ||X_{k+1} - X_k|| / ||X_k|| per
    iteration: the first equals the change from X0 computed directly, and
    the list has one entry per iteration."""
    import numpy as np
    from oracle import rl_oracle as O
    rng = np.random.default_rng(5)
    shape = (8, 12, 16)
    X0 = rng.uniform(1.0, 5.0, shape).astype(np.float32)
    H = np.exp(-rng.uniform(0, 1, (8, 12, 9))).astype(np.complex64)
    norms = []
    X1 = O.rl_iterations(X0, X0, H, 1, norms=norms)
    assert len(norms) == 1
    want = np.linalg.norm(X1.astype(np.float64) - X0) / np.linalg.norm(X0.astype(np.float64))
    assert abs(norms[0] - want) < 1e-12
    norms = []
    O.rl_iterations(X0, X0, H, 5, norms=norms)
    assert len(norms) == 5 and all(n >= 0 for n in norms)
