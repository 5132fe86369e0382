"""GPU parity of the sm_103a library against the oracle (CPU restatement of
the reference), through the C ABI.

Tolerances: FFTs and the RL loop are float32, compared by relative L2 error:
<= 1e-5 against the float32 oracle (the reference's own precision target for
the plain form), and the float64 oracle's error is reported.  The deskew and
rotate kernels must match bit for bit; camcor to one count (expf may differ
in the last bit between CUDA and the C library)."""

import ctypes

import numpy as np
import pytest

from conftest import rel_l2
from cudadecon_gb300 import synth

pytestmark = pytest.mark.gpu

RL_TOL = 1e-5


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _stream(torch):
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _init(cdx, tmp_path, shape_zyx, table, **kw):
    p = tmp_path / "otf.tif"
    synth.write_otf(p, table)
    args = dict(dr=0.1, dz=0.1, dr_psf=0.1, dz_psf=0.1, deskew_angle=0.0, rotation_angle=0.0,
                output_width=0, skewed_decon=False)
    args.update(kw)
    cdx.rl_init(shape_zyx, p, **args)
    return p


def _oracle_state(oracle, shape_zyx, table, **kw):
    nz, ny, nx = shape_zyx
    a = dict(dr=0.1, dz=0.1, dr_psf=0.1, dz_psf=0.1, deskew_angle=0.0, rotation_angle=0.0,
             output_width=0, skewed_decon=False)
    a.update(kw)
    return oracle.rl_init(nx, ny, nz, a["dr"], a["dz"], a["dr_psf"], a["dz_psf"], a["deskew_angle"],
                          a["rotation_angle"], a["output_width"], a["skewed_decon"],
                          synth.otf_table_to_image(table))


# ---------------------------------------------------------------- FFT
@pytest.mark.parametrize("shape", [(4, 6, 10), (9, 15, 21), (16, 18, 20), (25, 27, 49),
                                   (7, 5, 3), (32, 64, 100), (64, 256, 256), (100, 256, 756),
                                   (27, 35, 1620),
                                   # every length of the specialised-plan registry on each axis
                                   (128, 128, 128), (32, 512, 1024), (64, 1024, 256),
                                   (256, 64, 512), (100, 18, 756),
                                   # generated compile-time plans (y in [128, 512], z in
                                   # [32, 160]): two radices, three (343 = 7*7*7), odd
                                   (35, 135, 40), (49, 343, 24), (125, 500, 30),
                                   (147, 160, 20), (45, 405, 36),
                                   # generated x-pass plans (x in [128, 1024])
                                   (6, 10, 135), (5, 7, 343), (4, 9, 1000), (3, 12, 882)])
def test_rfft3d_matches_numpy(cdx, torch_cuda, shape):
    torch = torch_cuda
    nz, ny, nx = shape
    x = np.random.default_rng(nz * 1000 + ny + nx).standard_normal(shape).astype(np.float32)
    dx = _dev(torch, x)
    out = torch.empty((nz, ny, nx // 2 + 1), dtype=torch.complex64, device="cuda")
    ok = cdx.lib().cdx_rfft3d_device(ctypes.c_void_p(dx.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                     nx, ny, nz, _stream(torch))
    assert ok == 1, cdx.lib().cdx_last_error()
    ref = np.fft.rfftn(x.astype(np.float64))
    assert rel_l2(out.cpu().numpy(), ref) < 2e-6


@pytest.mark.parametrize("shape", [(16, 32, 30), (20, 24, 45), (64, 256, 256), (100, 256, 756),
                                   (128, 128, 128), (32, 512, 1024),
                                   (16, 40, 1620),     # registered x length (deskewed 1024)
                                   (63, 189, 50),      # generated y and z plans
                                   (150, 448, 24),
                                   (128, 512, 1024)])  # the 128x512x1024 precision-study grid
@pytest.mark.parametrize("conj", [0, 1])
def test_conv3d_matches_oracle(cdx, oracle, torch_cuda, tmp_path, shape, conj):
    torch = torch_cuda
    nz, ny, nx = shape
    tab = synth.gaussian_otf_table(nx // 2 + 1, nz, 1.5, 3.0)
    tab = (tab * np.exp(0.3j * np.arange(nz))[None, :]).astype(np.complex64)  # complex OTF
    _init(cdx, tmp_path, shape, tab)
    st = _oracle_state(oracle, shape, tab)
    x = np.random.default_rng(5).random(shape).astype(np.float32)
    dx = _dev(torch, x)
    dy = torch.empty_like(dx)
    ok = cdx.lib().cdx_conv3d_device(ctypes.c_void_p(dx.data_ptr()), ctypes.c_void_p(dy.data_ptr()),
                                     nx, ny, nz, conj, _stream(torch))
    assert ok == 1, cdx.lib().cdx_last_error()
    H = oracle.otf_on_grid(st, nx, ny, nz, dtype=np.float64)
    F = np.fft.rfftn(x.astype(np.float64)) * (np.conj(H) if conj else H)
    ref = np.fft.irfftn(F, s=shape, axes=(0, 1, 2))
    assert rel_l2(dy.cpu().numpy(), ref) < 2e-6


# ---------------------------------------------------------------- RL
RL_CASES = {
    "plain": dict(n_iters=10),
    "one_iter": dict(n_iters=1),
    "two_iter": dict(n_iters=2),
    "three_iter": dict(n_iters=3),
    "apodize": dict(n_iters=4, napodize=5),
    "zblend": dict(n_iters=4, nzblend=3),
    "duprev": dict(n_iters=4, dup_rev_stack=True),
    "no_iter": dict(n_iters=0),
}


@pytest.mark.parametrize("case", sorted(RL_CASES))
def test_rl_interface_matches_oracle(cdx, oracle, torch_cuda, tmp_path, case):
    kw = RL_CASES[case]
    shape = (22, 50, 64)  # nz rounded down to 21 (crop at the origin); odd z length
    raw = synth.bead_stack(shape, n_beads=40, psf_sigma_xy=1.2, psf_sigma_z=2.0, seed=11)
    tab = synth.gaussian_otf_table(33, 20, 1.2, 2.0)
    _init(cdx, tmp_path, shape, tab)
    assert cdx.output_shape() == (21, 50, 64)
    out = cdx.rl_decon(raw, background=100.0, **kw)
    st = _oracle_state(oracle, shape, tab)
    ref, _ = oracle.rl_interface(st, raw, background=100.0, nIters=kw.get("n_iters", 10),
                                 napodize=kw.get("napodize", 0), nZblend=kw.get("nzblend", 0),
                                 bDupRevStack=kw.get("dup_rev_stack", False))
    assert out.shape == ref.shape
    assert rel_l2(out, ref) < RL_TOL
    cdx.rl_cleanup()


@pytest.mark.parametrize("nx", [128, 256, 512, 756, 1024, 1620])
def test_rl_registered_x_lengths_match_oracle(cdx, oracle, torch_cuda, tmp_path, nx):
    """Every compile-time x plan through the whole loop (prediction, ratio,
    update and dot products); 1024 runs its ratio and update passes on their
    own 8*16*8 plan."""
    shape = (12, 24, nx)
    raw = synth.bead_stack(shape, n_beads=30, psf_sigma_xy=1.2, psf_sigma_z=1.5, seed=nx)
    tab = synth.gaussian_otf_table(nx // 2 + 1, 12, 1.2, 2.0)
    _init(cdx, tmp_path, shape, tab)
    assert cdx.decon_grid() == shape
    out = cdx.rl_decon(raw, background=100.0, n_iters=6)
    st = _oracle_state(oracle, shape, tab)
    ref, _ = oracle.rl_interface(st, raw, background=100.0, nIters=6)
    cdx.rl_cleanup()
    assert rel_l2(out, ref) < RL_TOL


def test_rl_bleach_rescale_state(cdx, oracle, torch_cuda, tmp_path):
    shape = (16, 40, 48)
    tab = synth.gaussian_otf_table(25, 16, 1.2, 2.0)
    _init(cdx, tmp_path, shape, tab)
    st = _oracle_state(oracle, shape, tab)
    a = synth.bead_stack(shape, n_beads=30, seed=21)
    b = (a.astype(np.float64) * 0.7).astype(np.uint16)
    for raw in (a, b):  # the second stack is rescaled to the first one's intensity
        out = cdx.rl_decon(raw, background=90.0, n_iters=3, rescale=True)
        ref, _ = oracle.rl_interface(st, raw, background=90.0, nIters=3, bDoRescale=True)
        assert rel_l2(out, ref) < RL_TOL
    cdx.rl_cleanup()


def test_rl_deskew_rotate_matches_oracle(cdx, oracle, torch_cuda, tmp_path):
    # stage-scan geometry, scaled down: deskew before decon, rotate after
    shape = (31, 40, 96)
    raw = synth.bead_stack(shape, n_beads=40, psf_sigma_xy=1.3, psf_sigma_z=3.0, seed=13)
    tab = synth.gaussian_otf_table(49, 32, 1.3, 3.0)
    kw = dict(dr=0.104, dz=0.3, dr_psf=0.104, dz_psf=0.2, deskew_angle=31.5, rotation_angle=31.5)
    _init(cdx, tmp_path, shape, tab, **kw)
    st = _oracle_state(oracle, shape, tab, **kw)
    nzr, nyr, nxr = cdx.output_shape()
    desk_shape = (st.output_nz, st.output_ny, st.deskewedXdim)
    out, desk = cdx.rl_decon(raw, background=100.0, n_iters=5, save_deskewed=True,
                             deskewed_shape=desk_shape)
    ref, ref_desk = oracle.rl_interface(st, raw, background=100.0, nIters=5, bSaveDeskewedRaw=True)
    np.testing.assert_array_equal(desk, ref_desk)  # deskew is bit exact
    assert out.shape == ref.shape == (nzr, nyr, nxr)
    assert rel_l2(out, ref) < RL_TOL
    cdx.rl_cleanup()


# ---------------------------------------------------------------- geometry
@pytest.mark.parametrize("factor,nxo,shift,pad", [(2.459538982623965, 756, 0, 0.0),
                                                  (-1.3, 300, 3, 7.5), (0.0, 100, -2, 0.0)])
def test_deskew_bit_exact(cdx, oracle, torch_cuda, factor, nxo, shift, pad):
    torch = torch_cuda
    a = np.random.default_rng(3).random((20, 8, 200)).astype(np.float32) * 1000
    da = _dev(torch, a)
    out = torch.empty((20, 8, nxo), dtype=torch.float32, device="cuda")
    ok = cdx.lib().cdx_deskew_device(ctypes.c_void_p(da.data_ptr()), 200, 8, 20, factor,
                                     ctypes.c_void_p(out.data_ptr()), nxo, shift, pad, _stream(torch))
    assert ok == 1
    ref = oracle.deskew(a, factor, nxo, shift, pad)
    np.testing.assert_array_equal(out.cpu().numpy().view(np.uint32), ref.view(np.uint32))


def test_rotate_bit_exact(cdx, oracle, torch_cuda):
    torch = torch_cuda
    a = np.random.default_rng(4).random((40, 6, 120)).astype(np.float32) * 1000
    rot = np.array([0.5657086, 0.34666663, -0.52249855, 0.85264015], np.float32)
    nxr, nzr = oracle.rotated_dims(120, 40, rot)
    da = _dev(torch, a)
    out = torch.empty((nzr, 6, nxr), dtype=torch.float32, device="cuda")
    ok = cdx.lib().cdx_rotate_device(ctypes.c_void_p(da.data_ptr()), 120, 6, 40,
                                     rot.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                     ctypes.c_void_p(out.data_ptr()), nxr, nzr, _stream(torch))
    assert ok == 1
    ref = oracle.rotate(a, rot, nxr, nzr)
    np.testing.assert_array_equal(out.cpu().numpy().view(np.uint32), ref.view(np.uint32))


def test_deskew_interface_width_rule(cdx, oracle, torch_cuda, tmp_path):
    a = np.random.default_rng(6).random((10, 4, 64)).astype(np.float32)
    # explicit output width
    out = cdx.deskew(a, 31.5, 0.3, 0.104, output_width=90, extra_shift=1, pad_val=2.0)
    f = np.cos(np.deg2rad(np.float32(31.5)).astype(np.float64)) * np.float32(0.3) / np.float32(0.104)
    import math
    f = math.cos(float(np.float32(31.5)) * math.pi / 180.) * float(np.float32(0.3)) / float(np.float32(0.104))
    ref = oracle.deskew(a, f, 90, 1, 2.0)
    np.testing.assert_array_equal(out, ref)


def test_camcor_matches_oracle(cdx, oracle, torch_cuda):
    rng = np.random.default_rng(8)
    raw = rng.integers(80, 3000, size=(6, 32, 40)).astype(np.uint16)
    raw[:, :2, :] = 60  # below the offset: the result saturates at 0
    p = synth.camcor_params(32, 40, seed=9)
    p[0] *= 500.0  # strong residual charge
    cdx.camcor_init(raw.shape, p)
    out = cdx.camcor(raw)
    ref = oracle.camcor(raw, p)
    d = np.abs(out.astype(np.int32) - ref.astype(np.int32))
    assert d.max() <= 1 and np.count_nonzero(d) <= raw.size // 1000
    assert np.all(out[:, :2, :] == 0)


def _trilinear_border(a, x, y, z):
    """Trilinear sample (texel centres at i + 0.5, zero outside) with the
    interpolation weights rounded to 8 fractional bits like texture units."""
    nz, ny, nx = a.shape
    xb, yb, zb = x - 0.5, y - 0.5, z - 0.5
    i, j, k = np.floor(xb).astype(int), np.floor(yb).astype(int), np.floor(zb).astype(int)
    ax = np.round((xb - i) * 256) / 256
    ay = np.round((yb - j) * 256) / 256
    az = np.round((zb - k) * 256) / 256

    def T(zz, yy, xx):
        ok = (xx >= 0) & (xx < nx) & (yy >= 0) & (yy < ny) & (zz >= 0) & (zz < nz)
        return np.where(ok, a[np.clip(zz, 0, nz - 1), np.clip(yy, 0, ny - 1), np.clip(xx, 0, nx - 1)], 0)

    return ((1 - az) * ((1 - ay) * ((1 - ax) * T(k, j, i) + ax * T(k, j, i + 1)) +
                        ay * ((1 - ax) * T(k, j + 1, i) + ax * T(k, j + 1, i + 1))) +
            az * ((1 - ay) * ((1 - ax) * T(k + 1, j, i) + ax * T(k + 1, j, i + 1)) +
                  ay * ((1 - ax) * T(k + 1, j + 1, i) + ax * T(k + 1, j + 1, i + 1))))


def test_affine_matches_texture_trilinear(cdx, torch_cuda):
    rng = np.random.default_rng(10)
    a = rng.random((12, 20, 24)).astype(np.float32)
    M = np.eye(4, dtype=np.float32)
    M[:3, :3] = [[0.9, 0.1, 0.0], [-0.1, 0.95, 0.05], [0.0, 0.02, 1.0]]
    M[:3, 3] = [1.3, -0.7, 0.4]
    out = cdx.affine(a, M)
    z, y, x = np.meshgrid(np.arange(12), np.arange(20), np.arange(24), indexing="ij")
    pts = np.stack([x, y, z, np.ones_like(x)], -1).astype(np.float64) @ M.T.astype(np.float64)
    ref = _trilinear_border(a.astype(np.float64), pts[..., 0] + 0.5, pts[..., 1] + 0.5, pts[..., 2] + 0.5)
    assert np.max(np.abs(out - ref)) < 5e-3
    # the non-RA kernel adds half a voxel, so the identity reproduces the input
    np.testing.assert_allclose(cdx.affine(a, np.eye(4, dtype=np.float32)), a, atol=1e-6)
    # the RA kernel does not (geometryTransform.cu:236-248): the identity
    # samples at voxel corners, averaging 2x2x2 neighbours with zero border
    out2 = cdx.affine_ra(a, np.eye(4, dtype=np.float32), 0.1, 0.1, 0.3)
    ref2 = _trilinear_border(a.astype(np.float64), x.astype(np.float64), y.astype(np.float64),
                             z.astype(np.float64))
    assert np.max(np.abs(out2 - ref2)) < 5e-3


# ---------------------------------------------------------------- acceleration factor
@pytest.mark.parametrize("n", [1, 1000, 8192, 8193, 19353600])
def test_accel_factor_matches_reference_formula(cdx, torch_cuda, n):
    torch = torch_cuda
    rng = np.random.default_rng(n)
    g1 = rng.standard_normal(n).astype(np.float32)
    g2 = (0.8 * g1 + 0.3 * rng.standard_normal(n)).astype(np.float32)
    d1, d2 = _dev(torch, g1), _dev(torch, g2)
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    lam = torch.zeros(1, dtype=torch.float32, device="cuda")
    for _ in range(2):  # the scratch is reused
        ok = cdx.lib().cdx_accel_factor_device(ctypes.c_void_p(d1.data_ptr()), ctypes.c_void_p(d2.data_ptr()),
                                               n, ctypes.c_void_p(out.data_ptr()),
                                               ctypes.c_void_p(lam.data_ptr()), _stream(torch))
        assert ok == 1
        o = out.cpu().numpy()
        num = np.sum((g1 * g2).astype(np.float32), dtype=np.float64)
        den = np.sum((g2 * g2).astype(np.float32), dtype=np.float64)
        np.testing.assert_allclose(o[:2], [num, den], rtol=1e-12)
        l = num / (den + np.finfo(np.float32).eps)
        np.testing.assert_allclose(o[2], l, rtol=1e-12)
        assert lam.item() == np.float32(min(max(l, 0.0), 1.0))
