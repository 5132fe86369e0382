"""The mixed-precision form: x-pass DFT stages as tcgen05 MMAs in split TF32
(cdx_set_dft_form(1)).

* The forward x pass alone, through the 3D FFT hook, against numpy float64
  for every length with a tensor-core plan (odd and partial row tiles).
* The RL loop (inverse x pass with the ratio and with the update + dot
  products) against the reference's own kernels with cuFFT and FP64, for
  every such length.
* The precision study of the 128x512x1024 grid: 20 iterations in the mixed
  and the plain form against FP64 (relative L2 and max-abs), the mixed form
  held to the 1e-4 target.

Tolerances: 3D FFT relative L2 <= 4e-6 against float64 (the plain form is
held to 2e-6 there; split TF32 keeps about 22 significant bits); RL <= 1e-4
against FP64 and <= 2e-5 against the reference's float32 kernels."""

import ctypes

import numpy as np
import pytest

from conftest import rel_l2
from cudadecon_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture
def mixed(cdx, torch_cuda):
    assert cdx.lib().cdx_set_dft_form(1) == 1
    try:
        yield cdx
    finally:
        cdx.lib().cdx_set_dft_form(0)


@pytest.fixture(scope="module")
def ref(torch_cuda):
    from oracle import ref_kernels as RK
    ok, why = RK.available()
    if not ok:
        pytest.skip(why)
    return RK


def test_form_switch_and_supported_lengths(cdx):
    L = cdx.lib()
    assert L.cdx_get_dft_form() == 0
    assert [L.cdx_tc_length_supported(n) for n in (256, 512, 756, 1024, 100, 1620)] == \
        [1, 1, 1, 1, 0, 0]
    assert L.cdx_set_dft_form(2) == 0
    assert L.cdx_get_dft_form() == 0


@pytest.mark.parametrize("shape", [(3, 9, 256), (5, 7, 512), (4, 15, 756), (3, 21, 1024),
                                   (16, 64, 1024), (100, 256, 756)])
def test_rfft3d_mixed_matches_numpy(mixed, torch_cuda, shape):
    torch = torch_cuda
    nz, ny, nx = shape
    x = np.random.default_rng(nz * 1000 + ny + nx).standard_normal(shape).astype(np.float32)
    dx = torch.from_numpy(x).cuda()
    out = torch.empty((nz, ny, nx // 2 + 1), dtype=torch.complex64, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    L = mixed.lib()
    ok = L.cdx_rfft3d_device(ctypes.c_void_p(dx.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                             nx, ny, nz, s)
    assert ok == 1, L.cdx_last_error()
    torch.cuda.synchronize()
    e = rel_l2(out.cpu().numpy(), np.fft.rfftn(x.astype(np.float64)))
    print(f"\nmixed rfft3d {shape}: rel L2 vs float64 {e:.2e}")
    assert e < 4e-6


@pytest.mark.parametrize("shape", [(12, 40, 256), (9, 21, 512), (20, 36, 756), (10, 30, 1024)])
def test_rl_mixed_vs_reference_and_fp64(mixed, oracle, ref, torch_cuda, tmp_path, shape):
    raw = synth.bead_stack(shape, n_beads=60, psf_sigma_xy=1.3, psf_sigma_z=2.5, seed=sum(shape))
    nz, ny, nx = shape
    tab = synth.gaussian_otf_table(129, 64, 1.3, 2.5)
    p = tmp_path / "otf.tif"
    synth.write_otf(p, tab)
    kw = dict(dr=0.104, dz=0.3, dr_psf=0.104, dz_psf=0.25)
    mixed.rl_init(shape, p, **kw)
    gz, gy, gx = mixed.decon_grid()
    L = mixed.lib()
    assert L.cdx_lambda_trace(10) == 1
    mine = mixed.rl_decon(raw, background=100.0, n_iters=10)
    lam = np.zeros(10, np.float32)
    assert L.cdx_lambda_read(lam.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), 10) == 10
    L.cdx_lambda_trace(0)
    assert L.cdx_tc_status() == 1
    mixed.lib().cdx_set_dft_form(0)
    plain = mixed.rl_decon(raw, background=100.0, n_iters=10)
    mixed.lib().cdx_set_dft_form(1)
    mixed.rl_cleanup()
    st = oracle.rl_init(nx, ny, nz, kw["dr"], kw["dz"], kw["dr_psf"], kw["dz_psf"], 0.0, 0.0, 0,
                        False, synth.otf_table_to_image(tab))
    X0 = oracle.bgsub(raw[:gz, :gy, :gx].astype(np.float32), 100.0)
    theirs, lam_ref = ref.rl_iterations(X0, X0, tab, oracle.kscales(st, gx, gy, gz), 10)
    fp64 = oracle.rl_iterations(X0, X0, oracle.otf_on_grid(st, gx, gy, gz, dtype=np.float64), 10,
                                dtype=np.float64)
    e_ref, e64, e64p = rel_l2(mine, theirs), rel_l2(mine, fp64), rel_l2(plain, fp64)
    print(f"\nmixed RL {gz}x{gy}x{gx} 10 it: rel L2 vs reference {e_ref:.2e}, vs FP64 {e64:.2e} "
          f"(plain form vs FP64 {e64p:.2e}); max |lambda - reference| "
          f"{np.abs(lam - lam_ref).max():.2e}")
    assert e_ref < 2e-5
    assert e64 < 1e-4
    assert np.abs(lam - lam_ref).max() < 1e-4


def test_precision_study_128x512x1024_mixed_and_plain_vs_fp64(cdx, oracle, torch_cuda, tmp_path):
    torch = torch_cuda
    from oracle import rl_oracle_torch as OT
    shape = (128, 512, 1024)
    nz, ny, nx = shape
    tab = synth.gaussian_otf_table(129, 64, 1.5, 4.0)
    p = tmp_path / "otf.tif"
    synth.write_otf(p, tab)
    cdx.rl_init(shape, p, dr=0.1, dz=0.2, dr_psf=0.1, dz_psf=0.2)
    st = oracle.rl_init(nx, ny, nz, 0.1, 0.2, 0.1, 0.2, 0.0, 0.0, 0, False,
                        synth.otf_table_to_image(tab))
    raw = synth.bead_stack_gpu(shape, n_beads=4000, psf_sigma_xy=1.5, psf_sigma_z=4.0, seed=1003)
    L = cdx.lib()
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    outs = {}
    try:
        for form, code in (("plain", 0), ("mixed", 1)):
            assert L.cdx_set_dft_form(code) == 1
            o = torch.empty(shape, dtype=torch.float32, device="cuda")
            ok = L.cdx_RL_device(ctypes.c_void_p(raw.data_ptr()), nx, ny, nz,
                                 ctypes.c_void_p(o.data_ptr()), None, 100.0, False, False, 20, 0,
                                 0, 0, 0.0, False, False, s)
            assert ok == 1, L.cdx_last_error()
            torch.cuda.synchronize()
            outs[form] = o
        assert L.cdx_tc_status() == 1
    finally:
        L.cdx_set_dft_form(0)
    cdx.rl_cleanup()
    X0 = (raw.float() - 100.0).clamp_min_(0.0)
    fp64 = OT.rl_iterations(X0, X0, OT.otf_on_grid(st, nx, ny, nz), 20)
    res = {}
    for form, o in outs.items():
        d = o.double() - fp64
        res[form] = (float(d.norm() / fp64.norm()), float(d.abs().max()))
    top = float(fp64.abs().max())
    print(f"\n128x512x1024 20 it vs FP64 (max |x| {top:.4g}): "
          + "; ".join(f"{f}: rel L2 {e:.2e}, max abs {m:.3g}" for f, (e, m) in res.items()))
    assert res["mixed"][0] < 1e-4
    assert res["plain"][0] < 1e-4
