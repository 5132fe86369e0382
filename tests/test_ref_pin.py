"""The library against the reference's own CUDA kernels on the GPU.

The reference's kernels (src/RLgpuImpl.cu, src/geometryTransform.cu,
src/camcor.cu) are compiled from its sources to PTX (oracle/build.py) and
launched with cuFFT in the order of its host code (oracle/ref_runner.cu).
Skipped when that build is absent.  Tolerances: geometry and camcor bit
for bit; the RL loop (our FFTs against cuFFT) relative L2 <= 1e-5; the error
of both against the float64 oracle is reported and bounded (<= 1e-4)."""

import numpy as np
import pytest

from conftest import rel_l2
from cudadecon_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref(torch_cuda):
    from oracle import ref_kernels as RK
    ok, why = RK.available()
    if not ok:
        pytest.skip(why)
    return RK


def _stage_scan_state(oracle, raw_shape=(101, 256, 512)):
    nz, ny, nx = raw_shape
    tab = synth.gaussian_otf_table(129, 64, 1.3, 3.0)
    st = oracle.rl_init(nx, ny, nz, 0.104, 0.3, 0.104, 0.2, 31.5, 31.5, 0, False,
                        synth.otf_table_to_image(tab))
    return st, tab


def test_deskew_bit_exact_vs_reference_kernel(cdx, ref, oracle, torch_cuda):
    import ctypes
    torch = torch_cuda
    st, _ = _stage_scan_state(oracle)
    a = (np.random.default_rng(1).random((100, 16, 512)) * 1000).astype(np.float32)
    for factor, nxo, shift, pad in [(st.deskewFactor, st.deskewedXdim, 0, 0.0), (-0.7, 600, 3, 5.0)]:
        r = ref.deskew(a, factor, nxo, shift, pad)
        da = torch.from_numpy(a).cuda()
        out = torch.empty((100, 16, nxo), dtype=torch.float32, device="cuda")
        assert cdx.lib().cdx_deskew_device(ctypes.c_void_p(da.data_ptr()), 512, 16, 100, factor,
                                           ctypes.c_void_p(out.data_ptr()), nxo, shift, pad,
                                           None) == 1
        torch.cuda.synchronize()
        np.testing.assert_array_equal(out.cpu().numpy().view(np.uint32), r.view(np.uint32))
        np.testing.assert_array_equal(oracle.deskew(a, factor, nxo, shift, pad).view(np.uint32),
                                      r.view(np.uint32))


def test_rotate_bit_exact_vs_reference_kernel(cdx, ref, oracle, torch_cuda):
    import ctypes
    torch = torch_cuda
    st, _ = _stage_scan_state(oracle)
    a = (np.random.default_rng(2).random((100, 8, 756)) * 1000).astype(np.float32)
    nxr, nzr = oracle.rotated_dims(756, 100, st.rot)
    r = ref.rotate(a, st.rot, nxr, nzr)
    da = torch.from_numpy(a).cuda()
    out = torch.empty((nzr, 8, nxr), dtype=torch.float32, device="cuda")
    assert cdx.lib().cdx_rotate_device(ctypes.c_void_p(da.data_ptr()), 756, 8, 100,
                                       st.rot.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                       ctypes.c_void_p(out.data_ptr()), nxr, nzr, None) == 1
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy().view(np.uint32), r.view(np.uint32))
    np.testing.assert_array_equal(oracle.rotate(a, st.rot, nxr, nzr).view(np.uint32),
                                  r.view(np.uint32))


def test_camcor_exact_vs_reference_kernel(cdx, ref, oracle):
    rng = np.random.default_rng(3)
    raw = rng.integers(50, 6000, size=(8, 64, 96)).astype(np.uint16)
    p = synth.camcor_params(64, 96, seed=4)
    p[0] *= 800.0
    r = ref.camcor(raw, p)
    cdx.camcor_init(raw.shape, p)
    np.testing.assert_array_equal(cdx.camcor(raw), r)
    d = np.abs(oracle.camcor(raw, p).astype(np.int32) - r.astype(np.int32))
    assert d.max() <= 1


def test_affine_exact_vs_reference_kernel(cdx, ref):
    rng = np.random.default_rng(5)
    a = rng.random((20, 30, 40)).astype(np.float32)
    M = np.eye(4, dtype=np.float32)
    M[:3, :3] = [[0.9, 0.1, 0.0], [-0.1, 0.95, 0.05], [0.0, 0.02, 1.0]]
    M[:3, 3] = [1.3, -0.7, 0.4]
    np.testing.assert_array_equal(cdx.affine(a, M), ref.affine(a, M))
    np.testing.assert_array_equal(cdx.affine_ra(a, M, 0.1, 0.1, 0.3),
                                  ref.affine(a, M, ra=True, dx=0.1, dy=0.1, dz=0.3))


def _rl_case(cdx, ref, oracle, tmp_path, raw, tab, n_iters, init_kw, background=100.0):
    nz, ny, nx = raw.shape
    p = tmp_path / "otf.tif"
    synth.write_otf(p, tab)
    cdx.rl_init(raw.shape, p, **init_kw)
    st = oracle.rl_init(nx, ny, nz, init_kw["dr"], init_kw["dz"], init_kw["dr_psf"],
                        init_kw["dz_psf"], init_kw.get("deskew_angle", 0.0), 0.0, 0, False,
                        synth.otf_table_to_image(tab))
    gz, gy, gx = cdx.decon_grid()
    X0 = oracle.bgsub(raw[:st.output_nz, :st.output_ny, :st.output_nx].astype(np.float32), background)
    if abs(st.deskewFactor) > 0:
        X0 = ref.deskew(X0, st.deskewFactor, st.deskewedXdim)
    assert X0.shape == (gz, gy, gx)
    mine = cdx.rl_decon(raw, background=background, n_iters=n_iters)
    theirs, lam = ref.rl_iterations(X0, X0, tab, oracle.kscales(st, gx, gy, gz), n_iters)
    H64 = oracle.otf_on_grid(st, gx, gy, gz, dtype=np.float64)
    fp64 = oracle.rl_iterations(X0, X0, H64, n_iters, dtype=np.float64)
    cdx.rl_cleanup()
    return mine, theirs, fp64, lam


def test_rl_plain_64x256x256_vs_reference(cdx, ref, oracle, tmp_path):
    # the 64x256x256 bead stack: 10 iterations, background 100, no deskew
    raw = synth.bead_stack((64, 256, 256), n_beads=200, seed=1001)
    tab = synth.gaussian_otf_table(129, 64, 1.5, 4.0)
    mine, theirs, fp64, lam = _rl_case(cdx, ref, oracle, tmp_path, raw, tab, 10,
                                       dict(dr=0.1, dz=0.2, dr_psf=0.1, dz_psf=0.2))
    e_ref = rel_l2(mine, theirs)
    e64, e64_ref = rel_l2(mine, fp64), rel_l2(theirs, fp64)
    print(f"\nbeads 64x256x256 10 it: rel L2 vs reference {e_ref:.2e}; vs FP64: ours {e64:.2e}, "
          f"reference {e64_ref:.2e}; lambdas {np.round(lam, 4).tolist()}")
    assert e_ref < 1e-5
    assert e64 < 1e-4


def test_rl_stage_scan_deskewed_vs_reference(cdx, ref, oracle, tmp_path):
    # the stage-scan stack: deskew 31.5 deg to 100x256x756, 15 iterations
    raw = synth.bead_stack((101, 256, 512), n_beads=300, psf_sigma_xy=1.3, psf_sigma_z=3.0,
                           n_filaments=12, seed=1002)
    tab = synth.gaussian_otf_table(129, 64, 1.3, 3.0)
    mine, theirs, fp64, lam = _rl_case(cdx, ref, oracle, tmp_path, raw, tab, 15,
                                       dict(dr=0.104, dz=0.3, dr_psf=0.104, dz_psf=0.2,
                                            deskew_angle=31.5))
    e_ref = rel_l2(mine, theirs)
    e64, e64_ref = rel_l2(mine, fp64), rel_l2(theirs, fp64)
    print(f"\nstage-scan 100x256x756 15 it: rel L2 vs reference {e_ref:.2e}; vs FP64: ours {e64:.2e}, "
          f"reference {e64_ref:.2e}; lambdas {np.round(lam, 4).tolist()}")
    assert e_ref < 1e-5
    assert e64 < 1e-4
