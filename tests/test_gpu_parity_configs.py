"""RL parity on the workloads and branches beyond the two pinned grids.

* 128x512x1024, 20 iterations (the precision study's grid): against the FP64
  oracle and against the reference's own kernels with cuFFT.
* A full 3D (non radially averaged) OTF file: the non-RA branch of
  dev_otfinterpolate (src/RLgpuImpl.cu:274-319) through the whole RL loop,
  against the reference's kernels.
* Six of the 64 uneven stacks of the batched workload (including the longest
  x), through cdx_RL_batch_device, against the reference's kernels and FP64;
  all 64 stacks of the headline batch, as bench.py generates them, against
  the reference's kernels.
* The acceleration factors of the library (float-float dot products, lambda
  in double) against the reference's (float products summed in double,
  RLgpuImpl.cu:584-592; lambda on the host, RL-Biggs-Andrews.cpp:297-298).
* The time-lapse grid (256x1024x1024 raw deskewed to 256x1024x1620), 20
  iterations with a Gaussian OTF, against FP64 on every 16th voxel along each
  axis (and on the whole volume).
* camcor chained into deskew + RL + rotate on the device, against the
  reference's camcor kernel followed by the float32 oracle.
* One length of every kind of tuned plan in use (padded stage layouts, two-
  or three-radix plans, other batches, radix orders, register budgets; from
  cudadecon_gb300/tuned_plans.json), through RL against the reference's
  kernels.

FP64 on the large grids is the torch restatement of the oracle
(oracle/rl_oracle_torch.py, cuFFT double), pinned to the numpy FP64 oracle in
tests/test_oracle_cpu.py.  Tolerances: relative L2 <= 1e-5 against the
reference's float32 kernels, <= 1e-4 against FP64."""

import ctypes
import json
import math
import sys
from pathlib import Path

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


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


def _run_device(cdx, torch, raw_dev, n_iters, background=100.0):
    """cdx_RL_device on a device u16 stack; returns the device result."""
    L = cdx.lib()
    nz, ny, nx = raw_dev.shape
    out = torch.empty(cdx.output_shape(), dtype=torch.float32, device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ok = L.cdx_RL_device(_vp(raw_dev), nx, ny, nz, _vp(out), None, background, False, False,
                         n_iters, 0, 0, 0, 0.0, False, False, st)
    assert ok == 1, L.cdx_last_error()
    torch.cuda.synchronize()
    return out


def _start_volume(cdx, torch, st, raw_dev, background):
    """The loop's start: crop, background subtraction, deskew (the library's
    bit-exact deskew, pinned to the reference kernel)."""
    gz, gy, gx = cdx.decon_grid()
    x = (raw_dev[:st.output_nz, :st.output_ny, :st.output_nx].float() - background).clamp_min_(0.0)
    if abs(st.deskewFactor) > 0:
        nz, ny, nx = x.shape
        out = torch.empty((gz, gy, gx), dtype=torch.float32, device="cuda")
        assert cdx.lib().cdx_deskew_device(_vp(x.contiguous()), nx, ny, nz, st.deskewFactor,
                                           _vp(out), gx, 0, 0.0, None) == 1
        torch.cuda.synchronize()
        x = out
    assert tuple(x.shape) == (gz, gy, gx)
    return x.contiguous()


def _errs(a, b):
    a = a.double()
    b = b.double()
    return (float(torch_norm(a - b) / torch_norm(b)), float((a - b).abs().max()),
            float(b.abs().max()))


def torch_norm(t):
    return t.double().norm()


def test_rl_128x512x1024_20_iterations_vs_fp64_and_reference(cdx, oracle, torch_cuda, ref,
                                                             tmp_path):
    torch = torch_cuda
    from oracle import rl_oracle_torch as OT
    shape = (128, 512, 1024)
    nz, ny, nx = shape
    tab = synth.gaussian_otf_table(129, 64, 1.5, 4.0)
    p = tmp_path / "otf.tif"
    synth.write_otf(p, tab)
    kw = dict(dr=0.1, dz=0.2, dr_psf=0.1, dz_psf=0.2)
    cdx.rl_init(shape, p, **kw)
    st = oracle.rl_init(nx, ny, nz, 0.1, 0.2, 0.1, 0.2, 0.0, 0.0, 0, False,
                        synth.otf_table_to_image(tab))
    raw = synth.bead_stack_gpu(shape, n_beads=4000, psf_sigma_xy=1.5, psf_sigma_z=4.0, seed=1003)
    mine = _run_device(cdx, torch, raw, 20)
    X0 = _start_volume(cdx, torch, st, raw, 100.0)
    cdx.rl_cleanup()
    theirs, _ = ref.rl_iterations(X0.cpu().numpy(), X0.cpu().numpy(), tab,
                                  oracle.kscales(st, nx, ny, nz), 20)
    theirs = torch.from_numpy(theirs).cuda()
    H = OT.otf_on_grid(st, nx, ny, nz)
    fp64 = OT.rl_iterations(X0, X0, H, 20)
    del H
    e_ref = rel_l2(mine.cpu().numpy(), theirs.cpu().numpy())
    e64, m64, top = _errs(mine, fp64)
    e64r, m64r, _ = _errs(theirs, fp64)
    print(f"\n128x512x1024 20 it: rel L2 vs reference {e_ref:.2e}; vs FP64: ours {e64:.2e} "
          f"(max abs {m64:.3g} of {top:.4g}), reference {e64r:.2e} (max abs {m64r:.3g})")
    assert e_ref < 1e-5
    assert e64 < 1e-4


def _otf3d_image(nzo, nyo, nxp, sig, shift):
    """OTF file image (nz_otf, ny_otf, 2*(nxp/2+1)) float32 of a Gaussian PSF
    on an (nzo, nyo, nxp) grid displaced by `shift` pixels from the origin
    (a complex OTF; the rfft of a real PSF keeps the Hermitian symmetry)."""
    z = np.fft.fftfreq(nzo) * nzo
    y = np.fft.fftfreq(nyo) * nyo
    x = np.fft.fftfreq(nxp) * nxp
    Z, Y, X = np.meshgrid(z - shift[0], y - shift[1], x - shift[2], indexing="ij")
    psf = np.exp(-0.5 * ((Z / sig[0]) ** 2 + (Y / sig[1]) ** 2 + (X / sig[2]) ** 2))
    otf = np.fft.rfftn(psf / psf.sum()).astype(np.complex64)
    return otf, np.ascontiguousarray(otf).view(np.float32).reshape(nzo, nyo, -1)


def test_rl_full_3d_otf_vs_reference(cdx, oracle, ref, torch_cuda, tmp_path):
    raw = synth.bead_stack((40, 96, 120), n_beads=80, psf_sigma_xy=1.4, psf_sigma_z=2.5, seed=2024)
    nz, ny, nx = raw.shape
    otf, img = _otf3d_image(32, 64, 64, (2.5, 1.4, 1.4), (0.3, -0.2, 0.25))
    p = tmp_path / "otf3d.tif"
    synth.write_tiff(p, img)
    kw = dict(dr=0.104, dz=0.3, dr_psf=0.1, dz_psf=0.25)
    cdx.rl_init(raw.shape, p, **kw)
    st = oracle.rl_init(nx, ny, nz, kw["dr"], kw["dz"], kw["dr_psf"], kw["dz_psf"], 0.0, 0.0, 0,
                        False, img)
    assert st.ny_otf == 64 and st.nz_otf == 32 and st.nx_otf == 33
    gz, gy, gx = cdx.decon_grid()
    mine = cdx.rl_decon(raw, background=100.0, n_iters=10)
    cdx.rl_cleanup()
    X0 = oracle.bgsub(raw[:gz, :gy, :gx].astype(np.float32), 100.0)
    theirs, _ = ref.rl_iterations(X0, X0, st.otf, oracle.kscales(st, gx, gy, gz), 10)
    H64 = oracle.otf_on_grid(st, gx, gy, gz, dtype=np.float64)
    fp64 = oracle.rl_iterations(X0, X0, H64, 10, dtype=np.float64)
    e_ref, e64 = rel_l2(mine, theirs), rel_l2(mine, fp64)
    print(f"\n3D OTF (32x64x33) on {gz}x{gy}x{gx}, 10 it: rel L2 vs reference {e_ref:.2e}, "
          f"vs FP64 {e64:.2e} (reference vs FP64 {rel_l2(theirs, fp64):.2e})")
    assert e_ref < 1e-5
    assert e64 < 1e-4


BATCH_SEED = 1003


def _batch_shapes():
    """The 64 shapes of the batched workload, in its seeded draw order."""
    rng = np.random.default_rng(BATCH_SEED)
    shapes, jit = [], []
    for _ in range(64):
        shapes.append(tuple(int(rng.choice(synth.smooth_sizes(lo, hi)))
                            for lo, hi in ((32, 160), (128, 512), (128, 1024))))
        jit.append(rng.uniform(0.8, 1.2, 2))
    return shapes, jit


def test_batch_subset_of_uneven_stacks_vs_reference_and_fp64(cdx, oracle, ref, torch_cuda):
    torch = torch_cuda
    from oracle import rl_oracle_torch as OT
    shapes, jit = _batch_shapes()
    vol = [int(np.prod(s)) for s in shapes]
    longest = max(range(64), key=lambda i: (shapes[i][2], -vol[i]))
    pick = [longest] + [i for i in sorted(range(64), key=lambda i: vol[i]) if i != longest][:5]
    gen = torch.Generator(device="cuda")
    gen.manual_seed(BATCH_SEED)
    stacks = []
    for i in pick:
        lam = 100.0 + 3000.0 * (torch.rand(shapes[i], generator=gen, device="cuda") < 2e-4).float()
        raw = torch.poisson(lam, generator=gen).clamp_(0, 65535).to(torch.int32).to(torch.uint16)
        tab = synth.gaussian_otf_table(129, 64, 1.5 * jit[i][0], 4.0 * jit[i][1])
        stacks.append(dict(raw=raw, otf=tab, dr=0.104, dz=0.3, dr_psf=0.104, dz_psf=0.3,
                           background=100.0))
    outs = cdx.rl_batch(stacks, n_iters=10)
    torch.cuda.synchronize()
    cdx.lib().cdx_batch_release()
    for i, d, o in zip(pick, stacks, outs):
        gz, gy, gx = cdx.batch_grid(shapes[i])
        st = oracle.rl_init(shapes[i][2], shapes[i][1], shapes[i][0], 0.104, 0.3, 0.104, 0.3,
                            0.0, 0.0, 0, False, synth.otf_table_to_image(d["otf"]))
        X0 = (d["raw"][:gz, :gy, :gx].float() - 100.0).clamp_min_(0.0).contiguous()
        theirs, _ = ref.rl_iterations(X0.cpu().numpy(), X0.cpu().numpy(), d["otf"],
                                      oracle.kscales(st, gx, gy, gz), 10)
        fp64 = OT.rl_iterations(X0, X0, OT.otf_on_grid(st, gx, gy, gz), 10)
        e_ref = rel_l2(o.cpu().numpy(), theirs)
        e64 = _errs(o, fp64)[0]
        print(f"\nstack {i} {shapes[i]} -> {gz}x{gy}x{gx}: rel L2 vs reference {e_ref:.2e}, "
              f"vs FP64 {e64:.2e}")
        assert e_ref < 1e-5, (i, e_ref)
        assert e64 < 1e-4, (i, e64)


def test_batch_all_64_headline_stacks_vs_reference_and_fp64(cdx, oracle, ref, torch_cuda):
    """Every stack of the headline batch, generated as bench.py generates it
    (the same seeded draws), through cdx_RL_batch_device with the default
    graph streams and the tuned plans, against the reference's kernels +
    cuFFT on the same stack (relative L2 <= 1e-5 for each) and against FP64
    (<= 1e-4 for each; the whole batch's error is printed)."""
    torch = torch_cuda
    shapes, jit = _batch_shapes()
    gen = torch.Generator(device="cuda")
    gen.manual_seed(BATCH_SEED)
    stacks = []
    for i in range(64):
        lam = 100.0 + 3000.0 * (torch.rand(shapes[i], generator=gen, device="cuda") < 2e-4).float()
        raw = torch.poisson(lam, generator=gen).clamp_(0, 65535).to(torch.int32).to(torch.uint16)
        tab = synth.gaussian_otf_table(129, 64, 1.5 * jit[i][0], 4.0 * jit[i][1])
        stacks.append(dict(raw=raw, otf=tab, dr=0.104, dz=0.3, dr_psf=0.104, dz_psf=0.3,
                           background=100.0))
    outs = cdx.rl_batch(stacks, n_iters=10)
    torch.cuda.synchronize()
    cdx.lib().cdx_batch_release()
    from oracle import rl_oracle_torch as OT
    worst, worst64 = (0.0, None), (0.0, None)
    sq = sq64 = ref2 = 0.0
    for i, (d, o) in enumerate(zip(stacks, outs)):
        gz, gy, gx = cdx.batch_grid(shapes[i])
        st = oracle.rl_init(shapes[i][2], shapes[i][1], shapes[i][0], 0.104, 0.3, 0.104, 0.3,
                            0.0, 0.0, 0, False, synth.otf_table_to_image(d["otf"]))
        X0 = (d["raw"][:gz, :gy, :gx].float() - 100.0).clamp_min_(0.0).contiguous()
        Xn = X0.cpu().numpy()
        theirs, _ = ref.rl_iterations(Xn, Xn, d["otf"], oracle.kscales(st, gx, gy, gz), 10)
        e = rel_l2(o.cpu().numpy(), theirs)
        worst = max(worst, (e, (i, shapes[i])))
        fp64 = OT.rl_iterations(X0, X0, OT.otf_on_grid(st, gx, gy, gz), 10)
        diff = o.double() - fp64
        e64 = float(diff.norm() / fp64.norm())
        ref64 = float((torch.from_numpy(theirs).cuda().double() - fp64).norm() / fp64.norm())
        worst64 = max(worst64, (e64, (i, shapes[i], ref64)))
        sq64 += float(diff.norm()) ** 2
        ref2 += float(fp64.norm()) ** 2
        del fp64, diff
        assert e < 1e-5, (i, shapes[i], e)
        assert e64 < 1e-4, (i, shapes[i], e64)
    print(f"\n64 headline stacks, 10 it: worst rel L2 vs reference {worst[0]:.2e} (stack "
          f"{worst[1][0]}, {worst[1][1]}); vs FP64 worst {worst64[0]:.2e} (stack "
          f"{worst64[1][0]}; the reference's own {worst64[1][2]:.2e}), whole batch "
          f"{math.sqrt(sq64 / ref2):.2e}")


def test_lambda_sequence_vs_reference_fp64_sums(cdx, oracle, ref, torch_cuda, tmp_path):
    raw = synth.bead_stack((101, 256, 512), n_beads=300, psf_sigma_xy=1.3, psf_sigma_z=3.0,
                           n_filaments=12, seed=1002)
    nz, ny, nx = raw.shape
    tab = synth.gaussian_otf_table(129, 64, 1.3, 3.0)
    p = tmp_path / "otf.tif"
    synth.write_otf(p, tab)
    kw = dict(dr=0.104, dz=0.3, dr_psf=0.104, dz_psf=0.2, deskew_angle=31.5)
    cdx.rl_init(raw.shape, p, **kw)
    L = cdx.lib()
    n = 15
    assert L.cdx_lambda_trace(n) == 1
    cdx.rl_decon(raw, background=100.0, n_iters=n)
    lam = np.zeros(n, np.float32)
    assert L.cdx_lambda_read(lam.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), n) == n
    L.cdx_lambda_trace(0)
    gz, gy, gx = cdx.decon_grid()
    cdx.rl_cleanup()
    st = oracle.rl_init(nx, ny, nz, 0.104, 0.3, 0.104, 0.2, 31.5, 0.0, 0, False,
                        synth.otf_table_to_image(tab))
    X0 = oracle.bgsub(raw[:st.output_nz, :st.output_ny, :st.output_nx].astype(np.float32), 100.0)
    X0 = ref.deskew(X0, st.deskewFactor, st.deskewedXdim)
    _, lam_ref = ref.rl_iterations(X0, X0, tab, oracle.kscales(st, gx, gy, gz), n)
    l64 = []
    oracle.rl_iterations(X0, X0, oracle.otf_on_grid(st, gx, gy, gz, dtype=np.float64), n,
                         dtype=np.float64, lambdas=l64)
    d_ref = np.abs(lam.astype(np.float64) - lam_ref)
    d64 = np.abs(lam[2:].astype(np.float64) - np.asarray(l64))
    print(f"\nlambdas (ours) {np.round(lam, 5).tolist()}\nmax |ours - reference| {d_ref.max():.2e}, "
          f"max |ours - FP64 oracle| {d64.max():.2e}, "
          f"max |reference - FP64 oracle| {np.abs(lam_ref[2:] - l64).max():.2e}")
    assert np.all(lam[:2] == 0.0)
    assert d_ref.max() < 2e-5
    assert d64.max() < 1e-4


def test_timelapse_grid_20_iterations_vs_fp64_subsampled(cdx, oracle, torch_cuda, tmp_path):
    torch = torch_cuda
    from oracle import rl_oracle_torch as OT
    shape = (256, 1024, 1024)
    nz, ny, nx = shape
    tab = synth.gaussian_otf_table(129, 64, 1.3, 3.0)
    p = tmp_path / "otf.tif"
    synth.write_otf(p, tab)
    kw = dict(dr=0.104, dz=0.3, dr_psf=0.104, dz_psf=0.2, deskew_angle=31.5, rotation_angle=0.0)
    cdx.rl_init(shape, p, **kw)
    gz, gy, gx = cdx.decon_grid()
    assert (gz, gy, gx) == (256, 1024, 1620)
    st = oracle.rl_init(nx, ny, nz, 0.104, 0.3, 0.104, 0.2, 31.5, 0.0, 0, False,
                        synth.otf_table_to_image(tab))
    raw = synth.bead_stack_gpu(shape, n_beads=20000, psf_sigma_xy=1.3, psf_sigma_z=3.0, seed=1005)
    mine = _run_device(cdx, torch, raw, 20)
    X0 = _start_volume(cdx, torch, st, raw, 100.0)
    cdx.rl_cleanup()
    del raw
    fp64 = OT.rl_iterations(X0, X0, OT.otf_on_grid(st, gx, gy, gz), 20)
    del X0
    sub = (slice(None, None, 16),) * 3
    e_sub, m_sub, top = _errs(mine[sub], fp64[sub])
    e_all = _errs(mine, fp64)[0]
    print(f"\n256x1024x1620 20 it vs FP64: rel L2 {e_all:.2e} (all voxels), {e_sub:.2e} on the "
          f"16^3-subsampled set (max abs {m_sub:.3g} of {top:.4g})")
    assert e_sub < 1e-4
    assert e_all < 1e-4


def test_camcor_then_rl_chain_vs_reference_camcor_and_oracle(cdx, oracle, ref, torch_cuda,
                                                             tmp_path):
    """Camera correction, deskew, 20 RL iterations and rotation on the device
    (the time-lapse pipeline on a reduced stack), against the reference's
    camcor kernel followed by the float32 oracle's RL_interface."""
    torch = torch_cuda
    shape = (64, 128, 256)
    nz, ny, nx = shape
    raw = synth.bead_stack(shape, n_beads=120, psf_sigma_xy=1.3, psf_sigma_z=3.0, seed=31)
    cam = synth.camcor_params(ny, nx, seed=32)
    tab = synth.gaussian_otf_table(129, 64, 1.3, 3.0)
    p = tmp_path / "otf.tif"
    synth.write_otf(p, tab)
    kw = dict(dr=0.104, dz=0.3, dr_psf=0.104, dz_psf=0.2, deskew_angle=31.5, rotation_angle=31.5)
    cdx.rl_init(shape, p, **kw)
    d_raw = torch.from_numpy(raw).cuda()
    d_cam = torch.from_numpy(cam).cuda()
    d_cc = torch.empty_like(d_raw)
    L = cdx.lib()
    assert L.cdx_camcor_device(_vp(d_raw), nx, ny, nz, _vp(d_cam), _vp(d_cc), None) == 1
    mine = _run_device(cdx, torch, d_cc, 20).cpu().numpy()
    cdx.rl_cleanup()
    cc_ref = ref.camcor(raw, cam)
    assert np.array_equal(d_cc.cpu().numpy(), cc_ref)
    st = oracle.rl_init(nx, ny, nz, 0.104, 0.3, 0.104, 0.2, 31.5, 31.5, 0, False,
                        synth.otf_table_to_image(tab))
    want, _ = oracle.rl_interface(st, cc_ref, background=100.0, nIters=20)
    e = rel_l2(mine, want)
    print(f"\ncamcor -> deskew -> 20 it -> rotate on {shape}: rel L2 vs oracle {e:.2e}")
    assert mine.shape == want.shape
    assert e < 1e-5


@pytest.mark.parametrize("shape", [(12, 20, 243), (10, 16, 245), (8, 24, 1000), (9, 30, 135)])
def test_rl_generated_x_plans_vs_reference(cdx, oracle, ref, torch_cuda, tmp_path, shape):
    """RL through the generated compile-time x plans (x in [128, 1024] outside
    the hand-tuned registry; 243 and 245 need just over 48 KB of shared
    memory in the update pass) against the reference's kernels + cuFFT."""
    raw = synth.bead_stack(shape, n_beads=40, psf_sigma_xy=1.3, psf_sigma_z=2.5, seed=sum(shape))
    nz, ny, nx = shape
    tab = synth.gaussian_otf_table(129, 64, 1.3, 2.5)
    p = tmp_path / "otf.tif"
    synth.write_otf(p, tab)
    kw = dict(dr=0.104, dz=0.3, dr_psf=0.104, dz_psf=0.25)
    cdx.rl_init(shape, p, **kw)
    gz, gy, gx = cdx.decon_grid()
    mine = cdx.rl_decon(raw, background=100.0, n_iters=8)
    cdx.rl_cleanup()
    st = oracle.rl_init(nx, ny, nz, kw["dr"], kw["dz"], kw["dr_psf"], kw["dz_psf"], 0.0, 0.0, 0,
                        False, synth.otf_table_to_image(tab))
    X0 = oracle.bgsub(raw[:gz, :gy, :gx].astype(np.float32), 100.0)
    theirs, _ = ref.rl_iterations(X0, X0, tab, oracle.kscales(st, gx, gy, gz), 8)
    e = rel_l2(mine, theirs)
    print(f"\ngenerated x plan {gz}x{gy}x{gx}, 8 it: rel L2 vs reference {e:.2e}")
    assert e < 1e-5


def _tuned_variants():
    """(axis, feature, length): one length per kind of tuned plan in use."""
    pkg = Path(__file__).resolve().parents[1] / "cudadecon_gb300"
    if str(pkg) not in sys.path:
        sys.path.insert(0, str(pkg))
    import gen_plans as G
    tuned = json.loads(G.TUNED.read_text()) if G.TUNED.exists() else {}
    lens = G.lengths()
    picked = {}
    for axis in "xyz":
        for L in lens[axis]:
            rad, b, rx, pads = G.choose(axis, L, None, tuned)
            c0 = G.candidates(axis, L)[0]
            feats = []
            if pads != [0, 0]:
                feats.append("padded")
            if len(rad) != len(c0[0]):
                feats.append(f"{len(rad)} radices")
            if rx:
                feats.append("more registers")
            if b < c0[1]:
                feats.append("smaller batch")
            if b > c0[1]:
                feats.append("larger batch")
            if len(rad) == len(c0[0]) and rad != c0[0]:
                feats.append("radix order")
            for f in feats:
                picked.setdefault((axis, f), L)
    return sorted((a, f, L) for (a, f), L in picked.items())


@pytest.mark.parametrize("axis,feature,L", _tuned_variants())
def test_rl_tuned_plan_variants_vs_reference(cdx, oracle, ref, torch_cuda, tmp_path, axis,
                                             feature, L):
    """RL through a tuned generated plan on one axis (the other two lengths
    small) against the reference's kernels + cuFFT, 8 iterations."""
    shape = {"x": (10, 24, L), "y": (10, L, 128), "z": (L, 24, 128)}[axis]
    raw = synth.bead_stack(shape, n_beads=40, psf_sigma_xy=1.3, psf_sigma_z=2.5, seed=L)
    nz, ny, nx = shape
    tab = synth.gaussian_otf_table(129, 64, 1.3, 2.5)
    p = tmp_path / "otf.tif"
    synth.write_otf(p, tab)
    kw = dict(dr=0.104, dz=0.3, dr_psf=0.104, dz_psf=0.25)
    cdx.rl_init(shape, p, **kw)
    gz, gy, gx = cdx.decon_grid()
    assert (gz, gy, gx) == shape
    mine = cdx.rl_decon(raw, background=100.0, n_iters=8)
    cdx.rl_cleanup()
    st = oracle.rl_init(nx, ny, nz, kw["dr"], kw["dz"], kw["dr_psf"], kw["dz_psf"], 0.0, 0.0, 0,
                        False, synth.otf_table_to_image(tab))
    X0 = oracle.bgsub(raw.astype(np.float32), 100.0)
    theirs, _ = ref.rl_iterations(X0, X0, tab, oracle.kscales(st, gx, gy, gz), 8)
    e = rel_l2(mine, theirs)
    print(f"\ntuned {axis} plan ({feature}) {gz}x{gy}x{gx}, 8 it: rel L2 vs reference {e:.2e}")
    assert e < 1e-5


def test_convergence_norm_trace_vs_oracle(cdx, oracle, torch_cuda, tmp_path):
    """cdx_change_trace: the relative change of the estimate per iteration,
    ||X_{k+1} - X_k|| / ||X_k|| summed in FP64 on the device, against the
    float32 oracle's (same float32 estimates up to FFT rounding; relative
    difference <= 1e-3 per iteration) and the FP64 oracle's (<= 1e-2); the
    trace adds two launches per iteration and none when it is off."""
    shape = (40, 96, 128)
    nz, ny, nx = shape
    raw = synth.bead_stack(shape, n_beads=60, psf_sigma_xy=1.3, psf_sigma_z=2.5, seed=77)
    tab = synth.gaussian_otf_table(129, 64, 1.3, 2.5)
    p = tmp_path / "otf.tif"
    synth.write_otf(p, tab)
    kw = dict(dr=0.104, dz=0.3, dr_psf=0.104, dz_psf=0.25)
    cdx.rl_init(shape, p, **kw)
    L = cdx.lib()
    n = 12
    cdx.rl_decon(raw, background=100.0, n_iters=n)
    plain_launches = L.cdx_last_launch_count()
    assert L.cdx_change_trace(n) == 1
    try:
        mine = cdx.rl_decon(raw, background=100.0, n_iters=n)
        assert L.cdx_last_launch_count() == plain_launches + 2 * n
        got = np.zeros(n, np.float64)
        assert L.cdx_change_read(got.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), n) == n
    finally:
        L.cdx_change_trace(0)
    assert L.cdx_change_read(np.zeros(1).ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 1) == -1
    gz, gy, gx = cdx.decon_grid()
    cdx.rl_cleanup()
    st = oracle.rl_init(nx, ny, nz, kw["dr"], kw["dz"], kw["dr_psf"], kw["dz_psf"], 0.0, 0.0, 0,
                        False, synth.otf_table_to_image(tab))
    X0 = oracle.bgsub(raw[:gz, :gy, :gx].astype(np.float32), 100.0)
    H = oracle.otf_on_grid(st, gx, gy, gz)
    n32, n64 = [], []
    oracle.rl_iterations(X0, X0, H, n, norms=n32)
    oracle.rl_iterations(X0, X0, oracle.otf_on_grid(st, gx, gy, gz, dtype=np.float64), n,
                         dtype=np.float64, norms=n64)
    r32 = np.abs(got - n32) / np.array(n32)
    r64 = np.abs(got - n64) / np.array(n64)
    print(f"\nconvergence norms {gz}x{gy}x{gx}: first {got[0]:.4e}, last {got[-1]:.4e}; "
          f"max rel diff vs float32 oracle {r32.max():.2e}, vs FP64 {r64.max():.2e}")
    assert np.all(got > 0)
    assert r32.max() < 1e-3
    assert r64.max() < 1e-2
