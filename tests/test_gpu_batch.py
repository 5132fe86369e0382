"""Batched deconvolution of uneven stacks (cdx_RL_batch_device), config-4
style: several stacks of different shapes, each with its own OTF, in one
call whose iterations run as one CUDA graph.

Each stack must give exactly what the single-stack path gives (RL_interface
initialised for that stack and OTF), which the parity tests pin against the
oracle: the same kernels run on the same data, so the comparison is bit for
bit."""

import numpy as np
import pytest

from cudadecon_gb300 import synth

pytestmark = pytest.mark.gpu

# (shape zyx, PSF sigma xy / z in pixels, background, dr, dz)
STACKS = [
    ((22, 50, 64), (1.2, 2.0), 100.0, 0.104, 0.3),   # z cropped 22 -> 21
    ((16, 64, 128), (1.4, 2.5), 90.0, 0.1, 0.25),    # registered x length (128)
    ((32, 40, 45), (1.0, 1.8), 110.0, 0.11, 0.3),    # odd x, registered z length (32)
    ((33, 30, 100), (1.1, 2.2), 100.0, 0.104, 0.2),  # z 33 -> 32
    ((20, 36, 756), (1.3, 3.0), 100.0, 0.104, 0.15), # registered x length (756)
]


def _stacks(torch, seed0=0):
    out = []
    for i, (shape, (sxy, sz), bg, dr, dz) in enumerate(STACKS):
        raw = synth.bead_stack(shape, n_beads=30, psf_sigma_xy=sxy, psf_sigma_z=sz, seed=seed0 + i)
        tab = synth.gaussian_otf_table(33 + 2 * i, 16 + 4 * i, sxy, sz)
        out.append(dict(raw_np=raw, raw=torch.from_numpy(raw).cuda(), otf=tab, dr=dr, dz=dz,
                        dr_psf=dr, dz_psf=dz, background=bg))
    return out


def _single(cdx, tmp_path, d, n_iters):
    p = tmp_path / "otf.tif"
    synth.write_otf(p, d["otf"])
    cdx.rl_init(d["raw_np"].shape, p, dr=d["dr"], dz=d["dz"], dr_psf=d["dr_psf"],
                dz_psf=d["dz_psf"], deskew_angle=0.0, rotation_angle=0.0)
    out = cdx.rl_decon(d["raw_np"], background=d["background"], n_iters=n_iters)
    cdx.rl_cleanup()
    return out


def test_batch_matches_single_stack_path(cdx, torch_cuda, tmp_path):
    torch = torch_cuda
    st = _stacks(torch)
    outs = cdx.rl_batch(st, n_iters=5)
    torch.cuda.synchronize()
    assert cdx.lib().cdx_batch_last_launch_count() >= len(st) * 5 * 9
    for d, o in zip(st, outs):
        ref = _single(cdx, tmp_path, d, 5)
        got = o.cpu().numpy()
        assert got.shape == ref.shape == cdx.batch_grid(d["raw_np"].shape)
        assert np.array_equal(got, ref)


def test_batch_graph_replay_and_recapture(cdx, torch_cuda, tmp_path):
    torch = torch_cuda
    cdx.rl_batch(_stacks(torch), n_iters=4)
    # same shapes, new data: the kept graph is replayed
    st = _stacks(torch, seed0=100)
    outs = cdx.rl_batch(st, n_iters=4)
    torch.cuda.synchronize()
    for d, o in zip(st, outs):
        assert np.array_equal(o.cpu().numpy(), _single(cdx, tmp_path, d, 4))
    # another iteration count: captured again
    outs = cdx.rl_batch(st, n_iters=3)
    torch.cuda.synchronize()
    for d, o in zip(st[:2], outs[:2]):
        assert np.array_equal(o.cpu().numpy(), _single(cdx, tmp_path, d, 3))
    # fewer stacks: new state
    outs = cdx.rl_batch(st[1:3], n_iters=3)
    torch.cuda.synchronize()
    for d, o in zip(st[1:3], outs):
        assert np.array_equal(o.cpu().numpy(), _single(cdx, tmp_path, d, 3))
    cdx.lib().cdx_batch_release()


def test_batch_zero_iterations_returns_conditioned_stack(cdx, torch_cuda, tmp_path):
    torch = torch_cuda
    st = _stacks(torch)[:2]
    outs = cdx.rl_batch(st, n_iters=0)
    torch.cuda.synchronize()
    for d, o in zip(st, outs):
        gz, gy, gx = cdx.batch_grid(d["raw_np"].shape)
        want = np.maximum(d["raw_np"][:gz, :gy, :gx].astype(np.float32) - d["background"], 0)
        assert np.array_equal(o.cpu().numpy(), want)
    cdx.lib().cdx_batch_release()


def test_batch_host_buffers_match_device_batch(cdx, torch_cuda):
    """cdx_RL_batch_host (pinned host stacks and results, transfers inside
    the graph) gives the device batch's results bit for bit, on repeated
    calls, after new host buffers (the graph is captured again), and for
    nIters = 0 (the conditioned stacks)."""
    torch = torch_cuda
    st = _stacks(torch)
    ref = [o.cpu().numpy() for o in cdx.rl_batch(st, n_iters=5)]
    torch.cuda.synchronize()
    host = [dict(d, raw=d["raw"].cpu().pin_memory()) for d in st]
    for _ in range(2):
        outs = cdx.rl_batch_host(host, n_iters=5)
        for o, r in zip(outs, ref):
            assert np.array_equal(o.numpy(), r)
    host2 = [dict(d, raw=d["raw"].clone().pin_memory()) for d in host]
    for o, r in zip(cdx.rl_batch_host(host2, n_iters=5), ref):
        assert np.array_equal(o.numpy(), r)
    for d, o in zip(st, cdx.rl_batch_host(host2, n_iters=0)):
        gz, gy, gx = cdx.batch_grid(d["raw_np"].shape)
        want = np.maximum(d["raw_np"][:gz, :gy, :gx].astype(np.float32) - d["background"], 0)
        assert np.array_equal(o.numpy(), want)
    cdx.lib().cdx_batch_release()


def test_batch_host_rejects_pageable_buffers(cdx, torch_cuda):
    st = _stacks(torch_cuda)[:1]
    host = [dict(st[0], raw=st[0]["raw"].cpu())]  # not pinned
    with pytest.raises(cdx.CudaDeconError, match="page-locked"):
        cdx.rl_batch_host(host, n_iters=2)


def test_batch_results_do_not_depend_on_the_stream_counts(cdx, torch_cuda):
    """The stacks' chains spread over 1, 3 or 16 streams (device batch) and
    1 or 5 (host batch) give the default counts' results bit for bit; the
    graph is captured again when a count changes; out-of-range counts are
    refused."""
    torch = torch_cuda
    st = _stacks(torch)
    default = cdx.batch_streams()
    assert default == (2, 2)
    ref = [o.cpu().numpy() for o in cdx.rl_batch(st, n_iters=4)]
    host = [dict(d, raw=d["raw"].cpu().pin_memory()) for d in st]
    try:
        for k in (1, 3, 16):
            assert cdx.batch_streams(device=k) == (k, 2)
            outs = cdx.rl_batch(st, n_iters=4)
            torch.cuda.synchronize()
            for o, r in zip(outs, ref):
                assert np.array_equal(o.cpu().numpy(), r)
        for k in (1, 5):
            assert cdx.batch_streams(host=k)[1] == k
            for o, r in zip(cdx.rl_batch_host(host, n_iters=4), ref):
                assert np.array_equal(o.numpy(), r)
        L = cdx.lib()
        assert L.cdx_batch_set_streams(0, 4) == 0
        assert L.cdx_batch_set_streams(2, 17) == 0
    finally:
        cdx.batch_streams(device=default[0], host=default[1])
        cdx.lib().cdx_batch_release()
    assert cdx.batch_streams() == default
