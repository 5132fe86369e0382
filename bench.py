#!/usr/bin/env python3
"""Benchmark: Richardson-Lucy voxel-iterations/s, batched uneven stacks in
the plain FP32 and the mixed-precision forms.

Headline workload (one step = one call that deconvolves every stack):
64 synthetic stacks of uneven shape, z from the 2,3,5,7-smooth sizes in
[32, 160], y in [128, 512], x in [128, 1024] (seeded), each with its own
Gaussian OTF (sigmas jittered by +-20%), uint16 with a Poisson background
and sparse beads, 10 Biggs-Andrews RL iterations, through
cdx_RL_batch_device (one CUDA graph of every stack's iterations).

  value   : plain FP32 form, stacks resident in HBM, CUDA events on the
            launch stream; voxel-iterations/s of all decon grids
  forms   : the same in the mixed-precision form (x-pass DFT stages as
            tcgen05 MMAs in split TF32) and the ratio mixed / plain
  e2e     : the same batch with host buffers (cdx_RL_batch_host): each
            step uploads the 64 raw stacks from pinned host memory and
            downloads the 64 results, inside the call's graph
  roofline: the dominant pass of the batch (per-pass CUDA events over
            the 64 stacks, one profiled call per stack outside the timed
            region) against the measured HBM copy bandwidth, with its DRAM
            traffic from profiles/traffic_batch_x_ratio.json; whole_call is
            56 B per voxel-iteration over the timed batch call
  secondary:
    stage_scan : 101x256x512 u16 at 31.5 deg -> deskew to 100x256x756,
                 15 iterations, rotate (single stack, RL_interface and
                 cdx_RL_device; pinned and pageable e2e; per-pass timing)
    grid_128x512x1024 : 20 iterations, plain and mixed forms
    timelapse  : 8 timepoints x 2 channels of 256x1024x1024 u16: camcor,
                 deskew (-> 256x1024x1620), 20 iterations, rotate, with
                 one OTF per channel
  cpu_baseline : the CPU restatement in oracle/ (scipy.fft float32, all
                 host cores) on a bounded sample of the stage-scan volume

--impl reference times the reference's own implementation of the path on
the same batch: its CUDA kernels (compiled to PTX from its sources) with
cuFFT, launched in the order of one RL_interface call per stack
(oracle/ref_runner.cu), one reference session (plans, OTF, buffers) per
stack; the reference has no CPU implementation of this loop.

Multi-GPU: independent stacks do not exchange data, so N ranks run N
replicas (weak scaling); value is the work of all ranks over the slowest
rank's time.
"""

from __future__ import annotations

import argparse
import ctypes
import datetime
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

ALG_BYTES_PER_VOXEL_ITER = 56.0  # one fused iteration, float32 storage
# algorithmic bytes per voxel of each pass of an iteration (cdx_profile order:
# x forward, y, z, y inverse, x ratio, y, z conjugate, y inverse, x update)
PASS_BYTES = [16, 8, 8, 8, 12, 8, 8, 8, 20]
NOMINAL_HBM_GBS = 8000.0         # GB300's nominal HBM3e bandwidth

BATCH = {"stacks": 64, "iterations": 10, "seed": 1003, "z": (32, 160), "y": (128, 512),
         "x": (128, 1024)}
BATCH_NAME = (f"{BATCH['stacks']} uneven stacks, z/y/x 2-3-5-7-smooth in {BATCH['z']}/"
              f"{BATCH['y']}/{BATCH['x']}, own Gaussian OTF each, {BATCH['iterations']} RL it")

STAGE = dict(
    name="stage-scan light-sheet 101x256x512 u16, deskew 31.5deg -> 100x256x756, 15 RL it, rotate",
    raw_shape=(101, 256, 512), dr=0.104, dz=0.3, dr_psf=0.104, dz_psf=0.2, angle=31.5,
    background=100.0, n_iters=15, otf_nr=129, otf_nz=64, psf_sigma_xy=1.3, psf_sigma_z=3.0,
    seed=1002,
)
GRID3 = dict(shape=(128, 512, 1024), n_iters=20, seed=1003)
LAPSE = dict(timepoints=8, channels=2, shape=(256, 1024, 1024), n_iters=20, angle=31.5,
             dr=0.104, dz=0.3, seed=1005)


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------- inputs
def stage_inputs(tmpdir):
    from cudadecon_gb300 import synth
    w = STAGE
    raw = synth.bead_stack(w["raw_shape"], n_beads=300, sigma_range=(0.5, 2.0),
                           amp_range=(500.0, 5000.0), psf_sigma_xy=w["psf_sigma_xy"],
                           psf_sigma_z=w["psf_sigma_z"], background=w["background"],
                           n_filaments=12, seed=w["seed"])
    tab = synth.gaussian_otf_table(w["otf_nr"], w["otf_nz"], w["psf_sigma_xy"], w["psf_sigma_z"])
    otf_path = Path(tmpdir) / "otf.tif"
    synth.write_otf(otf_path, tab)
    return raw, tab, otf_path


def batch_inputs(dev):
    """The 64 stacks (device u16 tensors) with their OTF tables, seeded."""
    import torch
    from cudadecon_gb300 import synth
    rng = np.random.default_rng(BATCH["seed"])
    gen = torch.Generator(device=dev)
    gen.manual_seed(BATCH["seed"])
    stacks = []
    for _ in range(BATCH["stacks"]):
        shape = tuple(int(rng.choice(synth.smooth_sizes(*BATCH[a]))) for a in ("z", "y", "x"))
        j = rng.uniform(0.8, 1.2, 2)
        tab = synth.gaussian_otf_table(129, 64, 1.5 * j[0], 4.0 * j[1])
        lam = 100.0 + 3000.0 * (torch.rand(shape, generator=gen, device=dev) < 2e-4).float()
        raw = torch.poisson(lam, generator=gen).clamp_(0, 65535).to(torch.int32).to(torch.uint16)
        stacks.append(dict(raw=raw, otf=tab, dr=0.104, dz=0.3, dr_psf=0.104, dz_psf=0.3,
                           background=100.0))
    return stacks


class ClockSampler:
    """nvidia-smi clock/throttle sampling of the timed region.  Sampling starts
    before the warm-up (nvidia-smi takes a while to produce its first row) at
    50 ms; the samples time-stamped inside the timed region are kept, or, when
    the region is shorter than the interval, the ones nearest to it."""

    Q = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, dev_index):
        self.dev = dev_index
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self, t0=None, t1=None):
        """Summary of the samples time-stamped within [t0, t1] (wall-clock
        seconds), else of the two nearest to that window."""
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        rows = [r.split(",") for r in Path(self.f.name).read_text().splitlines() if r.strip()]
        os.unlink(self.f.name)
        if t0 is not None and t1 is not None and rows:
            def stamp(r):
                try:
                    return datetime.datetime.strptime(r[0].strip(), "%Y/%m/%d %H:%M:%S.%f").timestamp()
                except (ValueError, IndexError):
                    return None
            timed = [(stamp(r), r) for r in rows]
            timed = [(t, r) for t, r in timed if t is not None]
            inside = [r for t, r in timed if t0 <= t <= t1]
            if inside:
                rows = inside
            elif timed:
                mid = 0.5 * (t0 + t1)
                rows = [r for _, r in sorted(timed, key=lambda tr: abs(tr[0] - mid))[:2]]
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- CPU baseline
def cpu_prepare(raw, tab):
    """CPU-baseline leg: the oracle's deskewed start volume and OTF grid."""
    from oracle import rl_oracle as O
    from cudadecon_gb300 import synth
    w = STAGE
    nz, ny, nx = w["raw_shape"]
    st = O.rl_init(nx, ny, nz, w["dr"], w["dz"], w["dr_psf"], w["dz_psf"], w["angle"], w["angle"],
                   0, False, synth.otf_table_to_image(tab))
    X = raw[:st.output_nz, :st.output_ny, :st.output_nx].astype(np.float32)
    X = O.bgsub(X, w["background"])
    X = O.deskew(X, st.deskewFactor, st.deskewedXdim)
    H = O.otf_on_grid(st, st.deskewedXdim, st.output_ny, st.output_nz)
    return X, H


def cpu_time_iterations(X, H, n_iters, workers):
    """Time n_iters float32 RL iterations of the oracle: (voxel-iter/s, seconds)."""
    from oracle import rl_oracle as O
    t0 = time.perf_counter()
    O.rl_iterations(X, X, H, n_iters, workers=workers)
    dt = time.perf_counter() - t0
    return X.size * n_iters / dt, dt


def cpu_time_bounded(X, H, workers, min_s=10.0, chunk=5, max_iters=60):
    """Time the oracle's iterations in runs of `chunk` (each from the start volume)
    until at least min_s seconds of work: (voxel-iter/s, seconds, iterations)."""
    n, t = 0, 0.0
    while t < min_s and n < max_iters:
        _, dt = cpu_time_iterations(X, H, chunk, workers)
        n += chunk
        t += dt
    return X.size * n / t, t, n


def cpu_baseline_leg(min_s=10.0):
    """The oracle's float32 iteration (scipy.fft, all host cores) on a bounded
    sample of the stage-scan deskewed volume."""
    with tempfile.TemporaryDirectory() as td:
        raw, tab, _ = stage_inputs(td)
    cores = os.cpu_count() or 1
    X, H = cpu_prepare(raw, tab)
    cpu_time_iterations(X, H, 1, cores)  # warm-up (FFT plans, page faults)
    v, dt, n = cpu_time_bounded(X, H, cores, min_s=min_s)
    return {"value": v, "unit": "voxel-iter/s", "cores": cores, "kind": "port",
            "sample": f"{n} RL iterations (runs of 5) on the stage-scan deskewed {X.size}-voxel "
                      f"volume (scipy.fft float32, {cores} threads), {dt:.1f} s"}


# ---------------------------------------------------------------- distribution
def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "gloo" if args.impl == "reference" else "nccl"
        dist.init_process_group(backend=backend)
        pg = dist
    return world, rank, local, pg


def max_over_ranks(x, pg, device="cpu"):
    """Largest x over all ranks (the slowest rank's time); x itself without a group.
    The tensor lives on `device` (CPU for gloo, the rank's GPU for nccl)."""
    if pg is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def events_ms(torch, stream, fn, reps):
    """Average milliseconds of fn() over reps calls, CUDA events on stream."""
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


# ---------------------------------------------------------------- reference arm
def reference_gpu_available():
    try:
        import torch
        if not torch.cuda.is_available():
            return False, "no CUDA device"
        from oracle import ref_kernels as RK
        return RK.available()
    except Exception as e:  # noqa: BLE001 - reported in the JSON line
        return False, f"{type(e).__name__}: {e}"


def run_reference(args):
    """The reference's own implementation of the path.  Its RL loop exists
    only on the GPU (its kernels with cuFFT, src/RL-Biggs-Andrews.cpp:56-450):
    the reference's CUDA sources compiled to PTX and launched in the order of
    its host code by oracle/ref_runner.cu, one session (buffers, cuFFT plans,
    OTF array, as RL_interface_init) per stack, one RL_interface call's device
    work per stack and step.  Where the reference runner is not built, the
    timed arm is the CPU restatement (oracle port) on the stage-scan volume."""
    world, rank, local, pg = dist_setup(args)
    if rank != 0:
        if pg:
            pg.barrier()
        return 0
    cpu = None if args.no_cpu_baseline else cpu_baseline_leg()
    ok, why = reference_gpu_available()
    common = {"impl": "reference", "metric": "RL voxel-iterations/s", "unit": "voxel-iter/s",
              "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
              "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
              "data": "synthetic (seeded)"}
    if not ok:
        if cpu is None:
            cpu = cpu_baseline_leg()
        v = cpu["value"]
        line = dict(common, value=v, ms_per_step=None,
                    config={"workload": STAGE["name"], "l2_policy": "n/a (CPU)",
                            "reference_gpu_unavailable": why},
                    cpu_baseline=cpu,
                    e2e={"value": v, "unit": "voxel-iter/s", "h2d_bytes_per_step": 0,
                         "d2h_bytes_per_step": 0})
        print(json.dumps(line), flush=True)
        if pg:
            pg.barrier()
        return 0
    import torch
    from cudadecon_gb300 import synth
    from oracle import ref_kernels as RK
    from oracle import rl_oracle as O
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stacks = batch_inputs(dev)
    n_iters = BATCH["iterations"]
    sess, raws, outs, vox = [], [], [], 0
    for d in stacks:
        nz, ny, nx = d["raw"].shape
        st = O.rl_init(nx, ny, nz, d["dr"], d["dz"], d["dr_psf"], d["dz_psf"], 0.0, 0.0, 0, False,
                       synth.otf_table_to_image(d["otf"]))
        s = RK.Session(st)
        gz, gy, gx = s.raw_shape
        raws.append(d["raw"][:gz, :gy, :gx].float().contiguous())
        outs.append(torch.empty(s.out_shape, dtype=torch.float32, device=dev))
        sess.append(s)
        vox += int(np.prod(s.grid))
    del stacks

    def step():
        for s, r, o in zip(sess, raws, outs):
            s.step(r, 100.0, n_iters, o)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clk = ClockSampler(local)
    clk.start()
    time.sleep(0.3)  # nvidia-smi's first row
    t_wall0 = time.time()
    ms = events_ms(torch, torch.cuda.current_stream(), step, args.steps)
    t_wall1 = time.time()
    clocks = clk.stop(t_wall0, t_wall1)
    value = vox * n_iters / (ms * 1e-3)
    finite = all(bool(torch.isfinite(o).all().item()) for o in outs)
    # e2e: the float stacks in and the results out through pinned host buffers
    h_in = [r.cpu().pin_memory() for r in raws]
    h_out = [torch.empty(o.shape, dtype=torch.float32).pin_memory() for o in outs]
    torch.cuda.synchronize()
    reps = max(1, min(args.steps, 5))
    t0 = time.perf_counter()
    for _ in range(reps):
        for s, hi, r, o, ho in zip(sess, h_in, raws, outs, h_out):
            r.copy_(hi)
            s.step(r, 100.0, n_iters, o)
            ho.copy_(o)
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / reps
    for s in sess:
        s.close()
    line = dict(common, value=value, ms_per_step=ms,
                config={"workload": BATCH_NAME, "stacks": BATCH["stacks"], "decon_voxels": vox,
                        "iterations": n_iters, "form": "reference kernels + cuFFT (plain FP32)",
                        "reference_impl": "src/RLgpuImpl.cu, geometryTransform.cu compiled to PTX "
                                          "from the reference's sources, launched in the order of "
                                          "RichardsonLucy_GPU (oracle/ref_runner.cu); one session "
                                          "(buffers, cuFFT plans, OTF) per stack, made once",
                        "l2_policy": "working set ~30 GB > 129 MB L2 (no flush needed)"},
                cpu_baseline=cpu, clocks=clocks, output_finite=finite,
                e2e={"value": vox * n_iters / e2e_s, "unit": "voxel-iter/s",
                     "h2d_bytes_per_step": int(sum(r.numel() * 4 for r in raws)),
                     "d2h_bytes_per_step": int(sum(o.numel() * 4 for o in outs))})
    print(json.dumps(line), flush=True)
    if pg:
        pg.barrier()
    return 0


# ---------------------------------------------------------------- our arm
def measure_batch(cdx, torch, dev, stream, stacks, steps, warmup, form):
    """cdx_RL_batch_device over all stacks, device-resident: (ms per call,
    voxel-iterations per call, launches per call, outputs finite)."""
    L = cdx.lib()
    assert L.cdx_set_dft_form(form) == 1
    iters = BATCH["iterations"]
    vox = sum(int(np.prod(cdx.batch_grid(tuple(d["raw"].shape)))) for d in stacks)
    outs = cdx.rl_batch(stacks, n_iters=iters, stream=stream)
    for _ in range(warmup):
        outs = cdx.rl_batch(stacks, n_iters=iters, stream=stream)
    stream.synchronize()
    ms = events_ms(torch, stream, lambda: cdx.rl_batch(stacks, n_iters=iters, stream=stream),
                   steps)
    launches = int(L.cdx_batch_last_launch_count())
    finite = all(bool(torch.isfinite(o).all().item()) for o in outs)
    L.cdx_set_dft_form(0)
    return ms, vox * iters, launches, finite


def measure_batch_passes(cdx, torch, dev, stacks):
    """Per-pass device time of the batch: each stack once more through
    cdx_RL_device with the per-pass CUDA events (cdx_profile_*), outside the
    timed region.  Returns {pass: {"ms": summed over the stacks, per
    iteration, "bytes_per_voxel", "gbs"}} and the dominant pass."""
    from cudadecon_gb300 import synth
    L = cdx.lib()
    stream = torch.cuda.Stream(device=dev)
    sp = ctypes.c_void_p(stream.cuda_stream)
    iters = BATCH["iterations"]
    tot = [0.0] * 9
    vox = 0
    td = tempfile.TemporaryDirectory()
    for i, d in enumerate(stacks):
        p = Path(td.name) / f"otf{i}.tif"
        synth.write_otf(p, d["otf"])
        nz, ny, nx = d["raw"].shape
        cdx.rl_init((nz, ny, nx), p, dr=d["dr"], dz=d["dz"], dr_psf=d["dr_psf"],
                    dz_psf=d["dz_psf"])
        gz, gy, gx = cdx.decon_grid()
        out = torch.empty(cdx.output_shape(), dtype=torch.float32, device=dev)

        def call():
            if L.cdx_RL_device(ctypes.c_void_p(d["raw"].data_ptr()), nx, ny, nz,
                               ctypes.c_void_p(out.data_ptr()), None, d["background"], False,
                               False, iters, 0, 0, 0, 0.0, False, False, sp) != 1:
                raise RuntimeError(L.cdx_last_error().decode())

        with torch.cuda.stream(stream):
            call()
            L.cdx_profile_enable(1)
            call()
        stream.synchronize()
        pm = (ctypes.c_double * 9)()
        pn = (ctypes.c_longlong * 9)()
        it_ms = ctypes.c_double(0)
        it_n = ctypes.c_longlong(0)
        L.cdx_profile_read(pm, pn, 9, ctypes.byref(it_ms), ctypes.byref(it_n))
        L.cdx_profile_enable(0)
        for k in range(9):
            tot[k] += pm[k] / max(pn[k], 1)
        vox += gz * gy * gx
        del out
    cdx.rl_cleanup()
    td.cleanup()
    passes = {}
    for k in range(9):
        passes[L.cdx_profile_pass_name(k).decode()] = {
            "ms": round(tot[k], 5), "bytes_per_voxel": PASS_BYTES[k],
            "gbs": round(PASS_BYTES[k] * vox / (tot[k] * 1e-3) / 1e9, 1) if tot[k] > 0 else None}
    top = max(passes, key=lambda n: passes[n]["ms"])
    return passes, top, vox


def measure_batch_e2e(cdx, torch, stacks, reps):
    """The batch with host buffers, through cdx_RL_batch_host: the 64 raw
    stacks in pinned host memory are uploaded and the results downloaded by
    the call itself (each stack's transfers are nodes of its chain in the
    graph, overlapping other stacks' iterations); wall clock per call."""
    iters = BATCH["iterations"]
    host = [dict(d, raw=d["raw"].cpu().pin_memory()) for d in stacks]
    outs = cdx.rl_batch_host(host, n_iters=iters)
    t0 = time.perf_counter()
    for _ in range(reps):
        outs = cdx.rl_batch_host(host, n_iters=iters, results=outs)
    s = (time.perf_counter() - t0) / reps
    return s, int(sum(h["raw"].numel() * 2 for h in host)), int(sum(o.numel() * 4 for o in outs))


def measure_stage_scan(cdx, torch, dev, steps, pg):
    """The single stage-scan stack: device-resident step, one iteration's time
    and per-pass timing, e2e through RL_interface (pinned and pageable)."""
    L = cdx.lib()
    w = STAGE
    nz, ny, nx = w["raw_shape"]
    td = tempfile.TemporaryDirectory()
    raw, tab, otf_path = stage_inputs(td.name)
    cdx.rl_init(w["raw_shape"], otf_path, dr=w["dr"], dz=w["dz"], dr_psf=w["dr_psf"],
                dz_psf=w["dz_psf"], deskew_angle=w["angle"], rotation_angle=w["angle"])
    onz, ony, onx = cdx.output_shape()
    gz, gy, gx = cdx.decon_grid()
    stream = torch.cuda.Stream(device=dev)
    sp = ctypes.c_void_p(stream.cuda_stream)
    d_raw = torch.from_numpy(raw).to(dev)
    d_out = torch.empty((onz, ony, onx), dtype=torch.float32, device=dev)
    n_iters = w["n_iters"]

    def step(iters=n_iters):
        ok = L.cdx_RL_device(ctypes.c_void_p(d_raw.data_ptr()), nx, ny, nz,
                             ctypes.c_void_p(d_out.data_ptr()), None, w["background"], False,
                             False, iters, 0, 0, 0, 0.0, False, False, sp)
        if ok != 1:
            raise RuntimeError(L.cdx_last_error().decode())

    with torch.cuda.stream(stream):
        for _ in range(3):
            step()
    stream.synchronize()
    ms = events_ms(torch, stream, step, steps)
    prepost = events_ms(torch, stream, lambda: step(0), steps)
    iter_ms = (ms - prepost) / n_iters
    vox = gx * gy * gz
    # per-pass timing (events between the passes break the programmatic
    # launch chain, so the profiled iteration is a little slower)
    L.cdx_profile_enable(1)
    with torch.cuda.stream(stream):
        for _ in range(2):
            step()
    stream.synchronize()
    pm = (ctypes.c_double * 9)()
    pn = (ctypes.c_longlong * 9)()
    it_ms = ctypes.c_double(0)
    it_n = ctypes.c_longlong(0)
    L.cdx_profile_read(pm, pn, 9, ctypes.byref(it_ms), ctypes.byref(it_n))
    L.cdx_profile_enable(0)
    pass_bytes = PASS_BYTES
    passes = {}
    for i in range(9):
        pms = pm[i] / max(pn[i], 1)
        passes[L.cdx_profile_pass_name(i).decode()] = {
            "ms": round(pms, 5), "bytes_per_voxel": pass_bytes[i],
            "gbs": round(pass_bytes[i] * vox / (pms * 1e-3) / 1e9, 1) if pms > 0 else None}
    # e2e through the reference ABI: pinned host buffers, then pageable
    h_raw = torch.from_numpy(raw).pin_memory()
    h_out = torch.empty((onz, ony, onx), dtype=torch.float32).pin_memory()
    u16p = ctypes.POINTER(ctypes.c_ushort)
    f32p = ctypes.POINTER(ctypes.c_float)
    bufs = {"pinned": (ctypes.cast(ctypes.c_void_p(h_raw.data_ptr()), u16p),
                       ctypes.cast(ctypes.c_void_p(h_out.data_ptr()), f32p))}
    p_raw = np.ascontiguousarray(raw)
    p_out = np.empty((onz, ony, onx), np.float32)
    bufs["pageable"] = (p_raw.ctypes.data_as(u16p), p_out.ctypes.data_as(f32p))
    e2e = {}
    for kind, (rp, op) in bufs.items():
        def e2e_step():
            ok = L.RL_interface(rp, nx, ny, nz, op, None, w["background"], False, False, n_iters,
                                0, 0, 0, 0.0, False, False)
            if ok != 1:
                raise RuntimeError(L.cdx_last_error().decode())
        e2e_step()
        if pg:
            pg.barrier()
        t0 = time.perf_counter()
        for _ in range(steps):
            e2e_step()
        e2e[kind] = (time.perf_counter() - t0) / steps
    finite = bool(torch.isfinite(d_out).all().item())
    launches = int(L.cdx_last_launch_count())
    cdx.rl_cleanup()
    td.cleanup()
    hbm, _ = peaks()
    achieved = ALG_BYTES_PER_VOXEL_ITER * vox / (iter_ms * 1e-3) / 1e9
    traffic = None
    tfile = ROOT / "profiles" / "traffic_rl_iteration_stage_scan.json"
    if tfile.exists():
        traffic = json.loads(tfile.read_text()).get("dram_bytes_per_iteration")
    return {"workload": w["name"], "decon_grid_zyx": [gz, gy, gx], "iterations": n_iters,
            "value": vox * n_iters / (ms * 1e-3), "ms_per_step": ms, "iteration_ms": iter_ms,
            "iteration_ms_profiled": it_ms.value / max(it_n.value, 1), "prepost_ms": prepost,
            "e2e": {"value": vox * n_iters / e2e["pinned"], "host_buffers": "pinned",
                    "h2d_bytes_per_step": int(raw.nbytes), "d2h_bytes_per_step": int(p_out.nbytes),
                    "pageable": {"value": vox * n_iters / e2e["pageable"],
                                 "ms_per_step": 1e3 * e2e["pageable"],
                                 "host_buffers": "pageable numpy arrays"}},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "traffic": traffic,
                         "kernel": "one RL iteration (9 fused passes and the lambda kernel)",
                         "passes": passes},
            "launches_per_step": launches, "output_finite": finite}


def measure_grid3(cdx, torch, dev, steps):
    """128x512x1024, 20 iterations, both forms (device-resident)."""
    from cudadecon_gb300 import synth
    L = cdx.lib()
    shape = GRID3["shape"]
    nz, ny, nx = shape
    td = tempfile.TemporaryDirectory()
    tab = synth.gaussian_otf_table(129, 64, 1.5, 4.0)
    p = Path(td.name) / "otf.tif"
    synth.write_otf(p, tab)
    cdx.rl_init(shape, p, dr=0.1, dz=0.2, dr_psf=0.1, dz_psf=0.2)
    raw = synth.bead_stack_gpu(shape, n_beads=4000, psf_sigma_xy=1.5, psf_sigma_z=4.0,
                               seed=GRID3["seed"])
    out = torch.empty(shape, dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    sp = ctypes.c_void_p(stream.cuda_stream)
    n = GRID3["n_iters"]
    res = {}
    for form, code in (("plain", 0), ("mixed", 1)):
        L.cdx_set_dft_form(code)

        def step(iters=n):
            ok = L.cdx_RL_device(ctypes.c_void_p(raw.data_ptr()), nx, ny, nz,
                                 ctypes.c_void_p(out.data_ptr()), None, 100.0, False, False,
                                 iters, 0, 0, 0, 0.0, False, False, sp)
            if ok != 1:
                raise RuntimeError(L.cdx_last_error().decode())

        with torch.cuda.stream(stream):
            step()
        ms = events_ms(torch, stream, step, steps)
        pre = events_ms(torch, stream, lambda: step(0), steps)
        res[form] = {"value": nz * ny * nx * n / (ms * 1e-3), "ms_per_step": ms,
                     "iteration_ms": (ms - pre) / n, "tc_status_ok": bool(L.cdx_tc_status())}
    L.cdx_set_dft_form(0)
    cdx.rl_cleanup()
    td.cleanup()
    res["mixed_over_plain"] = res["mixed"]["value"] / res["plain"]["value"]
    res["workload"] = f"{nz}x{ny}x{nx}, {n} RL it, Gaussian OTF"
    return res


def measure_timelapse(cdx, torch, dev, steps):
    """8 timepoints x 2 channels of 256x1024x1024 u16: camcor, deskew, 20
    iterations, rotate, one OTF per channel (RL_interface_init per channel and
    step, as a caller switching channels does).  Device-resident raw stacks."""
    from cudadecon_gb300 import synth
    L = cdx.lib()
    w = LAPSE
    nz, ny, nx = w["shape"]
    td = tempfile.TemporaryDirectory()
    otfs = []
    for c, (sxy, sz) in enumerate(((1.3, 3.0), (1.5, 3.4))):
        p = Path(td.name) / f"otf{c}.tif"
        synth.write_otf(p, synth.gaussian_otf_table(129, 64, sxy, sz))
        otfs.append(p)
    gen = torch.Generator(device=dev)
    gen.manual_seed(w["seed"])
    raws = []
    for _ in range(w["timepoints"] * w["channels"]):
        lam = 100.0 + 3000.0 * (torch.rand(w["shape"], generator=gen, device=dev) < 2e-4).float()
        raws.append(torch.poisson(lam, generator=gen).clamp_(0, 65535).to(torch.int32)
                    .to(torch.uint16))
        del lam
    cam = torch.from_numpy(synth.camcor_params(ny, nx, seed=w["seed"])).to(dev)
    cc = torch.empty(w["shape"], dtype=torch.uint16, device=dev)
    kw = dict(dr=w["dr"], dz=w["dz"], dr_psf=w["dr"], dz_psf=0.2, deskew_angle=w["angle"],
              rotation_angle=w["angle"])
    stream = torch.cuda.Stream(device=dev)
    sp = ctypes.c_void_p(stream.cuda_stream)
    state = {}

    def step():
        for c in range(w["channels"]):
            cdx.rl_init(w["shape"], otfs[c], **kw)
            if "out" not in state:
                state["out"] = torch.empty(cdx.output_shape(), dtype=torch.float32, device=dev)
                state["grid"] = cdx.decon_grid()
            out = state["out"]
            for t in range(w["timepoints"]):
                r = raws[t * w["channels"] + c]
                if L.cdx_camcor_device(ctypes.c_void_p(r.data_ptr()), nx, ny, nz,
                                       ctypes.c_void_p(cam.data_ptr()),
                                       ctypes.c_void_p(cc.data_ptr()), sp) != 1:
                    raise RuntimeError(L.cdx_last_error().decode())
                if L.cdx_RL_device(ctypes.c_void_p(cc.data_ptr()), nx, ny, nz,
                                   ctypes.c_void_p(out.data_ptr()), None, 100.0, False, False,
                                   w["n_iters"], 0, 0, 0, 0.0, False, False, sp) != 1:
                    raise RuntimeError(L.cdx_last_error().decode())

    step()
    stream.synchronize()
    ms = events_ms(torch, stream, step, steps)
    gz, gy, gx = state["grid"]
    vox = gz * gy * gx * w["timepoints"] * w["channels"]
    finite = bool(torch.isfinite(state["out"]).all().item())
    cdx.rl_cleanup()
    td.cleanup()
    hbm, _ = peaks()
    v = vox * w["n_iters"] / (ms * 1e-3)
    return {"workload": f"{w['timepoints']} timepoints x {w['channels']} channels of "
                        f"{nz}x{ny}x{nx} u16, camcor, deskew {w['angle']} deg -> {gz}x{gy}x{gx}, "
                        f"{w['n_iters']} RL it, rotate, 2 OTFs",
            "value": v, "unit": "voxel-iter/s", "ms_per_step": ms,
            "roofline_frac": ALG_BYTES_PER_VOXEL_ITER * v / 1e9 / hbm, "output_finite": finite}


def measure_batch_per_stack(cdx, torch, dev, stacks):
    """The batch's stacks one cdx_RL_device call at a time (RL_interface_init
    per stack, no CUDA graph): the same kernels as the batch call, launched
    individually, for profilers that list launches one by one."""
    from cudadecon_gb300 import synth
    L = cdx.lib()
    stream = torch.cuda.Stream(device=dev)
    sp = ctypes.c_void_p(stream.cuda_stream)
    iters = BATCH["iterations"]
    vox = 0
    td = tempfile.TemporaryDirectory()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i, d in enumerate(stacks):
        p = Path(td.name) / f"otf{i}.tif"
        synth.write_otf(p, d["otf"])
        nz, ny, nx = d["raw"].shape
        cdx.rl_init((nz, ny, nx), p, dr=d["dr"], dz=d["dz"], dr_psf=d["dr_psf"], dz_psf=d["dz_psf"])
        out = torch.empty(cdx.output_shape(), dtype=torch.float32, device=dev)
        if L.cdx_RL_device(ctypes.c_void_p(d["raw"].data_ptr()), nx, ny, nz,
                           ctypes.c_void_p(out.data_ptr()), None, d["background"], False, False,
                           iters, 0, 0, 0, 0.0, False, False, sp) != 1:
            raise RuntimeError(L.cdx_last_error().decode())
        vox += int(np.prod(out.shape))
    torch.cuda.synchronize()
    s = time.perf_counter() - t0
    cdx.rl_cleanup()
    td.cleanup()
    return {"workload": BATCH_NAME + " (one call per stack, no graph)", "value": vox * iters / s,
            "unit": "voxel-iter/s", "seconds": s}


def measure_one_stack(cdx, torch, dev, zyx, steps, warmup):
    """One synthetic stack of shape zyx (u16 beads on a Poisson background,
    the batch's Gaussian OTF), 10 RL iterations per cdx_RL_device call:
    voxel-iter/s and the per-pass times of one iteration (for profiling and
    for tuning one length's plans)."""
    from cudadecon_gb300 import synth
    L = cdx.lib()
    nz, ny, nx = zyx
    iters = BATCH["iterations"]
    gen = torch.Generator(device=dev)
    gen.manual_seed(nz * 1000003 + ny * 1009 + nx)
    lam = 100.0 + 3000.0 * (torch.rand(zyx, generator=gen, device=dev) < 2e-4).float()
    raw = torch.poisson(lam, generator=gen).clamp_(0, 65535).to(torch.int32).to(torch.uint16)
    td = tempfile.TemporaryDirectory()
    p = Path(td.name) / "otf.tif"
    synth.write_otf(p, synth.gaussian_otf_table(129, 64, 1.5, 4.0))
    cdx.rl_init(zyx, p, dr=0.104, dz=0.3, dr_psf=0.104, dz_psf=0.3)
    gz, gy, gx = cdx.decon_grid()
    out = torch.empty(cdx.output_shape(), dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    sp = ctypes.c_void_p(stream.cuda_stream)

    def step():
        if L.cdx_RL_device(ctypes.c_void_p(raw.data_ptr()), nx, ny, nz,
                           ctypes.c_void_p(out.data_ptr()), None, 100.0, False, False, iters,
                           0, 0, 0, 0.0, False, False, sp) != 1:
            raise RuntimeError(L.cdx_last_error().decode())

    with torch.cuda.stream(stream):
        for _ in range(warmup):
            step()
    stream.synchronize()
    ms = events_ms(torch, stream, step, steps)
    L.cdx_profile_enable(1)
    with torch.cuda.stream(stream):
        step()
    stream.synchronize()
    pm = (ctypes.c_double * 9)()
    pn = (ctypes.c_longlong * 9)()
    it_ms = ctypes.c_double(0)
    it_n = ctypes.c_longlong(0)
    L.cdx_profile_read(pm, pn, 9, ctypes.byref(it_ms), ctypes.byref(it_n))
    L.cdx_profile_enable(0)
    passes = {L.cdx_profile_pass_name(i).decode(): round(pm[i] / max(pn[i], 1), 5)
              for i in range(9)}
    vox = gz * gy * gx
    cdx.rl_cleanup()
    td.cleanup()
    return {"workload": f"one stack {nz}x{ny}x{nx} u16, {iters} RL it",
            "decon_grid_zyx": [gz, gy, gx], "value": vox * iters / (ms * 1e-3),
            "unit": "voxel-iter/s", "ms_per_step": ms, "pass_ms": passes,
            "output_finite": bool(torch.isfinite(out).all().item())}


def run_only(args):
    """One workload alone (for profiling): prints its JSON result."""
    import torch
    import cudadecon_gb300 as cdx
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    if args.only == "stage_scan":
        r = measure_stage_scan(cdx, torch, dev, args.steps, None)
    elif args.only == "grid3":
        r = measure_grid3(cdx, torch, dev, args.steps)
    elif args.only == "timelapse":
        r = measure_timelapse(cdx, torch, dev, args.steps)
    elif args.only == "stack":
        zyx = tuple(int(v) for v in args.zyx.split(","))
        r = measure_one_stack(cdx, torch, dev, zyx, args.steps, args.warmup)
    else:
        r = measure_batch_per_stack(cdx, torch, dev, batch_inputs(dev))
    print(json.dumps({"only": args.only, **r}), flush=True)
    return 0


def run_gb300(args):
    import torch
    world, rank, local, pg = dist_setup(args)
    torch.cuda.set_device(local)
    import cudadecon_gb300 as cdx
    L = cdx.lib()
    if args.batch_streams:
        d_s, h_s = (int(v) for v in args.batch_streams.split(","))
        cdx.batch_streams(device=d_s, host=h_s)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    stacks = batch_inputs(dev)
    # ---- headline: the batch, plain FP32 form
    clk = ClockSampler(local)
    clk.start()
    # warm-up (graph capture, plans) before the barrier
    measure_batch(cdx, torch, dev, stream, stacks, 1, args.warmup, 0)
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    t_wall0 = time.time()
    ms, vox_iters, launches, finite = measure_batch(cdx, torch, dev, stream, stacks, args.steps,
                                                    0, 0)
    t_wall1 = time.time()
    clocks = clk.stop(t_wall0, t_wall1)
    ms = max_over_ranks(ms, pg, dev)
    value = world * vox_iters / (ms * 1e-3)
    # ---- the mixed-precision form on the same batch
    ms_mixed, _, launches_mixed, finite_mixed = measure_batch(cdx, torch, dev, stream, stacks,
                                                              args.steps, args.warmup, 1)
    ms_mixed = max_over_ranks(ms_mixed, pg, dev)
    value_mixed = world * vox_iters / (ms_mixed * 1e-3)
    # ---- e2e (host buffers)
    e2e_s, h2d, d2h = measure_batch_e2e(cdx, torch, stacks, max(1, min(args.steps, 5)))
    e2e_s = max_over_ranks(e2e_s, pg, dev)
    L.cdx_batch_release()
    # ---- per-pass device times over the batch's stacks (untimed region)
    passes, top, vox_grid = measure_batch_passes(cdx, torch, dev, stacks)
    del stacks
    torch.cuda.empty_cache()
    hbm, peak_kind = peaks()
    achieved = ALG_BYTES_PER_VOXEL_ITER * vox_iters / (ms * 1e-3) / 1e9
    top_gbs = passes[top]["gbs"]
    traffic = None
    tfile = ROOT / "profiles" / "traffic_batch_x_ratio.json"
    if top == "x_ratio_fwd" and tfile.exists():
        traffic = json.loads(tfile.read_text()).get("dram_bytes_per_iteration")
    secondary = {}
    if not args.no_secondary:
        secondary["stage_scan"] = measure_stage_scan(cdx, torch, dev, args.steps, pg)
        secondary["grid_128x512x1024"] = measure_grid3(cdx, torch, dev, max(3, args.steps // 4))
        torch.cuda.empty_cache()
        if not args.no_timelapse:
            secondary["timelapse"] = measure_timelapse(cdx, torch, dev, 2)
            torch.cuda.empty_cache()
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline_leg()
    if rank == 0:
        line = {
            "metric": "RL voxel-iterations/s", "value": value, "unit": "voxel-iter/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded Poisson background "
                                                         "+ sparse beads, generated on the GPU)",
            "config": {"workload": BATCH_NAME, "stacks": BATCH["stacks"],
                       "decon_voxels": vox_iters // BATCH["iterations"],
                       "iterations": BATCH["iterations"], "form": "plain FP32",
                       "parallelism": f"replicas x{world}",
                       "graph_streams": dict(zip(("device", "host"), cdx.batch_streams())),
                       "l2_policy": "working set ~10 GB > 129 MB L2 (no flush needed)"},
            "forms": {"plain": {"value": value, "ms_per_step": ms},
                      "mixed": {"value": value_mixed, "ms_per_step": ms_mixed,
                                "what": "x-pass DFT stages of rows with a tensor-core plan "
                                        "(256, 512, 756, 1024) as tcgen05 MMAs in split TF32"},
                      "mixed_over_plain": value_mixed / value},
            "e2e": {"value": world * vox_iters / e2e_s, "unit": "voxel-iter/s",
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "host_buffers": "pinned", "api": "cdx_RL_batch_host"},
            "roofline": {"bound": "hbm", "achieved": top_gbs, "peak": hbm, "unit": "GB/s",
                         "frac": top_gbs / hbm, "traffic": traffic,
                         "kernel": f"{top}: the dominant pass, one launch per stack summed "
                                   "over the 64 stacks (per-pass CUDA events on the launch "
                                   "stream, one profiled call per stack outside the timed "
                                   "region)",
                         "alg_bytes_per_voxel": PASS_BYTES[list(passes).index(top)],
                         "traffic_per": "one launch per stack, all 64 stacks",
                         "passes": passes,
                         "whole_call": {"achieved": achieved, "frac": achieved / hbm,
                                        "alg_bytes_per_voxel_iter": ALG_BYTES_PER_VOXEL_ITER,
                                        "nominal_gbs": NOMINAL_HBM_GBS,
                                        "frac_of_nominal": achieved / NOMINAL_HBM_GBS},
                         "peak_source": f"{peak_kind} hbm_gbs"},
            "cpu_baseline": cpu,
            "clocks": clocks,
            "gpu_launches": launches * args.steps,
            "output_finite": finite and finite_mixed,
            "secondary": secondary,
        }
        print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true",
                    help="only the batched headline workload")
    ap.add_argument("--no-timelapse", action="store_true",
                    help="skip the 16-stack time-lapse secondary workload")
    ap.add_argument("--only", choices=["stage_scan", "grid3", "timelapse", "batch_per_stack",
                                       "stack"],
                    help="run one workload alone and print its result (for profiling)")
    ap.add_argument("--zyx", default="100,256,600",
                    help="stack shape z,y,x of --only stack")
    ap.add_argument("--batch-streams", default=None,
                    help="DEVICE,HOST graph streams of the batch (cdx_batch_set_streams; "
                         "default: the library's, 2,2)")
    args = ap.parse_args()
    if args.only:
        return run_only(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
