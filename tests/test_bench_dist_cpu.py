"""Multi-rank paths of bench.py on CPU (world size 2, gloo).

The stacks shard as independent replicas (one stack per GPU, no data
exchange), so the only cross-rank operations are the barrier around the
timed region and the max-over-ranks of the step time; these tests run them
as gloo ranks on the host.
"""

import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dist.barrier()
        # each rank reports a different step time; all must agree on the slowest
        q.put((rank, bench.max_over_ranks(1.5 + rank, dist)))
        # without a group the value passes through
        q.put((rank + 10, bench.max_over_ranks(7.0, None)))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo_world2():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = dict(q.get(timeout=5) for _ in range(4))
    assert got[0] == 2.5 and got[1] == 2.5
    assert got[10] == 7.0 and got[11] == 7.0


def test_reference_arm_torchrun_world2():
    """`bench.py --impl reference` under torchrun with two ranks: rank 0 times
    the CPU restatement and prints the one JSON line, rank 1 exits cleanly."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["n_gpus"] == 2
    assert d["value"] > 0 and d["unit"] == "voxel-iter/s"
    assert d["cpu_baseline"]["kind"] == "port"
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
