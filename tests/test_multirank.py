"""
The multi-GPU contract of bench.py on the CPU (gloo, world size 2): the
structures are independent, so N ranks run N replicas with no data-path
collective; the only collectives are the timing barrier and the max over
ranks of the timed region.  ``--impl reference`` under torchrun prints one
line from rank 0 and the other ranks exit 0 without work.
"""

from __future__ import annotations

import json
import os
import socket
import subprocess
import sys

import torch.multiprocessing as mp

from conftest import REPO


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, str(REPO))
    import bench
    import torch.distributed as dist

    w, r, _ = bench.dist_setup(world)
    bench.barrier(w)
    out[rank] = bench.max_over_ranks(float(rank + 1) * 0.25, w)
    dist.destroy_process_group()


def test_max_over_ranks_and_barrier_gloo():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        assert dict(out) == {0: 0.5, 1: 0.5}


def test_reference_arm_under_torchrun_prints_one_line():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py",
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0",
           "--cpu-seconds", "0.2", "--nstruct", "4"]
    res = subprocess.run(cmd, cwd=REPO, capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [json.loads(l) for l in res.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["value"] > 0 and line["e2e"]["h2d_bytes_per_step"] == 0
