"""Host logic of bench.py's multi-process form, on CPU: two ranks over gloo.

A single solve does not shard (one IEKS loop per problem), so `bench.py
--gpus N` runs N independent replicas: the job's time is the slowest rank's,
and the reference arm runs on rank 0 alone while the other ranks exit 0
without work.  These tests run both pieces with world_size 2 and no GPU.
"""

import json
import os
import socket
import subprocess
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, values, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        got = bench.max_over_ranks(values[rank], world, torch.device("cpu"))
    finally:
        dist.destroy_process_group()
    with open(os.path.join(out_dir, "rank%d.txt" % rank), "w") as f:
        f.write(repr(got))


def test_max_over_ranks_two_ranks(tmp_path):
    values = [3.25, 7.5]
    mp.start_processes(_rank_main, args=(2, _free_port(), values, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    got = [float(open(tmp_path / ("rank%d.txt" % r)).read()) for r in range(2)]
    assert got == [7.5, 7.5]


def test_max_over_ranks_one_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench

    assert not dist.is_initialized()
    assert bench.max_over_ranks(2.5, 1, torch.device("cpu")) == 2.5


@pytest.mark.timeout(600)
def test_reference_arm_prints_one_line_from_rank_zero():
    """`torchrun --nproc-per-node 2 bench.py --impl reference`: rank 0 times
    the oracle on a bounded sample and prints one JSON line; rank 1 exits 0."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(_free_port()), os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0", "--workload", "fhn_q3_N16384"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    out = json.loads(lines[0])
    assert out["impl"] == "reference" and out["n_gpus"] == 2
    assert out["value"] > 0 and out["unit"] == "IVP*steps/s"
    assert out["cpu_baseline"]["kind"] == "port" and out["cpu_baseline"]["cores"] >= 1
    assert out["e2e"] == {"value": out["value"], "unit": "IVP*steps/s", "h2d_bytes_per_step": 0,
                          "d2h_bytes_per_step": 0}
