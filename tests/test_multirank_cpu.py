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


# ---------------------------------------------------------------------------
# One fixed batch split across ranks (pof.batch.solve_batch_sharded)
# ---------------------------------------------------------------------------

def _oracle_batch_solver(problems, order, maxiters=50, **kw):
    """A CPU stand-in for pof.batch.solve_batch with its BatchResult: the
    oracle's solve of each problem on its own (a problem's result depends on
    its own inputs only, as in libpof's batched solve)."""
    import numpy as np

    from oracle import ivp as oivp, solver as osolver
    from pof.batch import BatchResult

    means, chols, its, objs = [], [], [], []
    for nm, p, y0, ts in problems:
        ivp = oivp.logistic(r=p[0], y0=list(y0), tmax=float(ts[-1]))
        (m, L), info = osolver.solve(ivp, ts, order, init="constant", maxiters=maxiters)
        means.append(torch.as_tensor(m))
        chols.append(torch.as_tensor(L))
        its.append(info["iterations"])
        objs.append(info["obj"])
    offsets = np.concatenate([[0], np.cumsum([m.shape[0] for m in means])]).astype(np.int64)
    info = {"iterations": torch.tensor(its), "obj": torch.tensor(objs, dtype=torch.float64), "calibrated": True}
    return BatchResult(torch.cat(means), torch.cat(chols), offsets, info)


def _sharded_problems():
    import numpy as np

    rng = np.random.default_rng(3)
    return [("logistic", (float(rng.uniform(2.0, 4.0)),), [0.01], np.linspace(0.0, 10.0, int(n)))
            for n in rng.integers(8, 40, size=7)]


def _shard_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    for p in (ROOT, os.path.join(ROOT, "parallel-in-time-ode-filters_gb300")):
        sys.path.insert(0, p)
    from pof import batch as pbatch

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        res = pbatch.solve_batch_sharded(_sharded_problems(), 2, rank, world, solver=_oracle_batch_solver)
    finally:
        dist.destroy_process_group()
    torch.save({"mean": res.mean, "chol": res.chol, "offsets": torch.as_tensor(res.offsets),
                "iterations": res.info["iterations"],
                "obj": res.info["obj"]}, os.path.join(out_dir, "shard%d.pt" % rank))


def test_shard_partition_balances_steps():
    import numpy as np

    for p in (ROOT, os.path.join(ROOT, "parallel-in-time-ode-filters_gb300")):
        sys.path.insert(0, p)
    from pof import batch as pbatch

    ns = np.random.default_rng(0).integers(255, 8192, size=4096)
    for world in (1, 2, 3, 8):
        parts = pbatch.shard(ns, world)
        assert sorted(np.concatenate(parts).tolist()) == list(range(4096))  # each problem exactly once
        loads = [int(ns[p].sum()) for p in parts]
        assert max(loads) - min(loads) <= ns.max()
        assert all((np.diff(p) > 0).all() for p in parts)
        assert all((a == b).all() for a, b in zip(parts, pbatch.shard(ns, world)))  # deterministic


@pytest.mark.timeout(600)
def test_sharded_batch_equals_one_rank(tmp_path):
    """Two gloo ranks each solve their share of one batch; after the
    all-gather both hold the whole batch, equal bit for bit to one rank
    solving all of it."""
    for p in (ROOT, os.path.join(ROOT, "parallel-in-time-ode-filters_gb300")):
        sys.path.insert(0, p)
    mp.start_processes(_shard_main, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    one = _oracle_batch_solver(_sharded_problems(), 2)
    for r in range(2):
        got = torch.load(tmp_path / ("shard%d.pt" % r))
        assert torch.equal(got["mean"], one.mean) and torch.equal(got["chol"], one.chol)
        assert got["offsets"].tolist() == list(one.offsets)
        assert torch.equal(got["iterations"], one.info["iterations"])
        assert torch.equal(got["obj"], one.info["obj"])
