"""One batch split over two ranks (pof.batch.solve_batch_sharded) with
libpof doing the solves: two processes over gloo, both on cuda:0.  The
ranks' kernels never wait on one another: each solves its share, then one
all-gather of the per-problem results runs on the host.  Both ranks end with
the whole batch in the original order; each rank's rows are bit for bit a
single-process solve_batch of that rank's share, and every row agrees with
the single-process solve of the whole batch to 1e-8 (the segmented scans
may pair a problem's chunks differently when its neighbours change)."""

import os
import socket
import sys

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "parallel-in-time-ode-filters_gb300")

pytestmark = pytest.mark.gpu

WHOLE_BATCH_TOL = 1e-8


def _problems():
    rng = np.random.default_rng(11)
    out = []
    for b, n in enumerate(rng.integers(60, 700, size=9)):
        mu = float(rng.uniform(0.8, 1.2))
        out.append(("vanderpol", (mu,), [2.0, 0.1 * b], np.linspace(0.0, 6.3, int(n))))
    return out


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    for p in (ROOT, PKG):
        sys.path.insert(0, p)
    from pof import batch as pbatch

    torch.cuda.set_device(0)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        res = pbatch.solve_batch_sharded(_problems(), 3, rank, world, maxiters=500)
    finally:
        dist.destroy_process_group()
    torch.save({"mean": res.mean, "chol": res.chol, "offsets": torch.as_tensor(res.offsets),
                "iterations": res.info["iterations"], "status": res.info["status"]},
               os.path.join(out_dir, "rank%d.pt" % rank))


def test_sharded_batch_on_the_gpu_matches_single_process_solves(tmp_path):
    for p in (ROOT, PKG):
        if p not in sys.path:
            sys.path.insert(0, p)
    from pof import batch as pbatch

    mp.start_processes(_rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    probs = _problems()
    got = [torch.load(tmp_path / ("rank%d.pt" % r)) for r in range(2)]
    for r in range(1, 2):  # every rank holds the same gathered batch
        for k in ("mean", "chol", "offsets", "iterations", "status"):
            assert torch.equal(got[r][k], got[0][k]), k
    g = got[0]
    off = g["offsets"].numpy()

    parts = pbatch.shard([len(p[3]) - 1 for p in probs], 2)
    assert all(len(p) > 0 for p in parts)
    for part in parts:  # a rank's rows: bit for bit the same solve in one process
        sub = pbatch.solve_batch([probs[b] for b in part], order=3, maxiters=500)
        for i, b in enumerate(part):
            (m, L), info = sub.problem(i)
            s, e = int(off[b]), int(off[b + 1])
            assert torch.equal(g["mean"][s:e], m.cpu()) and torch.equal(g["chol"][s:e], L.cpu()), b
            assert int(g["iterations"][b]) == int(info["iterations"]) and int(g["status"][b]) == 0

    whole = pbatch.solve_batch(probs, order=3, maxiters=500)
    err = float((whole.mean.cpu() - g["mean"]).abs().max())
    print("sharded vs whole-batch solve: max |mean diff| %.3e (tolerance %.0e)" % (err, WHOLE_BATCH_TOL))
    assert err <= WHOLE_BATCH_TOL
    assert np.array_equal(whole.offsets, off)
