"""Batched IEKS solves: many IVPs with built-in fields in one libpof call.

No counterpart in the reference, whose ``pof.solver.solve`` takes one IVP
(pof/solver.py:11-73).  ``solve_batch`` runs that solve for B problems at
once -- each with its own field (of one dimension d), parameters, y0 and
uniform grid -- through ``pof_ieks_solve_batch``: per problem the same
set-up (convenience.py:13-45), the same initial trajectory and the same
device-resident IEKS loop as ``pof.solver.solve``.  Each problem's result
depends only on its own inputs, never on the rest of the batch.
"""

import math
from typing import Any, NamedTuple

import numpy as np
import torch

from . import _lib
from .transitions import IWP, preconditioned_discretize
from .utils import FORWARD_AD_LOCK, default_device

# Built-in fields with explicit parameters p (4 slots), the expressions of
# pof/ivp.py: used for the Taylor-mode initial states of a whole batch at
# once (torch.func.vmap over problems).
_NPARAMS = {"logistic": 1, "lotkavolterra": 4, "vanderpol": 1, "fitzhughnagumo": 4, "fhn_classic": 3,
            "rober": 3, "rigid_body": 3, "seir": 4, "threebody": 1, "henonheiles": 1}
_DIM = {"logistic": 1, "lotkavolterra": 2, "vanderpol": 2, "fitzhughnagumo": 2, "fhn_classic": 2,
        "rober": 3, "rigid_body": 3, "seir": 4, "threebody": 4, "henonheiles": 4}


def _field(name):
    if name == "logistic":
        return lambda y, p: p[0] * y * (1 - y)
    if name == "lotkavolterra":
        return lambda Y, p: torch.stack([p[0] * Y[0] - p[1] * Y[0] * Y[1], -p[2] * Y[1] + p[3] * Y[0] * Y[1]])
    if name == "vanderpol":
        return lambda Y, p: torch.stack([Y[1], p[0] * ((1.0 - Y[0] ** 2) * Y[1] - Y[0])])
    if name == "fitzhughnagumo":
        return lambda Y, p: torch.stack([Y[0] - (Y[0] ** 3) / 3 - Y[1] + p[3], p[2] * (Y[0] + p[0] - p[1] * Y[1])])
    if name == "fhn_classic":
        return lambda Y, p: torch.stack([p[2] * (Y[0] - Y[0] ** 3 / 3 + Y[1]), -(Y[0] - p[0] + p[1] * Y[1]) / p[2]])
    if name == "rober":
        return lambda Y, p: torch.stack([-p[0] * Y[0] + p[2] * Y[1] * Y[2],
                                         p[0] * Y[0] - p[1] * Y[1] ** 2 - p[2] * Y[1] * Y[2], p[1] * Y[1] ** 2])
    if name == "rigid_body":
        return lambda y, p: torch.stack([p[0] * y[1] * y[2], p[1] * y[0] * y[2], p[2] * y[0] * y[1]])
    if name == "seir":
        return lambda y, p: torch.stack([-p[1] * y[0] * y[2] / p[3], p[1] * y[0] * y[2] / p[3] - p[0] * y[1],
                                         p[0] * y[1] - p[2] * y[2], p[2] * y[2]])
    if name == "henonheiles":
        return lambda y, p: torch.stack([y[2], y[3], -y[0] - 2 * p[0] * y[0] * y[1],
                                         -y[1] - p[0] * (y[0] ** 2 - y[1] ** 2)])
    if name == "threebody":
        def f(y, p):
            mu = p[0]
            mp = 1.0 - mu
            D1 = torch.sqrt((y[0] + mu) ** 2 + y[1] ** 2) ** 3.0
            D2 = torch.sqrt((y[0] - mp) ** 2 + y[1] ** 2) ** 3.0
            du0p = y[0] + 2 * y[3] - mp * (y[0] + mu) / D1 - mu * (y[0] - mp) / D2
            du1p = y[1] - 2 * y[2] - mp * y[1] / D1 - mu * y[1] / D2
            return torch.stack([y[2], y[3], du0p, du1p])
        return f
    raise ValueError("no built-in field %r" % (name,))


def _taylor(g, y0, p, q):
    """(q+1, d) derivatives y^(k)(0) of y' = g(y, p), y(0) = y0 (nested jvp,
    as pof.initialization.taylor_derivatives)."""
    derivs = [y0]
    for k in range(1, q + 1):
        coeffs = [dj / math.factorial(j) for j, dj in enumerate(derivs)]

        def traj(t, coeffs=coeffs):
            y = coeffs[0] + 0 * t
            for j in range(1, len(coeffs)):
                y = y + coeffs[j] * t**j
            return g(y, p)

        h = traj
        for _ in range(k - 1):
            h = (lambda hh: (lambda t: torch.func.jvp(hh, (t,), (torch.ones_like(t),))[1]))(h)
        derivs.append(h(torch.zeros((), dtype=y0.dtype, device=y0.device)))
    return torch.stack(derivs)


def _nordsieck(q, hs):
    """(B, q+1) diagonals of P(h) and P(h)^-1 (pof/transitions.py:53-61), each
    entry computed as in pof.transitions._nordsieck_1d_np."""
    powers = np.arange(q, -1, -1)
    scales = np.array([math.factorial(int(p)) for p in powers], dtype=np.float64)
    powers = powers + 0.5
    ah = np.abs(np.asarray(hs, dtype=np.float64))[:, None]
    return (ah ** powers) / scales, (ah ** (-powers)) * scales


class BatchResult(NamedTuple):
    """Concatenated results of a batch: problem b owns rows
    offsets[b]:offsets[b+1] of mean (G, d) and chol (G, d, D)."""

    mean: Any
    chol: Any
    offsets: Any
    info: Any

    def problem(self, b):
        s, e = int(self.offsets[b]), int(self.offsets[b + 1])
        info = {k: v[b] for k, v in self.info.items() if k != "calibrated"}
        info["calibrated"] = self.info["calibrated"]
        return (self.mean[s:e], self.chol[s:e]), info


def prepare_rows(problems, order):
    """Per-problem set-up on the host (CPU tensors): x0 (B, D) (Taylor mode,
    times P^-1), the constant-init row (B, D) [y0, f(y0), 0, ...] times
    P^-1, steps, step sizes, field ids, parameters (B, 4), P[0, 0]."""
    B = len(problems)
    names = [p[0] for p in problems]
    d = _DIM[names[0]]
    if any(_DIM[nm] != d for nm in names):
        raise ValueError("every problem of a batch needs the same dimension d")
    q = int(order)
    D = d * (q + 1)
    n_steps = np.array([len(p[3]) - 1 for p in problems], dtype=np.int64)
    if (n_steps < 1).any():
        raise ValueError("every problem needs at least two grid points")
    hs = np.array([float(p[3][1]) - float(p[3][0]) for p in problems], dtype=np.float64)
    fields = np.array([_lib.FIELDS[nm] for nm in names], dtype=np.int32)
    params = torch.zeros((B, 4), dtype=torch.float64)
    for b, p in enumerate(problems):
        pv = tuple(float(x) for x in p[1])
        if len(pv) != _NPARAMS[p[0]]:
            raise ValueError("field %s takes %d parameters" % (p[0], _NPARAMS[p[0]]))
        params[b, : len(pv)] = torch.tensor(pv, dtype=torch.float64)
    y0 = torch.stack([torch.as_tensor(p[2], dtype=torch.float64).reshape(d) for p in problems])
    # Taylor-mode x0 and the constant-init row [y0, f(y0), 0, ...] per field group
    derivs = torch.zeros((B, q + 1, d), dtype=torch.float64)
    for nm in sorted(set(names)):
        idx = torch.tensor([b for b in range(B) if names[b] == nm], dtype=torch.long)
        g = _field(nm)
        with FORWARD_AD_LOCK:
            derivs[idx] = torch.func.vmap(lambda yy, pp: _taylor(g, yy, pp, q))(y0[idx], params[idx])
    P, PI = _nordsieck(q, hs)  # (B, q+1)
    PI_t = torch.as_tensor(PI, dtype=torch.float64)
    x0m = (derivs.transpose(1, 2) * PI_t[:, None, :]).reshape(B, D)  # dimension-major, times P^-1
    row = torch.zeros((B, d, q + 1), dtype=torch.float64)
    row[:, :, 0] = y0
    row[:, :, 1] = derivs[:, 1, :]
    row = (row * PI_t[:, None, :]).reshape(B, D)
    return {"B": B, "D": D, "d": d, "q": q, "n_steps": n_steps, "fields": fields, "h": hs, "params": params,
            "x0m": x0m, "row": row, "p0": torch.as_tensor(P[:, 0])}


def prepare_batch(problems, order, device=None, init="constant"):
    """Device inputs of pof_ieks_solve_batch for problems = [(field name,
    params, y0, ts), ...] (uniform grids ts; the step is ts[1] - ts[0] as in
    pof.convenience.set_up_solver).  Returns a dict of tensors and host
    arrays."""
    if init != "constant":
        raise NotImplementedError("solve_batch supports init='constant'")
    dev = device or default_device()
    r = prepare_rows(problems, order)
    B, D, d, q, n_steps = r["B"], r["D"], r["d"], r["q"], r["n_steps"]
    counts = torch.as_tensor(n_steps + 1)
    means0 = torch.repeat_interleave(r["row"], counts, dim=0)
    iwp = IWP(num_derivatives=q, wiener_process_dimension=d)
    F, QL = preconditioned_discretize(iwp, device=dev)
    offsets = np.concatenate([[0], np.cumsum(n_steps + 1)]).astype(np.int64)
    return {
        "B": B, "D": D, "d": d, "q": q, "n_steps": n_steps, "fields": r["fields"], "h": r["h"],
        "params": r["params"].to(dev), "x0m": r["x0m"].to(dev).contiguous(),
        "x0L": torch.zeros((B, D, D), dtype=torch.float64, device=dev), "F": F.contiguous(),
        "QL": QL.contiguous(), "means0": means0.to(dev).contiguous(), "p0": r["p0"], "offsets": offsets,
    }


def _host(prep):
    ns = np.ascontiguousarray(prep["n_steps"], dtype=np.int64)
    fl = np.ascontiguousarray(prep["fields"], dtype=np.int32)
    hs = np.ascontiguousarray(prep["h"], dtype=np.float64)
    return ns, fl, hs


def _vp(a):
    return a.ctypes.data_as(_lib.ctypes.c_void_p)


def workspace_bytes(prep, precision="float64", C0=0, Cg=0):
    lib = _lib.lib()
    ns, _, _ = _host(prep)
    if precision == "mixed":
        wsb = lib.pof_batch_mixed_workspace_bytes(prep["B"], _vp(ns), prep["D"], prep["d"], int(C0), int(Cg))
    else:
        wsb = lib.pof_batch_workspace_bytes(_lib.POF_F64, prep["B"], _vp(ns), prep["D"], prep["d"], int(C0), int(Cg))
    if wsb == 0:
        raise _lib.PofError("the batch workspace query refused the batch (shape (%d, %d) or sizes)"
                            % (prep["D"], prep["d"]))
    return wsb


def run_batch(prep, means, chols, info, maxiters=10_000, calibrate=True, C0=0, Cg=0, workspace=None,
              precision="float64", maxiters_f32=10_000, rtol_f32=1e-5, info_f32=None, settle_f32=float("inf")):
    """pof_ieks_solve_batch (precision="float64") or
    pof_ieks_solve_batch_mixed ("mixed") on prepared inputs; means (G, D)
    holds the initial trajectories on entry and the results on return.
    Returns the workspace (reusable for the same batch)."""
    lib = _lib.lib()
    B, D, d = prep["B"], prep["D"], prep["d"]
    ns, fl, hs = _host(prep)
    wsb = workspace_bytes(prep, precision, C0, Cg)
    if workspace is None or workspace.numel() < wsb:
        workspace = _lib.workspace(wsb, means.device)
    common = (_lib.ptr(prep["params"]), _vp(hs), _lib.ptr(prep["x0m"]), _lib.ptr(prep["x0L"]), _lib.ptr(prep["F"]),
              _lib.ptr(prep["QL"]), _lib.ptr(means), _lib.ptr(chols))
    if precision == "mixed":
        rc = lib.pof_ieks_solve_batch_mixed(B, _vp(ns), D, d, _vp(fl), *common, int(maxiters_f32), float(rtol_f32),
                                            float(settle_f32),
                                            int(maxiters), int(bool(calibrate)), int(C0), int(Cg), _lib.ptr(info),
                                            _lib.ptr(info_f32), _lib.ptr(workspace), int(workspace.numel()),
                                            _lib.stream_handle())
        _lib.check(rc, "pof_ieks_solve_batch_mixed")
    elif precision == "float64":
        rc = lib.pof_ieks_solve_batch(_lib.POF_F64, B, _vp(ns), D, d, _vp(fl), *common, int(maxiters),
                                      int(bool(calibrate)), int(C0), int(Cg), _lib.ptr(info), _lib.ptr(workspace),
                                      int(workspace.numel()), _lib.stream_handle())
        _lib.check(rc, "pof_ieks_solve_batch")
    else:
        raise ValueError("precision must be 'float64' or 'mixed'")
    return workspace


class _TeamWidth:
    """Level-0 team width of the batched kernels for the calls inside the
    block (lanes per chunk: the narrow teams by default, the wide ones with
    POF_BATCH_TEAM_WIDE=1, read by libpof at each call)."""

    def __init__(self, wide):
        self.wide = wide

    def __enter__(self):
        import os

        self.old = os.environ.get("POF_BATCH_TEAM_WIDE")
        if self.wide is not None:
            os.environ["POF_BATCH_TEAM_WIDE"] = "1" if self.wide else "0"
        return self

    def __exit__(self, *a):
        import os

        if self.wide is None:
            return
        if self.old is None:
            os.environ.pop("POF_BATCH_TEAM_WIDE", None)
        else:
            os.environ["POF_BATCH_TEAM_WIDE"] = self.old


def autotune_key(prep, device=None):
    """Cache key of a batch's tuning: the GPU, the state shape (D, d) and
    the total step count to a factor of two."""
    dev = device if device is not None else prep["x0m"].device
    name = torch.cuda.get_device_name(dev) if torch.cuda.is_available() else "cpu"
    steps = int(np.asarray(prep["n_steps"]).sum())
    return "%s|D%d|d%d|steps2^%d" % (name, prep["D"], prep["d"], int(round(math.log2(max(steps, 1)))))


def _cache_path(path=None):
    import os

    if path:
        return path
    env = os.environ.get("POF_AUTOTUNE_CACHE")
    if env:
        return env
    return os.path.join(os.path.expanduser("~"), ".cache", "pof_gb300", "autotune.json")


def load_tuning(prep, path=None):
    """(C0, Cg, wide) cached for this batch's key, or None."""
    import json
    import os

    p = _cache_path(path)
    if not os.path.exists(p):
        return None
    try:
        with open(p) as f:
            entry = json.load(f).get(autotune_key(prep))
    except (OSError, ValueError):
        return None
    if not entry:
        return None
    return int(entry["C0"]), int(entry["Cg"]), bool(entry["wide"])


def store_tuning(prep, C0, Cg, wide, times=None, path=None):
    """Write (C0, Cg, wide) under this batch's key (other keys are kept)."""
    import json
    import os

    p = _cache_path(path)
    os.makedirs(os.path.dirname(p) or ".", exist_ok=True)
    data = {}
    if os.path.exists(p):
        try:
            with open(p) as f:
                data = json.load(f)
        except (OSError, ValueError):
            data = {}
    data[autotune_key(prep)] = {"C0": int(C0), "Cg": int(Cg), "wide": bool(wide),
                                "ms": None if times is None else min(times.values())}
    tmp = p + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, p)


def autotune(prep, C0s=(8, 16, 32, 64, 128), Cgs=(2, 4), widths=(False, True), iterations=3, repeats=2,
             timer=None):
    """Chunk length C0, group size Cg and level-0 team width (narrow or wide
    teams: lanes per chunk) for a prepared batch, by timing: each candidate
    runs `iterations` IEKS iterations of the whole batch (maxiters caps the
    solve; the work per iteration is what differs between candidates), best
    of `repeats`, CUDA events on the current stream.  Returns
    (C0, Cg, wide, {(C0, Cg, wide): ms}).  A problem's result depends on
    these only through rounding; pass the same values again to reproduce it.
    `timer(C0, Cg, wide)` (ms) replaces the measurement."""
    times = {}
    if timer is None:
        dev = prep["x0m"].device
        means = torch.empty_like(prep["means0"])
        G, D = means.shape
        chols = torch.empty((G, D, D), dtype=torch.float64, device=dev)
        info = torch.zeros((prep["B"], _lib.I_COUNT), dtype=torch.float64, device=dev)
        ws = [None]

        def timer(C0, Cg, wide):
            best = float("inf")
            with _TeamWidth(wide):
                for _ in range(repeats):
                    means.copy_(prep["means0"])
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record()
                    ws[0] = run_batch(prep, means, chols, info, maxiters=iterations - 1, C0=C0, Cg=Cg,
                                      workspace=ws[0])
                    e1.record()
                    e1.synchronize()
                    best = min(best, e0.elapsed_time(e1))
            return best

    for wide in widths:
        for C0 in C0s:
            for Cg in Cgs:
                times[(C0, Cg, wide)] = timer(C0, Cg, wide)
    C0, Cg, wide = min(times, key=times.get)
    return C0, Cg, wide, times


def tuned(prep, cache=True, path=None, **kwargs):
    """(C0, Cg, wide) for a batch: from the autotune cache when it has the
    batch's key (autotune_key), else by autotune, then stored (cache=True)."""
    if cache:
        hit = load_tuning(prep, path)
        if hit is not None:
            return hit
    C0, Cg, wide, times = autotune(prep, **kwargs)
    if cache:
        store_tuning(prep, C0, Cg, wide, times, path)
    return C0, Cg, wide


def project(prep, means, chols):
    """(E0 P) applied per problem: ys.mean (G, d) and ys.chol (G, d, D), as
    pof.solver.solve returns (gmul_stack(E0 P, states))."""
    q1 = prep["q"] + 1
    counts = torch.as_tensor(prep["n_steps"] + 1, device=means.device)
    p0 = torch.repeat_interleave(prep["p0"].to(means.device), counts)
    idx = torch.arange(prep["d"], device=means.device) * q1
    return means[:, idx] * p0[:, None], chols[:, idx, :] * p0[:, None, None]


def solve_batch(problems, order, init="constant", calibrate=True, maxiters=10_000, C0=0, Cg=0,
                precision="float64", maxiters_f32=10_000, rtol_f32=1e-5, settle_f32=float("inf")):
    """Solve every (field name, params, y0, ts) of ``problems`` with the
    parallel IEKS of pof.solver.solve (built-in fields, constant init).
    precision="mixed": float32 iterations first, float64 polish after, per
    problem (as pof.solver.solve's precision="mixed").  C0="auto" picks the
    chunk length, group size and level-0 team width by timing (autotune),
    or from the autotune cache file (POF_AUTOTUNE_CACHE, default
    ~/.cache/pof_gb300/autotune.json) for a batch of the same key.  Returns a
    BatchResult; ``result.problem(b)`` gives problem b's
    ((means (N_b, d), chol_covs (N_b, d, D)), info) as pof.solver.solve."""
    dev = default_device()
    prep = prepare_batch(problems, order, device=dev, init=init)
    wide = None
    if C0 == "auto":
        C0, Cg, wide = tuned(prep)
    means = prep["means0"].clone()
    G, D = means.shape
    chols = torch.empty((G, D, D), dtype=torch.float64, device=dev)
    info = torch.zeros((prep["B"], _lib.I_COUNT), dtype=torch.float64, device=dev)
    info32 = torch.zeros((prep["B"], 2), dtype=torch.float64, device=dev) if precision == "mixed" else None
    with _TeamWidth(wide):
        run_batch(prep, means, chols, info, maxiters=maxiters, calibrate=calibrate, C0=C0, Cg=Cg,
                  precision=precision, maxiters_f32=maxiters_f32, rtol_f32=rtol_f32, info_f32=info32,
                  settle_f32=settle_f32)
    ym, yc = project(prep, means, chols)
    info_d = {"iterations": info[:, _lib.I_ITERATIONS].to(torch.int64), "nll": info[:, _lib.I_NLL],
              "obj": info[:, _lib.I_OBJ], "sigma_squared": info[:, _lib.I_SSQ],
              "status": info[:, _lib.I_STATUS].to(torch.int64), "calibrated": bool(calibrate)}
    if info32 is not None:
        info_d["iterations_float32"] = info32[:, 0].to(torch.int64)
        info_d["best_change_float32"] = info32[:, 1]
    return BatchResult(ym, yc, prep["offsets"], info_d)


def shard(n_steps, world):
    """Split a batch across `world` ranks by work: problems are taken
    longest first and each goes to the rank holding the fewest steps so far
    (ties: the lower rank).  Returns one sorted index array per rank.  The
    partition depends only on the step counts, so every rank computes the
    same one without talking to the others."""
    n_steps = np.asarray(n_steps, dtype=np.int64)
    load = np.zeros(world, dtype=np.int64)
    parts = [[] for _ in range(world)]
    for b in np.argsort(-n_steps, kind="stable"):
        r = int(np.argmin(load))
        parts[r].append(int(b))
        load[r] += int(n_steps[b])
    return [np.array(sorted(p), dtype=np.int64) for p in parts]


def solve_batch_sharded(problems, order, rank, world, group=None, solver=None, **kwargs):
    """solve_batch of one fixed batch split over the ranks of a
    torch.distributed process group: rank `rank` solves its share
    (pof.batch.shard), then the per-problem results are all-gathered (one
    collective after the solve; the solve itself exchanges nothing) and every
    rank returns the whole batch's BatchResult on the host, in the original
    problem order.  A problem's result depends only on its own inputs, so it
    is the one a single-rank solve gives.  `solver(problems, order,
    **kwargs)` replaces solve_batch (it must return a BatchResult)."""
    import torch.distributed as dist

    solver = solver or solve_batch
    n_steps = [len(p[3]) - 1 for p in problems]
    mine = shard(n_steps, world)[rank]
    local = []
    if len(mine):
        res = solver([problems[b] for b in mine], order, **kwargs)
        for i, b in enumerate(mine):
            (m, L), info = res.problem(i)
            info = {k: (v.detach().cpu() if torch.is_tensor(v) else v) for k, v in info.items()}
            local.append((int(b), m.detach().cpu(), L.detach().cpu(), info))
    gathered = [None] * world
    dist.all_gather_object(gathered, local, group=group)
    per = {}
    for part in gathered:
        for b, m, L, info in part:
            per[b] = (m, L, info)
    order_b = range(len(problems))
    mean = torch.cat([per[b][0] for b in order_b])
    chol = torch.cat([per[b][1] for b in order_b])
    offsets = np.concatenate([[0], np.cumsum([per[b][0].shape[0] for b in order_b])]).astype(np.int64)
    keys = [k for k in per[0][2] if k != "calibrated"]
    info = {k: torch.stack([torch.as_tensor(per[b][2][k]) for b in order_b]) for k in keys}
    info["calibrated"] = per[0][2].get("calibrated", True)
    return BatchResult(mean, chol, offsets, info)
