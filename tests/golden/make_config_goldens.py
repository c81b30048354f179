"""Oracle results on the benchmark configurations, kept as a fixture.

The float64 oracle (``oracle/``, the NumPy restatement of the reference's
``pof.solver.solve``) needs minutes for these solves, too long to repeat in
every GPU test run, so its results are stored once:

* FitzHugh-Nagumo (a = b = 0.2, c = 3), y0 = (-1, 1), t in [0, 100],
  N = 1000, q = 3, constant init, the reference's default criterion: the
  IEKS in the reference's associative-scan order ("tree") and in the
  sequential filter/smoother order ("seq"): iteration counts, the objective
  and NLL of every iteration, the final solution y (N, 2), and the tree
  order's preconditioned iterates at a few iterations (inputs of the
  one-step parity test).  The sequential order does not meet the criterion
  within the reference's maxiters (10 000): its count is recorded as 10 001
  and only the first iterations of its trace are kept.
* Logistic y' = 3 y (1 - y), y0 = 0.01, t in [0, 10], q in {1, 2, 3, 5},
  N in {2^10, 2^12, 2^14}, constant init: iteration counts of both orders,
  obj / NLL / sigma^2, y at every 16th grid point (and the last), and the
  largest difference between the two orders' solutions (the spread that
  rounding alone produces on this problem).

Run from the repository root (about two hours on 8 cores: the sequential
order of the FitzHugh-Nagumo solve is the long one; --no-fhn-seq leaves it
out, about ten minutes, and records its iteration count as -1):

    python tests/golden/make_config_goldens.py [--no-fhn-seq]
"""

import concurrent.futures as cf
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "config_goldens.npz")

FHN_KEEP = (20, 400, 656)
LOGISTIC_Q = (1, 2, 3, 5)
LOGISTIC_N = (2**10, 2**12, 2**14)
SUB = 16


def _solve(kind, q, N, order):
    sys.path.insert(0, ROOT)
    from oracle import ivp as oivp, solver as osolver
    from oracle.scan import associative_scan, sequential_scan

    scan = associative_scan if order == "tree" else sequential_scan
    if kind == "fhn":
        ivp, t1 = oivp.fhn_classic(), 100.0
    else:
        ivp, t1 = oivp.logistic(r=3.0), 10.0
    ts = np.linspace(ivp.t0, t1, N)
    trace, keep = [], {}

    def cb(k, states, nll, obj, ssq):
        trace.append((obj, nll, ssq))
        if kind == "fhn" and order == "tree" and k in FHN_KEEP:
            keep[k] = states[0].copy()

    states, info, st = osolver.solve(ivp, ts, q, init="constant", maxiters=10_000, scan=scan, return_full=True,
                                     callback=cb)
    y = states[0] @ st.E0.T
    return dict(kind=kind, q=q, N=N, order=order, iterations=info["iterations"], obj=info["obj"],
                nll=info["nll"], ssq=info["sigma_squared"], y=y, trace=np.array(trace), keep=keep)


def main():
    for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[k] = "1"
    fhn_orders = ("tree",) if "--no-fhn-seq" in sys.argv else ("seq", "tree")
    jobs = [("fhn", 3, 1000, o) for o in fhn_orders]
    jobs += [("logistic", q, N, o) for q in LOGISTIC_Q for N in LOGISTIC_N for o in ("tree", "seq")]
    res = {}
    with cf.ProcessPoolExecutor(os.cpu_count(), mp_context=mp.get_context("spawn")) as ex:
        futs = {ex.submit(_solve, *j): j for j in jobs}
        for f in cf.as_completed(futs):
            r = f.result()
            res[futs[f]] = r
            print(futs[f], r["iterations"], flush=True)
    out = {}
    t = res[("fhn", 3, 1000, "tree")]
    s = res.get(("fhn", 3, 1000, "seq"))
    out["fhn_iterations"] = np.array([t["iterations"], s["iterations"] if s else -1])
    out["fhn_trace_tree"] = t["trace"]
    out["fhn_y_tree"] = t["y"]
    if s:  # its first iterations only (it runs to maxiters without meeting the criterion)
        out["fhn_trace_seq"] = s["trace"][:20]
        out["fhn_y_seq"] = s["y"]
    out["fhn_keep"] = np.array(FHN_KEEP)
    for k in FHN_KEEP:
        out["fhn_m%d" % k] = t["keep"][k]
    for q in LOGISTIC_Q:
        for N in LOGISTIC_N:
            t, s = res[("logistic", q, N, "tree")], res[("logistic", q, N, "seq")]
            idx = np.unique(np.r_[np.arange(0, N, SUB), N - 1])
            key = "log_q%d_N%d" % (q, N)
            out[key + "_iterations"] = np.array([t["iterations"], s["iterations"]])
            out[key + "_scalars"] = np.array([[t["obj"], t["nll"], t["ssq"]], [s["obj"], s["nll"], s["ssq"]]])
            out[key + "_idx"] = idx
            out[key + "_y"] = t["y"][idx, 0]
            out[key + "_spread"] = np.array(np.abs(t["y"] - s["y"]).max() / np.abs(t["y"]).max())
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
