"""Extract the reference's published float64 IEKS results into a fixture.

Source: the CSVs behind the reference paper's work-precision figures,
``experiments/3_work_precision_diagram/data/<setup>_Tesla_V100-SXM2-32GB.csv``
(written by ``experiments/3_work_precision_diagram/run_benchmark.py:170-230``:
``solve(f, y0, ts=linspace(t0, tmax, N), order=q, init="constant",
maxiters=1000)``, float64, ``pof.ivp`` default problem parameters).

For every (setup, N, q) row the fixture keeps the IEKS iteration count and
the trajectory / final-point RMSE against the reference's Kvaerno5 solution.

Run from the repository root:  python tests/golden/make_v100_goldens.py
"""

import csv
import json
import os
import sys

REF = "/root/reference/experiments/3_work_precision_diagram/data"
SETUPS = {
    # name: (csv stem, ivp constructor call used by run_benchmark.py:110-121)
    "logistic": ("logistic", "logistic()"),
    "fhn": ("fhn", "fitzhughnagumo()"),
    "vdp0": ("vdp0", "vanderpol(stiffness_constant=1e0)"),
    "rigidbody": ("rigidbody", "rigid_body()"),
    "henonheiles": ("henonheiles", "henonheiles(tmax=10.0)"),
}


def main(out=os.path.join(os.path.dirname(__file__), "v100_ieks.json")):
    rows = []
    for name, (stem, ctor) in SETUPS.items():
        path = os.path.join(REF, f"{stem}_Tesla_V100-SXM2-32GB.csv")
        for r in csv.DictReader(open(path)):
            for q in (1, 2, 3):
                it = r.get(f"IEKS({q})_iterations", "")
                if not it:
                    continue
                rows.append(
                    {
                        "setup": name,
                        "ivp": ctor,
                        "N": int(r["Ns"]),
                        "q": q,
                        "iterations": int(float(it)),
                        "rmse_traj": float(r[f"IEKS({q})_rmse_traj"]),
                        "rmse_final": float(r[f"IEKS({q})_rmse_final"]),
                        "runtime_s": float(r[f"IEKS({q})_runtime"]),
                        "seq_iterations": int(float(r[f"sIEKS({q})_iterations"])) if r.get(f"sIEKS({q})_iterations") else None,
                    }
                )
    doc = {
        "source": "experiments/3_work_precision_diagram/data/*_Tesla_V100-SXM2-32GB.csv",
        "generator": "tests/golden/make_v100_goldens.py",
        "solve": "pof.solver.solve(init='constant', maxiters=1000), ts = linspace(t0, tmax, N), float64",
        "rows": rows,
    }
    with open(out, "w") as f:
        json.dump(doc, f, indent=1)
    print(f"wrote {len(rows)} rows to {out}", file=sys.stderr)


if __name__ == "__main__":
    main()
