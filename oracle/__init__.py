"""NumPy float64 oracle for the parallel-in-time IEKS path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package imports this
package; only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of ``bench.py`` use it, and only as the checker (or, in ``bench.py``, as the
timed CPU restatement of the reference).

The reference (``pof``, a JAX package) cannot be imported on these machines:
JAX, tornadox and diffrax are not installed.  Every function here is a CPU
restatement of the reference's arithmetic and cites the reference file:line it
follows.  Parity of this restatement is pinned by

* the reference's own identity test (sequential filter/smoother == parallel
  filter/smoother, ``tests/test_filtsmooth.py:41-62``),
* its shape/identity tests (``tests/test_observations.py:23-33``,
  ``tests/test_transtions.py:21-44``), and
* the reference's published float64 solver outputs: IEKS iteration counts and
  trajectory RMSE per (IVP, N, q) from
  ``experiments/3_work_precision_diagram/data/*_Tesla_V100-SXM2-32GB.csv``
  (committed as ``tests/golden/v100_ieks.json`` by
  ``tests/golden/make_v100_goldens.py``).

Modules:
  core       -- tria, likelihood, whitening, objective, IWP prior, projections
  scan       -- JAX's odd/even associative-scan recursion (restated)
  filtsmooth -- parallel (associative-scan) and sequential sqrt filter/smoother
  blocked    -- the chunked three-phase algorithm the CUDA kernels execute
  taylor     -- truncated Taylor arithmetic for Taylor-mode initialisation
  ivp        -- the reference's built-in vector fields (+ analytic Jacobians)
  solver     -- set-up, initial trajectories, IEKS loop, convergence criterion
"""

from . import core, scan, filtsmooth, blocked, taylor, ivp, solver  # noqa: F401
