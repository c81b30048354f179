"""pof -- parallel-in-time probabilistic ODE solvers, GB300-native.

Drop-in for the reference package of the same name: the same modules and
entry points (pof.solver.solve, pof.parallel_filtsmooth.*, ...), with the
iterated extended Kalman smoother running in libpof, hand-written CUDA for
sm_103a behind a C ABI (include/pof.h).
"""

__version__ = "0.1.0"
