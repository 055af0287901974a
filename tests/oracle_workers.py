"""Oracle runs for process pools (test infrastructure; imports NumPy and the oracle only, no torch).

A pool that runs these must use the ``spawn`` start method: a process forked
after the parent has initialised CUDA can hang.
"""

import numpy as np

from oracle import fem_oracle as O


def fixed_iteration_dv(job):
    """One scene's velocity increment after one substep with exactly ``iterations`` CG updates.

    ``job`` is a dict of float32-rounded float64 arrays and settings, keyed like
    ``OracleFEM``'s keyword arguments plus ``x``, ``mass``, ``q``, ``v`` and ``iterations``.
    """
    job = dict(job)
    x, mass, q, v, iterations = (job.pop(k) for k in ("x", "mass", "q", "v", "iterations"))
    oracle = O.OracleFEM(x, mass, **job)
    oracle.refresh_tangent(q)
    oracle.step(q, v, oracle.dt, fixed_iterations=iterations)
    return oracle.dv, oracle.last_iterations
