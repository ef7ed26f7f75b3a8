"""FP64 NumPy oracle for the square-root parallel smoother.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package imports this
directory.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may use it, and
only as the checker or as the timed CPU port of the reference.

It restates, in batched NumPy, the algorithms of ``parsmooth``
(EEA-sensors/sqrt-parallel-smoothers).  Every function cites the reference
file:line it follows.  The reference itself (JAX 0.4.30) cannot be imported
in this environment, so parity is pinned against the reference's own golden
vectors (``tests/bearings/{ys.npy,icks.npz,ieks.npz}`` and the FP32 GPU
log-likelihoods in ``notebooks/robustness_data``), which are copied into
``tests/golden/`` by ``tests/golden/make_golden.py``.
"""

from .core import (tria, canon, cholesky_update, cholesky_update_many, mvn_loglikelihood,
                   solve_lower, solve_upper)
from .types import MVNSqrt, MVNStandard, FunctionalModel, ConditionalMomentsModel
from . import models, linearization, parallel, sequential, methods

__all__ = ["tria", "canon", "cholesky_update", "cholesky_update_many", "mvn_loglikelihood",
           "solve_lower", "solve_upper", "MVNSqrt", "MVNStandard", "FunctionalModel", "ConditionalMomentsModel",
           "models", "linearization", "parallel", "sequential", "methods"]
