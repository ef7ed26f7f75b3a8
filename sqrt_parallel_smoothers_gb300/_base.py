"""Container types with the names and fields of ``parsmooth._base`` (parsmooth/_base.py:5-30)."""
import itertools
from typing import Any, Callable, NamedTuple


class MVNStandard(NamedTuple):
    """Gaussian ``N(mean, cov)`` in covariance form.  The GPU path factors ``cov`` (``L L^T``)
    and computes in square-root form; covariance-form inputs give covariance-form outputs."""
    mean: Any
    cov: Any


class MVNSqrt(NamedTuple):
    """Gaussian ``N(mean, chol chol^T)`` with ``chol`` lower triangular."""
    mean: Any
    chol: Any


class FunctionalModel(NamedTuple):
    """``x' = function(x) + q``, ``q ~ mvn``.  ``function`` must be a device model from
    :mod:`sqrt_parallel_smoothers_gb300.models`."""
    function: Callable
    mvn: Any


class ConditionalMomentsModel(NamedTuple):
    """Conditional-moments model (parsmooth/_base.py:20-22).  On the GPU path both functions
    must be the conditional moments of one device model (``models.Ricker``,
    ``models.PoissonExp``, ``models.population_parameters``)."""
    conditional_mean: Callable
    conditional_covariance_or_cholesky: Callable


def are_inputs_compatible(*y):
    """Raise ``TypeError`` when consecutive inputs differ in type (parsmooth/_base.py:25-30)."""
    a, b = itertools.tee(map(type, y))
    next(b, None)
    if not sum(u == v for u, v in zip(a, b)):
        raise TypeError(f"All inputs should have the same type. {y} was given")
