"""Oracle container types (TEST INFRASTRUCTURE ONLY).

Restates ``parsmooth/_base.py:5-30``: plain named tuples, and the
"all inputs must have the same type" check that raises ``TypeError``.
"""
from typing import Any, Callable, NamedTuple


class MVNStandard(NamedTuple):
    """Gaussian in covariance form (parsmooth/_base.py:5-7)."""
    mean: Any
    cov: Any


class MVNSqrt(NamedTuple):
    """Gaussian in square-root form, ``cov = chol @ chol.T`` (parsmooth/_base.py:10-12)."""
    mean: Any
    chol: Any


class FunctionalModel(NamedTuple):
    """``x_next = function(x) + q``, ``q ~ mvn`` (parsmooth/_base.py:15-17)."""
    function: Callable
    mvn: Any


class ConditionalMomentsModel(NamedTuple):
    """``E[y | x]`` and ``Cov[y | x]`` (or its Cholesky factor) as callables (parsmooth/_base.py:20-22)."""
    conditional_mean: Callable
    conditional_covariance_or_cholesky: Callable


def are_inputs_compatible(*ys):
    """Raise ``TypeError`` unless consecutive inputs share a type (parsmooth/_base.py:25-30)."""
    types = [type(y) for y in ys]
    if not any(a == b for a, b in zip(types[:-1], types[1:])):
        raise TypeError(f"All inputs should have the same type. {ys} was given")
