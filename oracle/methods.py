"""Oracle public entry points (TEST INFRASTRUCTURE ONLY).

Restates parsmooth/methods.py:14-76 and the fixed-point loop of
parsmooth/_utils.py:103-149 (forward semantics only).
"""
import numpy as np

from . import parallel as par
from . import sequential as seq


def filtering(observations, x0, transition_model, observation_model, linearization_method,
              nominal_trajectory=None, parallel=True, return_loglikelihood=False):
    """parsmooth/methods.py:14-26."""
    mod = par if parallel else seq
    return mod.filtering(observations, x0, transition_model, observation_model, linearization_method,
                         nominal_trajectory, return_loglikelihood)


def smoothing(transition_model, filter_trajectory, linearization_method, nominal_trajectory=None,
              parallel=True):
    """parsmooth/methods.py:29-35."""
    mod = par if parallel else seq
    return mod.smoothing(transition_model, filter_trajectory, linearization_method, nominal_trajectory)


def filter_smoother(observations, x0, transition_model, observation_model, linearization_method,
                    nominal_trajectory=None, parallel=True):
    """parsmooth/methods.py:38-47."""
    filt = filtering(observations, x0, transition_model, observation_model, linearization_method,
                     nominal_trajectory, parallel)
    return smoothing(transition_model, filt, linearization_method, nominal_trajectory, parallel)


def default_criterion(_i, prev, curr):
    """Continue while the mean squared change of the means exceeds 1e-6 (parsmooth/methods.py:50-51)."""
    return float(np.mean((np.asarray(prev.mean) - np.asarray(curr.mean)) ** 2)) > 1e-6


def fixed_point(f, x0, criterion):
    """Forward semantics of parsmooth/_utils.py:136-146.

    Starts from ``(i=1, x0, f(x0))`` and iterates ``x <- f(x)`` while
    ``criterion(i, x_prev, x)``.  Returns ``(x_star, n_calls)``.
    """
    i, x_prev, x = 1, x0, f(x0)
    while criterion(i, x_prev, x):
        i, x_prev, x = i + 1, x, f(x)
    return x, i


def iterated_smoothing(observations, x0, transition_model, observation_model, linearization_method,
                       init_nominal_trajectory=None, parallel=True, criterion=default_criterion,
                       return_loglikelihood=False):
    """parsmooth/methods.py:54-76."""
    if init_nominal_trajectory is None:
        init_nominal_trajectory = filter_smoother(observations, x0, transition_model, observation_model,
                                                  linearization_method, None, parallel)

    def body(nominal):
        return filter_smoother(observations, x0, transition_model, observation_model,
                               linearization_method, nominal, parallel)

    traj, _ = fixed_point(body, init_nominal_trajectory, criterion)
    if return_loglikelihood:
        _, ell = filtering(observations, x0, transition_model, observation_model, linearization_method,
                           traj, parallel, return_loglikelihood=True)
        return traj, ell
    return traj
