"""GB300-native square-root parallel smoother with the API of ``parsmooth``.

Drop-in for the parallel mode of ``parsmooth`` (EEA-sensors/sqrt-parallel-smoothers):
``filtering``, ``smoothing``, ``filter_smoother`` and ``iterated_smoothing``
with the extended, cubature, unscented and Gauss-Hermite linearisations, run
by hand-written CUDA kernels (``csrc/``) behind the C ABI of
``include/sqrtsmooth.h``.
"""
__version__ = "1.0.0"

from ._base import MVNSqrt, MVNStandard, FunctionalModel, ConditionalMomentsModel
from .methods import (filtering, smoothing, filter_smoother, iterated_smoothing, linearize, FixedIterations,
                      MeanSquaredChange, IteratedSmootherPlan, ModelTangent, filter_loglikelihood_grad,
                      BearingsLogLikelihood, set_large_state_options, sampling, filter_loglikelihood_adjoint,
                      LinearGaussianLogLikelihood)
from . import linearization, models, data

__all__ = ["MVNSqrt", "MVNStandard", "FunctionalModel", "ConditionalMomentsModel", "filtering", "smoothing",
           "filter_smoother", "iterated_smoothing", "linearize", "FixedIterations", "MeanSquaredChange",
           "IteratedSmootherPlan", "ModelTangent", "filter_loglikelihood_grad", "BearingsLogLikelihood",
           "set_large_state_options", "sampling", "filter_loglikelihood_adjoint", "LinearGaussianLogLikelihood",
           "linearization", "models", "data"]
