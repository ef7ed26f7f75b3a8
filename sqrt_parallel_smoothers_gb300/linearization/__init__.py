"""Linearisation methods with the names of ``parsmooth.linearization``
(parsmooth/linearization/__init__.py:1-5).

Each object is a callable ``method(model, x) -> (F, chol, b)`` like the
reference's ``linearize`` functions, evaluated by the CUDA library, and also
a descriptor that the filter and smoother kernels read.  Keyword variants
follow the reference's signatures: ``unscented(model, x, alpha, beta, kappa)``
(parsmooth/linearization/_unscented.py:10-12) and
``gauss_hermite(model, x, order)`` (parsmooth/linearization/_gh.py:13-14);
``functools.partial`` of these objects is accepted wherever a method is.
"""
import functools

from .. import _lib


class Method:
    """A linearisation method descriptor."""

    def __init__(self, name, code, **params):
        self.name = name
        self.code = code
        self.params = params

    def with_params(self, **params):
        p = dict(self.params)
        p.update(params)
        return Method(self.name, self.code, **p)

    def __call__(self, model, x, *args, **kwargs):
        from ..methods import linearize
        m = self
        if args or kwargs:
            names = list(self.params)
            kw = dict(zip(names, args))
            kw.update(kwargs)
            m = self.with_params(**kw)
        return linearize(model, x, m)

    def __repr__(self):
        return f"{self.name}({', '.join(f'{k}={v}' for k, v in self.params.items())})"


extended = Method("extended", _lib.SS_LIN_EXTENDED)
cubature = Method("cubature", _lib.SS_LIN_CUBATURE)
unscented = Method("unscented", _lib.SS_LIN_UNSCENTED, alpha=1.0, beta=0.0, kappa=None)
gauss_hermite = Method("gauss_hermite", _lib.SS_LIN_GAUSS_HERMITE, order=3)


def resolve(method):
    """Turn a method object (or a ``functools.partial`` of one) into a :class:`Method`."""
    if isinstance(method, Method):
        return method
    if isinstance(method, functools.partial) and isinstance(method.func, Method):
        base = method.func
        kw = dict(zip(list(base.params), method.args))
        kw.update(method.keywords)
        return base.with_params(**kw)
    raise NotImplementedError(f"unsupported linearization method {method!r}; use "
                              "extended, cubature, unscented or gauss_hermite from this package")


def get_conditional_model(*_args, **_kwargs):
    """parsmooth/linearization/_common.py:17-66 turns a Python callable ``f(x, q)`` with
    non-additive noise into conditional moments by linearising it in ``q`` at every point.  A
    Python callable cannot run inside the CUDA kernels, so this raises
    ``NotImplementedError``; a :class:`ConditionalMomentsModel` of device models
    (``models.Ricker``, ``models.PoissonExp``, ``models.population_parameters``) is supported."""
    raise NotImplementedError("get_conditional_model needs a Python callable f(x, q), which cannot run in the "
                              "CUDA kernels; build a ConditionalMomentsModel from device models instead")
