"""Evaluate the reference's CUDA-C expression strings with NumPy.

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports this module; only
``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
use the oracle, and only as the checker.

The reference pastes user strings (``V``, ``K``, ``diff_V``, observables,
initial conditions) verbatim into ``__device__`` bodies
(wigner_moyal_cuda_1d.py:241-247, :781-827).  The oracle needs the same
arithmetic on the host, so this module maps the small C subset those strings
use (arithmetic, calls of the CUDA math library, ``cuda_complex(re, im)``,
``double(...)`` casts, ``M_PI`` and the ``#define`` constants) onto NumPy.
C-only syntax (``?:``, ``&&``) is rejected; user ``functions`` written in C
must be supplied as Python callables through ``py_functions``.
"""
import re

import numpy as np

_C_ONLY = re.compile(r"\?|&&|\|\||->|\bint\s*\(")


def _to_double(x):
    return np.asarray(x, dtype=np.float64)


def _cuda_complex(re_part, im_part=0.0):
    return np.asarray(re_part) + 1j * np.asarray(im_part)


def _conj(z):
    return np.conj(z)


BASE_NAMESPACE = {
    "pow": np.power,
    "exp": np.exp,
    "sqrt": np.sqrt,
    "sin": np.sin,
    "cos": np.cos,
    "tan": np.tan,
    "atan": np.arctan,
    "atan2": np.arctan2,
    "asin": np.arcsin,
    "acos": np.arccos,
    "sinh": np.sinh,
    "cosh": np.cosh,
    "tanh": np.tanh,
    "log": np.log,
    "log10": np.log10,
    "fabs": np.abs,
    "abs": np.abs,
    "floor": np.floor,
    "ceil": np.ceil,
    "fmin": np.minimum,
    "fmax": np.maximum,
    "erf": None,  # filled lazily from scipy
    "conj": _conj,
    "double": _to_double,
    "cuda_complex": _cuda_complex,
    "M_PI": np.pi,
}


def translate(expr):
    """Return a Python expression equivalent to the C expression ``expr``."""
    if _C_ONLY.search(expr):
        raise ValueError("C construct not supported by the NumPy evaluator: %r" % expr)
    # C float suffixes (1.f, 2.0f) are not Python
    expr = re.sub(r"(\d\.?\d*)[fF]\b", r"\1", expr)
    return expr


class CExpr:
    """A compiled C expression evaluated over NumPy arrays.

    ``defines`` maps the reference's ``#define`` names to their values (already
    rounded exactly as ``'%.15e'`` rounds them, wigner_moyal_cuda_1d.py:171-176).
    """

    def __init__(self, expr, defines, py_functions=None):
        if callable(expr):
            self.fn = expr
            self.code = None
            return
        self.fn = None
        self.source = expr
        self.code = compile(translate(expr), "<cexpr>", "eval")
        ns = dict(BASE_NAMESPACE)
        if ns["erf"] is None:
            from scipy.special import erf

            ns["erf"] = erf
        ns.update(defines)
        if py_functions:
            ns.update(py_functions)
        self.ns = ns

    def __call__(self, **variables):
        if self.fn is not None:
            return self.fn(**variables)
        ns = dict(self.ns)
        ns.update(variables)
        return eval(self.code, ns)
