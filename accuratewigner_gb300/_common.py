"""Host-side helpers shared by the propagator classes.

Keyword handling, the ``#define`` block and the expression analysis follow the
reference constructors (wigner_moyal_cuda_1d.py:43-182,
rho_vneumann_cuda_1d.py:48-179, schrodinger_wigner_cuda_1d.py:50-151).
"""
import ctypes
import re
import threading
import types

import numpy as np

from . import _lib

_IDENT = re.compile(r"[A-Za-z_]\w*")
_DEFINE = re.compile(r"^\s*#\s*define\s+([A-Za-z_]\w*)(\([^)]*\))?\s*(.*)$", re.M)


def is_int_kwarg(v):
    return isinstance(v, (bool, int, np.integer))


def is_float_kwarg(v):
    return isinstance(v, (float, np.floating)) and not isinstance(v, bool)


def define_value(v):
    """The value a kernel sees for ``#define name %.15e`` (wigner_moyal_cuda_1d.py:176)."""
    if is_int_kwarg(v):
        return int(v)
    return float("%.15e" % v)


def cuda_defines(kwargs):
    """wigner_moyal_cuda_1d.py:171-176: ints as %d, floats as %.15e."""
    out = ""
    for name, value in kwargs.items():
        if is_int_kwarg(value):
            out += "#define %s %d\n" % (name, int(value))
        elif is_float_kwarg(value):
            out += "#define %s %.15e\n" % (name, value)
    return out


def bind_kwargs(obj, kwargs):
    """Every keyword becomes an attribute; functions become bound methods (wm:43-50)."""
    for name, value in kwargs.items():
        if isinstance(value, types.FunctionType):
            setattr(obj, name, types.MethodType(value, obj))
        else:
            setattr(obj, name, value)


def require(obj, name, message):
    if not hasattr(obj, name):
        raise AttributeError(message)


def assert_pow2(n, message):
    assert 2 ** int(np.log2(n)) == n, message


class ExprInfo:
    """Identifiers an expression depends on, expanding the user's own macros."""

    def __init__(self, consts_text):
        self.macros = {}
        for m in _DEFINE.finditer(consts_text or ""):
            self.macros[m.group(1)] = m.group(3)

    def tokens(self, expr):
        seen = set()
        todo = list(_IDENT.findall(expr))
        out = set()
        while todo:
            tok = todo.pop()
            if tok in seen:
                continue
            seen.add(tok)
            out.add(tok)
            if tok in self.macros:
                todo.extend(_IDENT.findall(self.macros[tok]))
        return out

    def depends_on(self, expr, name):
        return name in self.tokens(expr)

    def classify(self, expr):
        """'X' (no P), 'P' (no X) or '2d'."""
        tok = self.tokens(expr)
        has_x = "X" in tok or "i" in tok or "j" in tok
        has_p = "P" in tok or "i" in tok or "j" in tok
        if has_x and has_p:
            return "2d"
        if has_p:
            return "P"
        return "X"


def split_sum_terms(expr):
    """Top-level '+'-separated pieces of `a + b` strings built by the reference (wm:301)."""
    return [expr]


class TermTable:
    """Observables recorded every step, as sums of X-only and P-only terms."""

    def __init__(self, info):
        self.info = info
        self.obs_x = []
        self.obs_p = []
        self.terms = []   # (slot, kind, index, coef)
        self.n_slots = 0
        self.ok = True

    def _index(self, lst, expr):
        if expr not in lst:
            lst.append(expr)
        return lst.index(expr)

    def add_slot(self, parts):
        """parts: list of (expr, coef); returns the slot index."""
        slot = self.n_slots
        self.n_slots += 1
        for expr, coef in parts:
            kind = self.info.classify(expr)
            if kind == "2d":
                self.ok = False
                continue
            if kind == "X":
                self.terms.append((slot, _lib.AW_TERM_X, self._index(self.obs_x, expr), float(coef)))
            else:
                self.terms.append((slot, _lib.AW_TERM_P, self._index(self.obs_p, expr), float(coef)))
        return slot

    def fill(self, cfg, keep):
        """Populate the observable fields of an AwConfig; `keep` holds the ctypes arrays alive."""
        ox = (ctypes.c_char_p * max(1, len(self.obs_x)))(*[e.encode() for e in self.obs_x])
        op = (ctypes.c_char_p * max(1, len(self.obs_p)))(*[e.encode() for e in self.obs_p])
        n = max(1, len(self.terms))
        slot = (ctypes.c_int32 * n)(*[t[0] for t in self.terms])
        kind = (ctypes.c_int32 * n)(*[t[1] for t in self.terms])
        idx = (ctypes.c_int32 * n)(*[t[2] for t in self.terms])
        coef = (ctypes.c_double * n)(*[t[3] for t in self.terms])
        keep.extend([ox, op, slot, kind, idx, coef])
        cfg.n_obs_x = len(self.obs_x)
        cfg.obs_x = ox
        cfg.n_obs_p = len(self.obs_p)
        cfg.obs_p = op
        cfg.n_terms = len(self.terms)
        cfg.term_slot = slot
        cfg.term_kind = kind
        cfg.term_index = idx
        cfg.term_coef = coef
        cfg.n_slots = self.n_slots
        cfg.obs_p_time_dependent = int(any(self.info.depends_on(e, "t") for e in self.obs_p))


# precision of propagators constructed without the keyword: the reference's own arithmetic
# (pycuda::complex<double>, wigner_moyal_cuda_1d.py:629)
DEFAULT_PRECISION = "c128-fp64"


def precision_code(kwargs):
    """State and arithmetic of the passes.

    'c128-fp64' (default): complex128 state, passes in native FP64 arithmetic.
    'c128': complex128 state, passes in double-float arithmetic on the FP32 pipes (about 1e-13 from
            FP64, values below about 1e-30 lose their low part; about 3x faster).
    'c64': complex64 state and passes, FP64 tables and reductions.
    """
    p = kwargs.get("precision", DEFAULT_PRECISION)
    if isinstance(p, str) or p in (np.complex128, np.complex64):
        if p in ("c128", "complex128", np.complex128):
            return _lib.AW_C128
        if p in ("c128-fp64", "fp64"):
            return _lib.AW_C128_FP64
        if p in ("c64", "complex64", np.complex64):
            return _lib.AW_C64
    elif p in (_lib.AW_C128, _lib.AW_C64, _lib.AW_C128_FP64):
        return int(p)
    raise ValueError("precision must be 'c128', 'c128-fp64' or 'c64'")


def mask_mode(info, expr):
    """0: identically one, 1: fixed in time, 2: depends on t."""
    if expr.strip() in ("1.", "1", "1.0", "(1.)"):
        return 0
    return 2 if info.depends_on(expr, "t") else 1


def apply_batch(cfg, kwargs, keep):
    """Batch fields of an AwConfig from the keywords n_inst, batch_params, batch_init.

    n_inst instances of the propagator share the handle; batch_params are the names of the
    per-instance constants (usable in V, K, the absorbing boundaries, the observables and
    batch_init, the initial state of an instance).  No reference counterpart: the batched
    and served forms.
    """
    names = [str(n) for n in kwargs.get("batch_params", ()) or ()]
    cfg.n_inst = int(kwargs.get("n_inst", 1) or 1)
    cfg.n_params = len(names)
    arr = (ctypes.c_char_p * max(1, len(names)))(*[n.encode() for n in names])
    keep.append(arr)
    cfg.param_names = arr
    init = kwargs.get("batch_init", "") or ""
    b = init.encode()
    keep.append(b)
    cfg.init_expr = b


class _ConfigChecked(Exception):
    """Ends a constructor run by check_config once its configuration has been checked."""


_CHECK = threading.local()


def check_config(cls, arch="sm_103a", **kwargs):
    """Run the constructor of a propagator class up to its native handle, then validate the
    configuration and compile its expression strings with NVRTC for `arch` instead of creating the
    handle: no GPU is needed.  Raises what the constructor would raise (AttributeError for a
    missing keyword, AssertionError for a grid that is not a power of two, RuntimeError for an
    expression that does not compile); returns None when the configuration is good."""
    _CHECK.arch = arch
    try:
        cls(**kwargs)
    except _ConfigChecked:
        return None
    finally:
        _CHECK.arch = None
    raise RuntimeError("%s made no native handle" % cls.__name__)


class Handle:
    """Owns one native propagator handle."""

    def __init__(self, cfg):
        lib = _lib.load()
        arch = getattr(_CHECK, "arch", None)
        if arch is not None:
            _lib.check(lib.aw_check_config(ctypes.byref(cfg), arch.encode()))
            raise _ConfigChecked()
        h = ctypes.c_void_p()
        _lib.check(lib.aw_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().aw_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
