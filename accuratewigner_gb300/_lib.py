"""ctypes binding of libawigner.so (the C ABI declared in include/awigner.h).

The library is loaded from this package's directory.  There is no fallback:
if it is missing or cannot be loaded, importing a propagator raises.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libawigner.so")

AW_OK = 0
AW_E_ARG = -1
AW_E_CUDA = -2
AW_E_JIT = -3
AW_E_STATE = -4
AW_E_NOMEM = -5

AW_WIGNER_MOYAL = 0
AW_WIGNER_BLOCH = 1
AW_RHO_VNEUMANN = 2
AW_RHO_BLOCH = 3
AW_SCHRODINGER = 4

AW_C128 = 0
AW_C64 = 1
AW_C128_FP64 = 2

AW_BUF_RHO = 0
AW_BUF_WIGNER = 1
AW_BUF_PSI = 2
AW_BUF_SNAPSHOT = 3

AW_PROF_CLASSES = 5  # launch classes of aw_profile_read

AW_TERM_X = 0
AW_TERM_P = 1

c_int = ctypes.c_int32
c_i64 = ctypes.c_int64
c_dbl = ctypes.c_double
c_vp = ctypes.c_void_p
c_cp = ctypes.c_char_p


class AwConfig(ctypes.Structure):
    _fields_ = [
        ("kind", c_int),
        ("precision", c_int),
        ("x_grid_dim", c_int),
        ("p_grid_dim", c_int),
        ("dX", c_dbl),
        ("dP", c_dbl),
        ("dXX", c_dbl),
        ("dXX_prime", c_dbl),
        ("dPP", c_dbl),
        ("dPP_prime", c_dbl),
        ("dt", c_dbl),
        ("t_initial", c_dbl),
        ("dXdP", c_dbl),
        ("cuda_consts", c_cp),
        ("V", c_cp),
        ("K", c_cp),
        ("abs_boundary_x", c_cp),
        ("abs_boundary_p", c_cp),
        ("v_time_dependent", c_int),
        ("k_time_dependent", c_int),
        ("absx_mode", c_int),
        ("absp_mode", c_int),
        ("ehrenfest", c_int),
        ("n_obs_x", c_int),
        ("obs_x", ctypes.POINTER(c_cp)),
        ("n_obs_p", c_int),
        ("obs_p", ctypes.POINTER(c_cp)),
        ("n_terms", c_int),
        ("term_slot", ctypes.POINTER(c_int)),
        ("term_kind", ctypes.POINTER(c_int)),
        ("term_index", ctypes.POINTER(c_int)),
        ("term_coef", ctypes.POINTER(c_dbl)),
        ("n_slots", c_int),
        ("obs_p_time_dependent", c_int),
        ("n_inst", c_int),
        ("n_params", c_int),
        ("param_names", ctypes.POINTER(c_cp)),
        ("init_expr", c_cp),
    ]


# (name, restype, argtypes) of every entry point in include/awigner.h
SIGNATURES = [
    ("aw_version", c_int, []),
    ("aw_last_error", c_cp, []),
    ("aw_launch_count", c_i64, []),
    ("aw_profile", c_int, [c_vp, c_int]),
    ("aw_graph", c_int, [c_vp, c_int]),
    ("aw_group_propagate", c_int, [ctypes.POINTER(c_vp), c_int, c_i64, ctypes.POINTER(c_dbl)]),
    ("aw_pass_form", c_int, [c_vp, ctypes.POINTER(c_int), ctypes.POINTER(c_int)]),
    ("aw_profile_read", c_int, [c_vp, ctypes.POINTER(c_dbl), ctypes.POINTER(c_dbl), ctypes.POINTER(c_i64)]),
    ("aw_create", c_int, [ctypes.POINTER(AwConfig), ctypes.POINTER(c_vp)]),
    ("aw_destroy", c_int, [c_vp]),
    ("aw_check_config", c_int, [ctypes.POINTER(AwConfig), c_cp]),
    ("aw_stream", c_int, [c_vp, ctypes.POINTER(c_vp)]),
    ("aw_sync", c_int, [c_vp]),
    ("aw_bloch_min", c_int, [c_vp, ctypes.POINTER(c_dbl), ctypes.POINTER(c_dbl)]),
    ("aw_buffer", c_int, [c_vp, c_int, ctypes.POINTER(c_vp), ctypes.POINTER(c_i64), ctypes.POINTER(c_i64),
                          ctypes.POINTER(c_int)]),
    ("aw_set_buffer", c_int, [c_vp, c_int, c_vp, c_int]),
    ("aw_get_buffer", c_int, [c_vp, c_int, c_vp, c_int]),
    ("aw_copy_buffer", c_int, [c_vp, c_int, c_int]),
    ("aw_fill_expr", c_int, [c_vp, c_int, c_cp]),
    ("aw_fill_const", c_int, [c_vp, c_int, c_dbl, c_dbl]),
    ("aw_sum", c_int, [c_vp, c_int, ctypes.POINTER(c_dbl), ctypes.POINTER(c_dbl)]),
    ("aw_trace", c_int, [c_vp, ctypes.POINTER(c_dbl), ctypes.POINTER(c_dbl)]),
    ("aw_scale", c_int, [c_vp, c_int, c_dbl, c_dbl]),
    ("aw_wigner2rho", c_int, [c_vp]),
    ("aw_rho2wigner", c_int, [c_vp, c_int]),
    ("aw_normalize_rho_wigner", c_int, [c_vp]),
    ("aw_propagate", c_int, [c_vp, c_i64, ctypes.POINTER(c_dbl)]),
    ("aw_single_step", c_int, [c_vp, c_dbl]),
    ("aw_history", c_int, [c_vp, c_vp, c_i64, ctypes.POINTER(c_i64), ctypes.POINTER(c_int)]),
    ("aw_average", c_int, [c_vp, c_cp, c_dbl, ctypes.POINTER(c_dbl)]),
    ("aw_average_ops", c_int, [c_vp, ctypes.POINTER(c_cp), c_int, c_dbl, ctypes.POINTER(c_dbl)]),
    ("aw_purity", c_int, [c_vp, ctypes.POINTER(c_dbl)]),
    ("aw_bloch_step", c_int, [c_vp, c_dbl, c_vp]),
    ("aw_gibbs", c_int, [c_vp, c_dbl, c_i64, ctypes.POINTER(c_i64), ctypes.POINTER(c_dbl)]),
    ("aw_sw_imag_steps", c_int, [c_vp, c_i64, c_int]),
    ("aw_sw_store_state", c_int, [c_vp]),
    ("aw_sw_clear_states", c_int, [c_vp]),
    ("aw_sw_get_state", c_int, [c_vp, c_int, c_vp]),
    ("aw_sw_energy", c_int, [c_vp, c_dbl, ctypes.POINTER(c_dbl)]),
    ("aw_sw_ehrenfest", c_int, [c_vp, c_dbl, ctypes.POINTER(c_dbl)]),
    ("aw_reduce_noalloc", c_int, [c_vp, c_int, c_i64, c_i64, c_int, c_vp, c_vp]),
    ("aw_set_view", c_int, [c_vp, c_int, c_int]),
    ("aw_set_params", c_int, [c_vp, c_int, ctypes.POINTER(c_dbl)]),
    ("aw_set_active", c_int, [c_vp, ctypes.POINTER(c_int)]),
    ("aw_init_state", c_int, [c_vp]),
    ("aw_history_of", c_int, [c_vp, c_int, c_vp, c_i64, ctypes.POINTER(c_i64), ctypes.POINTER(c_int)]),
    ("aw_gibbs_batch", c_int, [c_vp, ctypes.POINTER(c_dbl), c_i64, ctypes.POINTER(c_i64), ctypes.POINTER(c_dbl)]),
    ("aw_bloch_min_of", c_int, [c_vp, c_int, ctypes.POINTER(c_dbl), ctypes.POINTER(c_dbl)]),
]

_lib = None


def load():
    """Load libawigner.so once; raise ImportError when it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            "libawigner.so is not built: run `python -c 'import __graft_entry__ as g; g.build()'` "
            "(or python accuratewigner_gb300/_build.py) first")
    lib = ctypes.CDLL(LIB_PATH)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class AwError(RuntimeError):
    pass


def check(code):
    """Map a status code to the exception type the reference raises for that failure."""
    if code == AW_OK:
        return
    msg = load().aw_last_error().decode(errors="replace")
    if code == AW_E_ARG:
        raise AssertionError(msg)
    if code == AW_E_JIT:
        raise RuntimeError(msg)
    if code == AW_E_NOMEM:
        raise MemoryError(msg)
    raise AwError("awigner error %d: %s" % (code, msg))


def launch_count():
    return int(load().aw_launch_count())


class DeviceArray:
    """A device buffer owned by a propagator handle (the reference's GPUArray).

    ``get()`` copies it to a complex128 NumPy array; ``set()`` / ``[:] =``
    overwrite it; ``__cuda_array_interface__`` lets torch or other CUDA
    libraries view it without a copy (``torch.as_tensor(arr, device="cuda")``).
    """

    def __init__(self, owner, which):
        self._owner = owner
        self._which = which

    def _info(self):
        lib = load()
        ptr = c_vp()
        rows = c_i64()
        cols = c_i64()
        eb = c_int()
        check(lib.aw_buffer(self._owner._h, self._which, ctypes.byref(ptr), ctypes.byref(rows), ctypes.byref(cols),
                            ctypes.byref(eb)))
        return ptr.value, int(rows.value), int(cols.value), int(eb.value)

    @property
    def shape(self):
        _, r, c, _ = self._info()
        return (r, c)

    @property
    def size(self):
        r, c = self.shape
        return r * c

    @property
    def dtype(self):
        return np.dtype(np.complex128 if self._info()[3] == 16 else np.complex64)

    @property
    def ptr(self):
        return self._info()[0]

    def get(self, ary=None):
        """The buffer as a complex128 array: a new one, or `ary` filled in place (a writeable C-contiguous
        complex128 array of the buffer's shape, e.g. in pinned memory), as pycuda's GPUArray.get(ary)."""
        _, r, c, _ = self._info()
        if ary is None:
            out = np.empty((r, c), np.complex128)
        else:
            out = ary
            if (not isinstance(out, np.ndarray) or out.dtype != np.complex128 or out.shape != (r, c) or
                    not out.flags.c_contiguous or not out.flags.writeable):
                raise ValueError("get(ary): ary must be a writeable C-contiguous complex128 array of shape %s" %
                                 ((r, c),))
        check(load().aw_get_buffer(self._owner._h, self._which, out.ctypes.data_as(c_vp), 0))
        return out

    def set(self, value):
        _, r, c, _ = self._info()
        if hasattr(value, "get") and not isinstance(value, np.ndarray):
            value = value.get()
        arr = np.ascontiguousarray(np.broadcast_to(np.asarray(value, dtype=np.complex128), (r, c)))
        check(load().aw_set_buffer(self._owner._h, self._which, arr.ctypes.data_as(c_vp), 0))
        return self

    def fill(self, value):
        v = complex(value)
        check(load().aw_fill_const(self._owner._h, self._which, v.real, v.imag))
        return self

    def copy(self):
        return self.get()

    def __setitem__(self, key, value):
        if key != slice(None):
            raise NotImplementedError("only full assignment rho[:] = ... is supported")
        self.set(value)

    def __array__(self, dtype=None, copy=None):
        a = self.get()
        return a if dtype is None else a.astype(dtype)

    @property
    def __cuda_array_interface__(self):
        ptr, r, c, eb = self._info()
        return {"shape": (r, c), "typestr": "<c16" if eb == 16 else "<c8", "data": (ptr, False), "version": 3}

    def torch(self):
        """Zero-copy torch view (the propagator's stream is synchronised first)."""
        import torch

        check(load().aw_sync(self._owner._h))
        return torch.as_tensor(self, device="cuda")
