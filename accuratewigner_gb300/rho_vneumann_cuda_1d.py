"""RhoVNeumannCUDA1D on GB300: drop-in for rho_vneumann_cuda_1d.py:15-822.

The density matrix rho(x, x') on an N x N grid, propagated by the second-order
split-operator method; the Wigner function comes from the padded Wigner
transform of rho.  The arithmetic runs in libawigner.so.
"""
import ctypes

import numpy as np

from . import _lib
from ._common import (apply_batch, ExprInfo, Handle, TermTable, assert_pow2, bind_kwargs, cuda_defines, define_value, mask_mode,
                      precision_code, require)

_c = ctypes


class RhoVNeumannCUDA1D:
    """
    The second-order split-operator propagator for the von Neumann equation for the density matrix rho(x,x',t)
    with the time-dependent Hamiltonian H = K(p, t) + V(x, t), on one GB300.

    Keywords (as rho_vneumann_cuda_1d.py:24-46): X_gridDIM, X_amplitude, V, K, dt, t, consts, functions,
    diff_V, diff_K, abs_boundary_x (function of X), abs_boundary_p (function of P).
    Extra keyword: precision ('c128' default, 'c128-fp64' or 'c64').
    """

    _kind = _lib.AW_RHO_VNEUMANN

    def __init__(self, **kwargs):
        bind_kwargs(self, kwargs)
        require(self, "X_gridDIM", "Coordinate grid size (X_gridDIM) was not specified")
        assert_pow2(self.X_gridDIM, "Coordinate grid size (X_gridDIM) must be a power of two")
        require(self, "X_amplitude", "Coordinate grid range (X_amplitude) was not specified")
        require(self, "V", "Potential energy (V) was not specified")
        require(self, "K", "Momentum dependence (K) was not specified")
        require(self, "dt", "Time-step (dt) was not specified")
        if hasattr(self, "t"):
            del kwargs["t"]
        else:
            print("Warning: Initial time (t) was not specified, thus it is set to zero.")
            self.t = 0.0
        kwargs.update(t_initial=self.t)  # vn:94
        self.t = np.float64(self.t)

        # grids (vn:104-145)
        N = self.X_gridDIM
        self.dX = 2.0 * self.X_amplitude / N
        self.X = np.linspace(-self.X_amplitude, self.X_amplitude - self.dX, N)
        self.P = np.arange(N, dtype=float) - N // 2
        self.P *= 2.0 * np.pi / (N * self.dX)
        self.dP = self.P[1] - self.P[0]
        self.wigner_padding = N // 2
        self.XX_gridDIM = N + 2 * self.wigner_padding
        self.X_wigner = np.arange(self.XX_gridDIM, dtype=float) - self.XX_gridDIM // 2
        self.X_wigner *= self.dX / np.sqrt(2.0)
        self.dX_wigner = self.X_wigner[1] - self.X_wigner[0]
        PP = np.arange(self.XX_gridDIM, dtype=float) - self.XX_gridDIM // 2
        PP *= 2.0 * np.pi / (self.XX_gridDIM * self.dX)
        self.dPP = PP[1] - PP[0]
        self.P_wigner = PP / np.sqrt(2.0)
        self.dP_wigner = self.P_wigner[1] - self.P_wigner[0]
        self.dXdP_wigner = self.dX_wigner * self.dP_wigner
        self.X_wigner = self.X_wigner[np.newaxis, :]
        self.P_wigner = self.P_wigner[:, np.newaxis]

        kwargs.update(dX=self.dX, dP=self.dP, XX_gridDIM=self.XX_gridDIM, dXX=self.dX, dPP=self.dPP,
                      P_max=self.P.max(), X_max=self.X.max())
        self._defines = kwargs
        self.cuda_consts = cuda_defines(kwargs)
        self.cuda_consts += getattr(self, "consts", "")
        if not hasattr(self, "abs_boundary_x"):
            self.abs_boundary_x = "1."
        if not hasattr(self, "abs_boundary_p"):
            self.abs_boundary_p = "1."
        if not hasattr(self, "max_thread_block"):
            self.max_thread_block = 512
        self.cuda_consts += getattr(self, "functions", "")

        self.isEhrenfest = hasattr(self, "diff_K") and hasattr(self, "diff_V")
        if self.isEhrenfest:
            self.X_average = []
            self.P_average = []
            self.X_average_RHS = []
            self.P_average_RHS = []
            self.hamiltonian_average = []
            self.wigner_time = []
        self._create(kwargs)
        self.rho = _lib.DeviceArray(self._handle, _lib.AW_BUF_RHO)
        self.wignerfunction = _lib.DeviceArray(self._handle, _lib.AW_BUF_WIGNER)

    def _slots(self, table):
        self._ehrenfest_slots = None
        if self.isEhrenfest:
            self._ehrenfest_slots = [
                table.add_slot([("X", 1.0)]),
                table.add_slot([(self.diff_K, 1.0)]),
                table.add_slot([("P", 1.0)]),
                table.add_slot([(self.diff_V, -1.0)]),
                table.add_slot([(self.K, 1.0), (self.V, 1.0)]),
            ]

    def _create(self, kwargs):
        info = ExprInfo(getattr(self, "consts", ""))
        table = TermTable(info)
        self._slots(table)
        self._native_ehrenfest = table.ok
        d = {k: define_value(v) for k, v in kwargs.items() if isinstance(v, (int, float, np.number))}
        cfg = _lib.AwConfig()
        keep = []
        cfg.kind = self._kind
        cfg.precision = precision_code(kwargs)
        cfg.x_grid_dim = int(self.X_gridDIM)
        cfg.p_grid_dim = int(self.X_gridDIM)
        cfg.dX, cfg.dP = d["dX"], d["dP"]
        cfg.dXX, cfg.dXX_prime = d["dXX"], d["dXX"]
        cfg.dPP, cfg.dPP_prime = d["dPP"], d["dPP"]
        cfg.dt = d["dt"]
        cfg.t_initial = d.get("t_initial", 0.0)
        cfg.dXdP = self.dXdP_wigner
        for name in ("cuda_consts", "V", "K", "abs_boundary_x", "abs_boundary_p"):
            b = getattr(self, name).encode()
            keep.append(b)
            setattr(cfg, name, b)
        cfg.v_time_dependent = int(info.depends_on(self.V, "t"))
        cfg.k_time_dependent = int(info.depends_on(self.K, "t"))
        cfg.absx_mode = mask_mode(info, self.abs_boundary_x)
        cfg.absp_mode = mask_mode(info, self.abs_boundary_p)
        cfg.ehrenfest = int(bool(self._native_ehrenfest and self.isEhrenfest))
        (table if self._native_ehrenfest else TermTable(info)).fill(cfg, keep)
        self._n_slots = cfg.n_slots
        apply_batch(cfg, kwargs, keep)
        self._handle = Handle(cfg)
        self._h = self._handle._h

    @classmethod
    def print_memory_info(cls):
        import torch

        free, total = torch.cuda.mem_get_info()
        print("\n\n\t\tGPU memory Total %.2f GB\n\t\tGPU memory Free %.2f GB\n" % (total / 2.0 ** 30, free / 2.0 ** 30))

    # ------------------------------------------------------------------ state (vn:348-427)
    def _trace(self):
        re, im = _c.c_double(), _c.c_double()
        _lib.check(_lib.load().aw_trace(self._h, _c.byref(re), _c.byref(im)))
        return complex(re.value, im.value)

    def set_rho(self, new_rho):
        lib = _lib.load()
        if isinstance(new_rho, (np.ndarray, _lib.DeviceArray)):
            arr = new_rho.get() if isinstance(new_rho, _lib.DeviceArray) else new_rho
            assert arr.shape == self.rho.shape, "The grid sizes does not match"
            self.rho.set(arr.astype(np.complex128))
        elif callable(new_rho) and not isinstance(new_rho, str):
            self.rho.set(np.broadcast_to(new_rho(self, self.X[:, np.newaxis], self.X[np.newaxis, :]), self.rho.shape))
        elif isinstance(new_rho, str):
            _lib.check(lib.aw_fill_expr(self._h, _lib.AW_BUF_RHO, new_rho.encode()))
        elif isinstance(new_rho, (float, complex, np.floating, np.complexfloating)):
            self.rho.fill(np.complex128(new_rho))
        else:
            raise NotImplementedError("new_rho must be either function or numpy.array")
        s = self._trace().real * self.dX
        _lib.check(lib.aw_scale(self._h, _lib.AW_BUF_RHO, 1.0 / s, 0.0))
        return self

    def get_wignerfunction(self):
        _lib.check(_lib.load().aw_rho2wigner(self._h, 0))
        return self.wignerfunction

    # ------------------------------------------------------------------ propagation (vn:429-501)
    def _history(self):
        lib = _lib.load()
        rows, cols = _c.c_int64(), _c.c_int32()
        _lib.check(lib.aw_history(self._h, None, 0, _c.byref(rows), _c.byref(cols)))
        n = int(rows.value)
        out = np.empty((n, int(cols.value)), np.float64)
        if n:
            _lib.check(lib.aw_history(self._h, out.ctypes.data_as(_c.c_void_p), n, None, None))
        return out

    def single_step_propagation(self):
        """One split step at the current self.t (vn:450-468); rho is not normalised."""
        _lib.check(_lib.load().aw_single_step(self._h, float(self.t)))
        return self.rho

    def propagate(self, steps=1):
        lib = _lib.load()
        steps = max(int(steps), 0)  # the reference loops over xrange(steps): a negative count steps nowhere
        if self.isEhrenfest and not self._native_ehrenfest:
            for _ in range(steps):
                t = _c.c_double(self.t)
                _lib.check(lib.aw_propagate(self._h, 1, _c.byref(t)))
                self.t = np.float64(t.value)
                self.get_Ehrenfest(self.t)
            return self
        t = _c.c_double(self.t)
        _lib.check(lib.aw_propagate(self._h, int(steps), _c.byref(t)))
        self.t = np.float64(t.value)
        if self.isEhrenfest:
            rows = self._history()
            s = self._ehrenfest_slots
            self.X_average.extend(rows[:, s[0]].tolist())
            self.X_average_RHS.extend(rows[:, s[1]].tolist())
            self.P_average.extend(rows[:, s[2]].tolist())
            self.P_average_RHS.extend(rows[:, s[3]].tolist())
            self.hamiltonian_average.extend(rows[:, s[4]].tolist())
        return self

    def get_Ehrenfest(self, t):
        if self.isEhrenfest:
            self.X_average.append(self.get_average(("X",)))
            self.X_average_RHS.append(self.get_average((None, self.diff_K)))
            self.P_average.append(self.get_average((None, "P")))
            self.P_average_RHS.append(-self.get_average((self.diff_V,)))
            self.hamiltonian_average.append(self.get_average((None, self.K)) + self.get_average((self.V,)))

    # ------------------------------------------------------------------ observables (vn:503-591)
    def get_average(self, observable):
        ops = [o.encode() if o else None for o in observable]
        arr = (_c.c_char_p * max(1, len(ops)))(*ops)
        out = _c.c_double()
        _lib.check(_lib.load().aw_average_ops(self._h, arr, len(ops), float(self.t), _c.byref(out)))
        return out.value

    def get_purity(self):
        out = _c.c_double()
        _lib.check(_lib.load().aw_purity(self._h, _c.byref(out)))
        return out.value

    def get_sigma_x_sigma_p(self):
        return np.sqrt(
            (self.get_average(("X * X",)) - self.get_average(("X",)) ** 2)
            * (self.get_average((None, "P * P")) - self.get_average((None, "P")) ** 2)
        )

    def close(self):
        self._handle.close()
