"""WignerMoyalCUDA1D on GB300: drop-in for wigner_moyal_cuda_1d.py:10-828.

Same constructor keywords, attributes and methods as the reference; the
arithmetic runs in libawigner.so (fused sm_103a FFT passes, NVRTC-compiled
user expressions).  See ``include/awigner.h`` for the native boundary.
"""
import ctypes

import numpy as np

from . import _lib
from ._common import (apply_batch, ExprInfo, Handle, TermTable, assert_pow2, bind_kwargs, cuda_defines, define_value, mask_mode,
                      precision_code, require)

_c = ctypes


class WignerMoyalCUDA1D:
    """
    The second-order split-operator propagator for the Moyal equation for the Wigner function W(x, p, t)
    with the time-dependent Hamiltonian H = K(p, t) + V(x, t), on one GB300.

    Keywords (as wigner_moyal_cuda_1d.py:19-41): X_gridDIM, X_amplitude, P_gridDIM, P_amplitude, V, K, dt,
    t (optional), consts, functions, diff_V, diff_K, abs_boundary_x, abs_boundary_p (optional).
    Extra keywords of this implementation: precision ('c128' default, 'c128-fp64' or 'c64'),
    extra_observables (tuple of strings recorded every step into self.extra_average).
    """

    _kind = _lib.AW_WIGNER_MOYAL

    def __init__(self, **kwargs):
        bind_kwargs(self, kwargs)
        require(self, "X_gridDIM", "Coordinate grid size (X_gridDIM) was not specified")
        assert_pow2(self.X_gridDIM, "Coordinate grid size (X_gridDIM) must be a power of two")
        require(self, "P_gridDIM", "Momentum grid size (P_gridDIM) was not specified")
        assert_pow2(self.P_gridDIM, "Momentum grid size (P_gridDIM) must be a power of two")
        require(self, "X_amplitude", "Coordinate grid range (X_amplitude) was not specified")
        require(self, "P_amplitude", "Momentum grid range (P_amplitude) was not specified")
        require(self, "V", "Potential energy (V) was not specified")
        require(self, "K", "Momentum dependence (K) was not specified")
        require(self, "dt", "Time-step (dt) was not specified")
        if hasattr(self, "t"):
            del kwargs["t"]
        else:
            print("Warning: Initial time (t) was not specified, thus it is set to zero.")
            self.t = 0.0
        self.t = np.float64(self.t)

        # grids (wm:110-143)
        Nx, Np = self.X_gridDIM, self.P_gridDIM
        self.dX = 2.0 * self.X_amplitude / Nx
        self.dP = 2.0 * self.P_amplitude / Np
        self.dXdP = self.dX * self.dP
        self.X = np.linspace(-self.X_amplitude, self.X_amplitude - self.dX, Nx)
        self.P = np.linspace(-self.P_amplitude, self.P_amplitude - self.dP, Np)
        self.PP_prime = np.sqrt(2.0) * self.P
        self.dPP_prime = self.PP_prime[1] - self.PP_prime[0]
        self.XX_prime = np.arange(Np, dtype=float) - Np // 2
        self.XX_prime *= np.pi / (np.sqrt(2.0) * self.P_amplitude)
        self.dXX_prime = self.XX_prime[1] - self.XX_prime[0]
        self.XX = np.sqrt(2.0) * self.X
        self.dXX = self.XX[1] - self.XX[0]
        self.PP = np.arange(Nx, dtype=float) - Nx // 2
        self.PP *= np.pi / (np.sqrt(2.0) * self.X_amplitude)
        self.dPP = self.PP[1] - self.PP[0]
        self.P = self.P[:, np.newaxis]
        self.X = self.X[np.newaxis, :]
        self.XX = self.XX[np.newaxis, :]
        self.PP = self.PP[np.newaxis, :]
        self.XX_prime = self.XX_prime[:, np.newaxis]
        self.PP_prime = self.PP_prime[:, np.newaxis]

        # constants (wm:151-182)
        kwargs.update(
            dX=self.dX, dP=self.dP, dXX=self.dXX, dXX_prime=self.dXX_prime, dPP=self.dPP,
            dPP_prime=self.dPP_prime, XX_max=self.XX.max(), XX_prime_max=self.XX_prime.max(),
            PP_max=self.PP.max(), PP_prime_max=self.PP_prime.max(),
        )
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

        self.hamiltonian = self.K + " + " + self.V
        self.isEhrenfest = hasattr(self, "diff_K") and hasattr(self, "diff_V")
        if self.isEhrenfest:
            self.X_average = []
            self.P_average = []
            self.X_average_RHS = []
            self.P_average_RHS = []
            self.hamiltonian_average = []
        self.extra_observables = tuple(getattr(self, "extra_observables", ()))
        self.extra_average = [[] for _ in self.extra_observables]

        self._create(kwargs)
        self.wignerfunction = _lib.DeviceArray(self._handle, _lib.AW_BUF_WIGNER)
        self.rho = _lib.DeviceArray(self._handle, _lib.AW_BUF_RHO)

    # ------------------------------------------------------------------ native handle
    def _slots(self, table):
        """Observables recorded every step: Ehrenfest set first (wm:584-606)."""
        self._ehrenfest_slots = None
        if self.isEhrenfest:
            self._ehrenfest_slots = [
                table.add_slot([("X", 1.0)]),
                table.add_slot([(self.diff_K, 1.0)]),
                table.add_slot([("P", 1.0)]),
                table.add_slot([(self.diff_V, -1.0)]),
                table.add_slot([(self.K, 1.0), (self.V, 1.0)]),
            ]
        self._extra_slots = [table.add_slot([(e, 1.0)]) for e in self.extra_observables]

    def _create(self, kwargs):
        info = ExprInfo(getattr(self, "consts", ""))
        self._info = info
        table = TermTable(info)
        self._slots(table)
        self._native_ehrenfest = table.ok
        cfg = _lib.AwConfig()
        keep = []
        d = {k: define_value(v) for k, v in kwargs.items() if isinstance(v, (int, float, np.number))}
        cfg.kind = self._kind
        cfg.precision = precision_code(kwargs)
        cfg.x_grid_dim = int(self.X_gridDIM)
        cfg.p_grid_dim = int(self.P_gridDIM)
        cfg.dX, cfg.dP = d["dX"], d["dP"]
        cfg.dXX, cfg.dXX_prime = d["dXX"], d["dXX_prime"]
        cfg.dPP, cfg.dPP_prime = d["dPP"], d["dPP_prime"]
        cfg.dt = d["dt"]
        cfg.t_initial = d.get("t_initial", 0.0)
        cfg.dXdP = self.dXdP
        for name in ("cuda_consts", "V", "K", "abs_boundary_x", "abs_boundary_p"):
            b = getattr(self, name).encode()
            keep.append(b)
            setattr(cfg, name, b)
        cfg.v_time_dependent = int(info.depends_on(self.V, "t"))
        cfg.k_time_dependent = int(info.depends_on(self.K, "t"))
        cfg.absx_mode = mask_mode(info, self.abs_boundary_x)
        cfg.absp_mode = mask_mode(info, self.abs_boundary_p)
        native = self._native_ehrenfest and (self.isEhrenfest or self.extra_observables)
        cfg.ehrenfest = int(bool(native))
        if self._native_ehrenfest:
            table.fill(cfg, keep)
        else:
            TermTable(info).fill(cfg, keep)
        self._n_slots = cfg.n_slots
        apply_batch(cfg, kwargs, keep)
        self._handle = Handle(cfg)
        self._h = self._handle._h

    @classmethod
    def print_memory_info(cls):
        import torch

        free, total = torch.cuda.mem_get_info()
        print("\n\n\t\tGPU memory Total %.2f GB\n\t\tGPU memory Free %.2f GB\n" % (total / 2.0 ** 30, free / 2.0 ** 30))

    # ------------------------------------------------------------------ observables (wm:329-366)
    def get_average(self, observable):
        out = _c.c_double()
        _lib.check(_lib.load().aw_average(self._h, observable.encode(), float(self.t), _c.byref(out)))
        return out.value

    def get_purity(self):
        out = _c.c_double()
        _lib.check(_lib.load().aw_purity(self._h, _c.byref(out)))
        return out.value

    def get_sigma_x_sigma_p(self):
        return np.sqrt(
            (self.get_average("X * X") - self.get_average("X") ** 2)
            * (self.get_average("P * P") - self.get_average("P") ** 2)
        )

    # ------------------------------------------------------------------ state (wm:379-501)
    def set_wignerfunction(self, new_wigner_func):
        lib = _lib.load()
        if isinstance(new_wigner_func, (np.ndarray, _lib.DeviceArray)) or hasattr(new_wigner_func, "__cuda_array_interface__"):
            arr = new_wigner_func.get() if isinstance(new_wigner_func, _lib.DeviceArray) else np.asarray(
                new_wigner_func.cpu() if hasattr(new_wigner_func, "cpu") else new_wigner_func)
            assert arr.shape == self.wignerfunction.shape, "The grid sizes does not match with the Wigner function"
            self.wignerfunction.set(arr.astype(np.complex128))
        elif callable(new_wigner_func) and not isinstance(new_wigner_func, str):
            self.wignerfunction.set(np.broadcast_to(new_wigner_func(self, self.X, self.P), self.wignerfunction.shape))
        elif isinstance(new_wigner_func, str):
            _lib.check(lib.aw_fill_expr(self._h, _lib.AW_BUF_WIGNER, new_wigner_func.encode()))
        elif isinstance(new_wigner_func, (float, complex, np.floating, np.complexfloating)):
            self.wignerfunction.fill(np.complex128(new_wigner_func))
        else:
            raise NotImplementedError("new_wigner_func must be either function or numpy.array")
        # normalise by the complex sum (wm:415)
        re, im = _c.c_double(), _c.c_double()
        _lib.check(lib.aw_sum(self._h, _lib.AW_BUF_WIGNER, _c.byref(re), _c.byref(im)))
        s = complex(re.value, im.value) * self.dXdP
        inv = 1.0 / s
        _lib.check(lib.aw_scale(self._h, _lib.AW_BUF_WIGNER, inv.real, inv.imag))
        self.wigner2rho()
        return self

    def wigner2rho(self):
        _lib.check(_lib.load().aw_wigner2rho(self._h))
        return self.rho

    def rho2wigner_(self):
        _lib.check(_lib.load().aw_rho2wigner(self._h, 0))
        return self.wignerfunction

    def rho2wigner_blackman(self):
        _lib.check(_lib.load().aw_rho2wigner(self._h, 1))
        return self.wignerfunction

    def rho2wigner(self):
        return self.rho2wigner_()

    def normalize_rho_wigner(self):
        _lib.check(_lib.load().aw_normalize_rho_wigner(self._h))
        return self

    # ------------------------------------------------------------------ propagation (wm:543-606)
    def _history(self):
        lib = _lib.load()
        rows, cols = _c.c_int64(), _c.c_int32()
        _lib.check(lib.aw_history(self._h, None, 0, _c.byref(rows), _c.byref(cols)))
        n = int(rows.value)
        if n == 0:
            return np.zeros((0, int(cols.value)))
        out = np.empty((n, int(cols.value)), np.float64)
        _lib.check(lib.aw_history(self._h, out.ctypes.data_as(_c.c_void_p), n, None, None))
        return out

    def _record(self, rows):
        if self._ehrenfest_slots is not None:
            s = self._ehrenfest_slots
            self.X_average.extend(rows[:, s[0]].tolist())
            self.X_average_RHS.extend(rows[:, s[1]].tolist())
            self.P_average.extend(rows[:, s[2]].tolist())
            self.P_average_RHS.extend(rows[:, s[3]].tolist())
            self.hamiltonian_average.extend(rows[:, s[4]].tolist())
        for lst, slot in zip(self.extra_average, self._extra_slots):
            lst.extend(rows[:, slot].tolist())

    def single_step_propagation(self):
        """One split step at the current self.t (wm:543-561); rho is not normalised and W is not
        updated."""
        _lib.check(_lib.load().aw_single_step(self._h, float(self.t)))
        return self.rho

    def propagate(self, steps=1):
        lib = _lib.load()
        steps = max(int(steps), 0)  # the reference loops over xrange(steps): a negative count steps nowhere
        if (self.isEhrenfest or self.extra_observables) and not self._native_ehrenfest:
            # an observable mixes X and P: step and average one at a time, as the reference does
            for _ in range(steps):
                t = _c.c_double(self.t)
                # one step, then normalize_rho_wigner (the native call ends with it)
                _lib.check(lib.aw_propagate(self._h, 1, _c.byref(t)))
                self.t = np.float64(t.value)
                self._averages_now()
            if steps == 0 and not self.isEhrenfest:
                self.normalize_rho_wigner()
            return self.wignerfunction
        t = _c.c_double(self.t)
        _lib.check(lib.aw_propagate(self._h, int(steps), _c.byref(t)))
        self.t = np.float64(t.value)
        if self.isEhrenfest or self.extra_observables:
            self._record(self._history())
        return self.wignerfunction

    def get_Ehrenfest(self, t):
        if self.isEhrenfest:
            self.normalize_rho_wigner()
        self._averages_now()

    def _averages_now(self):
        if self.isEhrenfest:
            self.X_average.append(self.get_average("X"))
            self.X_average_RHS.append(self.get_average(self.diff_K))
            self.P_average.append(self.get_average("P"))
            self.P_average_RHS.append(-self.get_average(self.diff_V))
            self.hamiltonian_average.append(self.get_average(self.hamiltonian))
        for lst, e in zip(self.extra_average, self.extra_observables):
            lst.append(self.get_average(e))

    def close(self):
        """Release the device buffers now (they are also released when the object is collected)."""
        self._handle.close()
