"""SchrodingerWignerCUDA1D on GB300: drop-in for schrodinger_wigner_cuda_1d.py:16-902.

A wave function psi(x) propagated by the split-operator method; the Wigner
function is obtained by Wigner transforming psi psi^*.  The reference leaves
the N x N buffer and FFT plans of get_wigner commented out (sw:244, sw:255-256);
here they exist, so get_wigner works as the code intends.
"""
import ctypes

import numpy as np

from . import _lib
from ._common import (ExprInfo, Handle, TermTable, assert_pow2, bind_kwargs, cuda_defines, define_value, mask_mode,
                      precision_code, require)

_c = ctypes


class SchrodingerWignerCUDA1D:
    """
    The second-order split-operator propagator for the Schrodinger equation, with the Wigner function of the
    propagated wave function on demand, on one GB300.

    Keywords (as schrodinger_wigner_cuda_1d.py:28-48): X_gridDIM, X_amplitude, V, K, dt, t, consts, functions,
    diff_V, diff_K, abs_boundary_x, abs_boundary_p.  Extra keyword: precision ('c128' default, or 'c64';
    'c128' runs the one-dimensional passes in native FP64).
    """

    _kind = _lib.AW_SCHRODINGER

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
        kwargs.update(t_initial=self.t)
        self.t = np.float64(self.t)

        # grids (sw:106-122)
        N = self.X_gridDIM
        self.dX = 2.0 * self.X_amplitude / N
        self.X = np.linspace(-self.X_amplitude, self.X_amplitude - self.dX, N)
        self.P = np.fft.fftshift(np.fft.fftfreq(self.X.size, self.dX / (2.0 * np.pi)))
        self.dP = self.P[1] - self.P[0]
        self.X_wigner = self.X / np.sqrt(2.0)
        self.dXX = self.X_wigner[1] - self.X_wigner[0]
        self.P_wigner = self.P / np.sqrt(2.0)
        self.dPP = self.P_wigner[1] - self.P_wigner[0]
        self.wigner_dXdP = self.dX * self.dP

        kwargs.update(dX=self.dX, dP=self.dP, P_max=self.P.max())
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
        self._create(kwargs)
        self.wavefunction = _lib.DeviceArray(self._handle, _lib.AW_BUF_PSI)
        self.wignerfunction = _lib.DeviceArray(self._handle, _lib.AW_BUF_WIGNER)

    def _create(self, kwargs):
        info = ExprInfo(getattr(self, "consts", ""))
        table = TermTable(info)
        self._ehrenfest_slots = None
        if self.isEhrenfest:
            # sw:412-459: <X>, <diff_K>, <P>, -<diff_V>, <V> + <K>
            self._ehrenfest_slots = [
                table.add_slot([("X", 1.0)]),
                table.add_slot([(self.diff_K, 1.0)]),
                table.add_slot([("P", 1.0)]),
                table.add_slot([(self.diff_V, -1.0)]),
                table.add_slot([(self.V, 1.0), (self.K, 1.0)]),
            ]
        self._native_ehrenfest = table.ok
        d = {k: define_value(v) for k, v in kwargs.items() if isinstance(v, (int, float, np.number))}
        cfg = _lib.AwConfig()
        keep = []
        cfg.kind = self._kind
        cfg.precision = precision_code(kwargs)
        cfg.x_grid_dim = int(self.X_gridDIM)
        cfg.p_grid_dim = 1
        cfg.dX, cfg.dP = d["dX"], d["dP"]
        cfg.dXX = cfg.dXX_prime = d["dX"]
        cfg.dPP = cfg.dPP_prime = d["dP"]
        cfg.dt = d["dt"]
        cfg.t_initial = d.get("t_initial", 0.0)
        cfg.dXdP = self.wigner_dXdP
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
        self._n_slots = int(cfg.n_slots)
        self._handle = Handle(cfg)
        self._h = self._handle._h

    @classmethod
    def print_memory_info(cls):
        import torch

        free, total = torch.cuda.mem_get_info()
        print("\n\n\t\tGPU memory Total %.2f GB\n\t\tGPU memory Free %.2f GB\n" % (total / 2.0 ** 30, free / 2.0 ** 30))

    # ------------------------------------------------------------------ state (sw:316-354)
    def _sum_abs2(self):
        psi = self.wavefunction.get()
        return float(np.sum(np.abs(psi) ** 2))

    def set_wavefunction(self, new_wave_func):
        lib = _lib.load()
        if isinstance(new_wave_func, (np.ndarray, _lib.DeviceArray)):
            arr = new_wave_func.get() if isinstance(new_wave_func, _lib.DeviceArray) else new_wave_func
            assert arr.shape == self.wavefunction.shape, "The grid sizes does not match with the wave function"
            self.wavefunction.set(arr.astype(np.complex128))
        elif callable(new_wave_func) and not isinstance(new_wave_func, str):
            self.wavefunction.set(np.broadcast_to(new_wave_func(self, self.X), self.wavefunction.shape))
        elif isinstance(new_wave_func, str):
            _lib.check(lib.aw_fill_expr(self._h, _lib.AW_BUF_PSI, new_wave_func.encode()))
        elif isinstance(new_wave_func, (float, complex, np.floating, np.complexfloating)):
            self.wavefunction.fill(np.complex128(new_wave_func))
        else:
            raise NotImplementedError("new_wave_func must be either function or numpy.array")
        norm = np.sqrt(self._sum_abs2()) * np.sqrt(self.dX)
        _lib.check(lib.aw_scale(self._h, _lib.AW_BUF_PSI, 1.0 / norm, 0.0))
        return self

    # ------------------------------------------------------------------ propagation (sw:356-459)
    def single_step_propagation(self):
        """One split step at the current self.t (sw:356-369); the wave function is not normalised."""
        _lib.check(_lib.load().aw_single_step(self._h, float(self.t)))
        return self.wavefunction

    def get_Ehrenfest(self, t):
        """Append the Ehrenfest observables of the current wave function at time t (sw:412-459)."""
        if not self.isEhrenfest:
            return
        if not self._native_ehrenfest:
            raise NotImplementedError("Ehrenfest observables must be functions of X or of P alone")
        row = np.empty(self._n_slots + 2, np.float64)
        _lib.check(_lib.load().aw_sw_ehrenfest(self._h, float(t), row.ctypes.data_as(_c.POINTER(_c.c_double))))
        s = self._ehrenfest_slots
        self.X_average.append(float(row[s[0]]))
        self.X_average_RHS.append(float(row[s[1]]))
        self.P_average.append(float(row[s[2]]))
        self.P_average_RHS.append(float(row[s[3]]))
        self.hamiltonian_average.append(float(row[s[4]]))

    def propagate(self, steps=1):
        lib = _lib.load()
        steps = max(int(steps), 0)  # the reference loops over xrange(steps): a negative count steps nowhere
        if self.isEhrenfest and not self._native_ehrenfest:
            raise NotImplementedError("Ehrenfest observables must be functions of X or of P alone")
        t = _c.c_double(self.t)
        _lib.check(lib.aw_propagate(self._h, int(steps), _c.byref(t)))
        self.t = np.float64(t.value)
        if self.isEhrenfest:
            rows, cols = _c.c_int64(), _c.c_int32()
            _lib.check(lib.aw_history(self._h, None, 0, _c.byref(rows), _c.byref(cols)))
            out = np.empty((int(rows.value), int(cols.value)))
            if rows.value:
                _lib.check(lib.aw_history(self._h, out.ctypes.data_as(_c.c_void_p), int(rows.value), None, None))
            s = self._ehrenfest_slots
            self.X_average.extend(out[:, s[0]].tolist())
            self.X_average_RHS.extend(out[:, s[1]].tolist())
            self.P_average.extend(out[:, s[2]].tolist())
            self.P_average_RHS.extend(out[:, s[3]].tolist())
            self.hamiltonian_average.extend(out[:, s[4]].tolist())
        return self

    def get_average(self, observable):
        """Sum |psi|^2 f(X, P, t) over the current wave function (sw:392-410)."""
        out = _c.c_double()
        _lib.check(_lib.load().aw_average(self._h, observable.encode(), float(self.t), _c.byref(out)))
        return out.value

    def get_energy(self):
        out = _c.c_double()
        _lib.check(_lib.load().aw_sw_energy(self._h, float(self.t), _c.byref(out)))
        return out.value

    # ------------------------------------------------------------------ imaginary time (sw:484-591)
    def set_ground_state(self, nsteps=10000):
        self.set_wavefunction(1.0)
        _lib.check(_lib.load().aw_sw_imag_steps(self._h, int(nsteps), 0))
        return self

    def get_stationary_states(self, nstates, nsteps=10000):
        lib = _lib.load()
        _lib.check(lib.aw_sw_clear_states(self._h))
        even = True
        for _ in range(nstates):
            if even:
                self.set_wavefunction(1.0)
            else:
                self.set_wavefunction("atan(X)")
            even = not even
            _lib.check(lib.aw_sw_imag_steps(self._h, int(nsteps), 1))
            _lib.check(lib.aw_sw_store_state(self._h))
        self._n_states = nstates
        return self

    def projectout_stationary_states(self, wavefunction):
        """The wave function normalised, with its projections on the stored stationary states removed
        and normalised again (sw:505-550; unweighted scalar products and norms, as there).  Accepts
        a host array or a device array of this package; returns the same kind of object."""
        dev = hasattr(wavefunction, "get") and not isinstance(wavefunction, np.ndarray)
        psi = np.array(wavefunction.get() if dev else wavefunction, dtype=np.complex128)
        psi /= np.linalg.norm(psi)
        states = self.stationary_states
        projs = [np.vdot(phi, psi) for phi in states]
        for phi, c in zip(states, projs):
            psi -= c * phi.reshape(psi.shape)
        psi /= np.linalg.norm(psi)
        if dev:
            wavefunction.set(psi)
            return wavefunction
        return psi

    @property
    def stationary_states(self):
        out = []
        for k in range(getattr(self, "_n_states", 0)):
            psi = np.empty((1, self.X_gridDIM), np.complex128)
            _lib.check(_lib.load().aw_sw_get_state(self._h, k, psi.ctypes.data_as(_c.c_void_p)))
            out.append(psi)
        return out

    # ------------------------------------------------------------------ Wigner function (sw:593-663)
    def get_wigner(self):
        _lib.check(_lib.load().aw_rho2wigner(self._h, 0))
        return self.wignerfunction

    def get_wigner_blackman(self):
        _lib.check(_lib.load().aw_rho2wigner(self._h, 1))
        return self.wignerfunction

    def close(self):
        self._handle.close()
