"""CPU restatement (NumPy, FP64) of AccurateWigner's split-operator propagators.

TEST INFRASTRUCTURE ONLY.  This module is the oracle: the GPU library never
imports it, and only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` execute it.

It follows the reference's arithmetic line by line, in the reference's op
order, with cuFFT replaced by pocketfft (``scipy.fft``):

* cuFFT forward (sign -1, unnormalised) is ``fft``; cuFFT inverse (sign +1,
  unnormalised) is ``ifft(..., norm="forward")`` (cufft.py:6-7, :226-238).
* ``Plan_Z2Z_2D_Axis0`` transforms columns (axis 0) and ``Plan_Z2Z_2D_Axis1``
  rows (axis 1) of the C-ordered ``[i, j]`` array (cufft.py:274-343).
* Every ``int``/``float`` keyword becomes a ``#define`` and so reaches the
  kernels rounded through ``'%.15e'`` (wigner_moyal_cuda_1d.py:171-176); the
  oracle evaluates its kernels with those rounded values.

Parity status: the reference cannot execute here (Python 2, PyCUDA, a GPU).
Its kernel source is compiled for the CPU by ``oracle/ref_build.py`` and the
golden vectors it produced are committed under ``tests/golden/``; the tests
check this restatement against them.
"""
import math
import os

import numpy as np
import scipy.fft as sfft

from .cexpr import CExpr

WORKERS = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)


# --------------------------------------------------------------------------------------
# cuFFT stand-ins (cufft.py:233-238: in-place Z2Z, unnormalised both ways)
# --------------------------------------------------------------------------------------

def fft0(a):
    return sfft.fft(a, axis=0, workers=WORKERS)


def ifft0(a):
    return sfft.ifft(a, axis=0, norm="forward", workers=WORKERS)


def fft1(a):
    return sfft.fft(a, axis=1, workers=WORKERS)


def ifft1(a):
    return sfft.ifft(a, axis=1, norm="forward", workers=WORKERS)


def define_value(value):
    """The value a kernel sees for a ``#define`` made from ``value``."""
    if isinstance(value, (bool, int, np.integer)):
        return int(value)
    return float("%.15e" % value)


def make_defines(kwargs):
    """wigner_moyal_cuda_1d.py:171-176: ints with %d, floats with %.15e."""
    out = {}
    for name, value in kwargs.items():
        if isinstance(value, (bool, int, np.integer)):
            out[name] = int(value)
        elif isinstance(value, (float, np.floating)):
            out[name] = define_value(value)
    return out


def round_half_away(x):
    """Python 2 ``round`` (used by get_dbeta_num_beta_steps)."""
    return math.floor(x + 0.5) if x >= 0 else -math.floor(-x + 0.5)


def dbeta_num_beta_steps(kT, dbeta):
    """wigner_bloch_cuda_1d.py:94-117 (identical in rho_bloch_cuda_1d.py:100-123)."""
    if kT > 0:
        num = 1.0 / (kT * dbeta)
        if round_half_away(num) != num:
            num = round_half_away(num)
            dbeta = 1.0 / (kT * num)
        num = int(num)
    else:
        num = np.inf
    return dbeta, num


def _is_pow2(n):
    return 2 ** int(np.log2(n)) == n


class _Base:
    _required = ()

    def _store_kwargs(self, kwargs):
        self.py_functions = kwargs.pop("py_functions", None) or {}
        for name, value in kwargs.items():
            setattr(self, name, value)

    def _expr(self, src):
        return CExpr(src, self.defines, self.py_functions)


# ======================================================================================
# Wigner-Moyal (wigner_moyal_cuda_1d.py)
# ======================================================================================

class WignerMoyalOracle(_Base):
    """wigner_moyal_cuda_1d.py:10-828, restated for the CPU."""

    def __init__(self, **kwargs):
        kwargs = dict(kwargs)
        self._store_kwargs(kwargs)
        # wm:52-92 required attributes and power-of-two sizes
        for name, msg in (("X_gridDIM", "Coordinate grid size (X_gridDIM) was not specified"),):
            if not hasattr(self, name):
                raise AttributeError(msg)
        assert _is_pow2(self.X_gridDIM), "Coordinate grid size (X_gridDIM) must be a power of two"
        if not hasattr(self, "P_gridDIM"):
            raise AttributeError("Momentum grid size (P_gridDIM) was not specified")
        assert _is_pow2(self.P_gridDIM), "Momentum grid size (P_gridDIM) must be a power of two"
        for name, msg in (
            ("X_amplitude", "Coordinate grid range (X_amplitude) was not specified"),
            ("P_amplitude", "Momentum grid range (P_amplitude) was not specified"),
            ("V", "Potential energy (V) was not specified"),
            ("K", "Momentum dependence (K) was not specified"),
            ("dt", "Time-step (dt) was not specified"),
        ):
            if not hasattr(self, name):
                raise AttributeError(msg)
        if "t" in kwargs:
            del kwargs["t"]
        else:
            self.t = 0.0
        self.t = np.float64(self.t)

        # wm:110-143 grids
        Nx, Np = self.X_gridDIM, self.P_gridDIM
        self.dX = 2.0 * self.X_amplitude / Nx
        self.dP = 2.0 * self.P_amplitude / Np
        self.dXdP = self.dX * self.dP
        X = np.linspace(-self.X_amplitude, self.X_amplitude - self.dX, Nx)
        P = np.linspace(-self.P_amplitude, self.P_amplitude - self.dP, Np)
        PP_prime = np.sqrt(2.0) * P
        self.dPP_prime = PP_prime[1] - PP_prime[0]
        XX_prime = np.arange(Np, dtype=float) - Np // 2
        XX_prime *= np.pi / (np.sqrt(2.0) * self.P_amplitude)
        self.dXX_prime = XX_prime[1] - XX_prime[0]
        XX = np.sqrt(2.0) * X
        self.dXX = XX[1] - XX[0]
        PP = np.arange(Nx, dtype=float) - Nx // 2
        PP *= np.pi / (np.sqrt(2.0) * self.X_amplitude)
        self.dPP = PP[1] - PP[0]
        self.P = P[:, np.newaxis]
        self.X = X[np.newaxis, :]
        self.XX = XX[np.newaxis, :]
        self.PP = PP[np.newaxis, :]
        self.XX_prime = XX_prime[:, np.newaxis]
        self.PP_prime = PP_prime[:, np.newaxis]

        # wm:151-176 constants
        kwargs.update(
            dX=self.dX, dP=self.dP, dXX=self.dXX, dXX_prime=self.dXX_prime,
            dPP=self.dPP, dPP_prime=self.dPP_prime,
            XX_max=self.XX.max(), XX_prime_max=self.XX_prime.max(),
            PP_max=self.PP.max(), PP_prime_max=self.PP_prime.max(),
        )
        self._kwargs_for_defines = kwargs
        self.defines = make_defines(kwargs)
        if not hasattr(self, "abs_boundary_x"):
            self.abs_boundary_x = "1."
        if not hasattr(self, "abs_boundary_p"):
            self.abs_boundary_p = "1."
        self._setup_exprs()

        self.wignerfunction = np.zeros((Np, Nx), np.complex128)
        self.rho = np.zeros_like(self.wignerfunction)
        self._compiled_observable = {}
        self.hamiltonian = self.K + " + " + self.V if isinstance(self.K, str) else None
        if hasattr(self, "diff_K") and hasattr(self, "diff_V"):
            self.X_average, self.P_average = [], []
            self.X_average_RHS, self.P_average_RHS = [], []
            self.hamiltonian_average = []
            self.isEhrenfest = True
        else:
            self.isEhrenfest = False

    def _setup_exprs(self):
        d = self.defines
        Nx, Np = self.X_gridDIM, self.P_gridDIM
        self.i = np.arange(Np)[:, None]
        self.j = np.arange(Nx)[None, :]
        # kernel-side coordinates (wm:645-646, 662-663, 748-749, 769-770, 797-798)
        self.kPP = d["dPP"] * (self.j - 0.5 * Nx)
        self.kPP_prime = d["dPP_prime"] * (self.i - 0.5 * Np)
        self.kXX = d["dXX"] * (self.j - 0.5 * Nx)
        self.kXX_prime = d["dXX_prime"] * (self.i - 0.5 * Np)
        self.kX = d["dX"] * (self.j - 0.5 * Nx)
        self.kP = d["dP"] * (self.i - 0.5 * Np)
        self._V = self._expr(self.V)
        self._K = self._expr(self.K)
        self._absx = self._expr(self.abs_boundary_x)
        self._absp = self._expr(self.abs_boundary_p)
        self.sign = 1.0 - 2.0 * ((self.i + self.j) % 2)

    # ---------------------------------------------------------------- kernels wm:639-778
    def phase_shearX(self, rho):
        a = np.tan(np.pi / 8.0)
        phase = -a * self.kPP * self.kXX_prime
        rho *= (np.cos(phase) + 1j * np.sin(phase)) / float(self.X_gridDIM)

    def phase_shearY(self, rho):
        b = -np.sin(np.pi / 4.0)
        phase = -b * self.kPP_prime * self.kXX
        rho *= (np.cos(phase) + 1j * np.sin(phase)) / float(self.P_gridDIM)

    def blackmanX(self, rho):
        Cj = self.j * 2.0 * np.pi / (self.X_gridDIM - 1.0)
        rho *= 0.42 - 0.5 * np.cos(Cj) + 0.08 * np.cos(2.0 * Cj)

    def blackmanY(self, rho):
        Ci = self.i * 2.0 * np.pi / (self.P_gridDIM - 1.0)
        rho *= 0.42 - 0.5 * np.cos(Ci) + 0.08 * np.cos(2.0 * Ci)

    def sign_flip(self, rho):
        rho *= 1 - 2 * ((self.i + self.j) % 2)

    def _locals(self, t):
        return dict(i=self.i, j=self.j, t=t, XX=self.kXX, XX_prime=self.kXX_prime,
                    PP=self.kPP, PP_prime=self.kPP_prime)

    def expK(self, rho, t):
        tt = t + 0.5 * self.defines["dt"]
        phase = -self.defines["dt"] * (self._K(P=self.kPP, t=tt) - self._K(P=self.kPP_prime, t=tt))
        rho *= (np.cos(phase) + 1j * np.sin(phase)) * self._absp(**self._locals(t))

    def expV(self, rho, t):
        tt = t + 0.5 * self.defines["dt"]
        phase = -0.5 * self.defines["dt"] * (self._V(X=self.kXX, t=tt) - self._V(X=self.kXX_prime, t=tt))
        rho *= self.sign * (np.cos(phase) + 1j * np.sin(phase)) * self._absx(**self._locals(t))

    # ---------------------------------------------------------------- observables wm:329-366
    def get_average(self, observable):
        f = self._compiled_observable.get(observable)
        if f is None:
            f = self._compiled_observable[observable] = self._expr(observable)
        weighted = self.wignerfunction.real * f(X=self.kX, P=self.kP, t=self.t, i=self.i, j=self.j)
        return np.sum(weighted) * self.dXdP

    def get_purity(self):
        return 2.0 * np.pi * np.sum(self.wignerfunction * self.wignerfunction).real * self.dXdP

    def get_sigma_x_sigma_p(self):
        return np.sqrt(
            (self.get_average("X * X") - self.get_average("X") ** 2)
            * (self.get_average("P * P") - self.get_average("P") ** 2)
        )

    # ---------------------------------------------------------------- state wm:379-501
    def set_wignerfunction(self, new):
        if isinstance(new, np.ndarray):
            assert new.shape == self.wignerfunction.shape, "The grid sizes does not match with the Wigner function"
            self.wignerfunction[:] = new.astype(np.complex128)
        elif callable(new):
            self.wignerfunction[:] = new(self, self.X, self.P)
        elif isinstance(new, str):
            f = self._expr(new)
            self.wignerfunction[:] = f(X=self.kX, P=self.kP, i=self.i, j=self.j)
        elif isinstance(new, (float, complex, np.floating, np.complexfloating)):
            self.wignerfunction.fill(np.complex128(new))
        else:
            raise NotImplementedError("new_wigner_func must be either function or numpy.array")
        self.wignerfunction /= np.sum(self.wignerfunction) * self.dXdP
        self.wigner2rho()
        return self

    def wigner2rho(self):
        rho = self.wignerfunction.copy()
        self.sign_flip(rho)
        rho = fft0(rho)
        rho = ifft1(rho); self.phase_shearX(rho); rho = fft1(rho)
        rho = ifft0(rho); self.phase_shearY(rho); rho = fft0(rho)
        rho = ifft1(rho); self.phase_shearX(rho); rho = fft1(rho)
        self.sign_flip(rho)
        self.rho = rho
        return self.rho

    def rho2wigner_(self):
        W = self.rho.copy()
        self.sign_flip(W)
        W = fft1(W); self.phase_shearX(W); W = ifft1(W)
        W = fft0(W); self.phase_shearY(W); W = ifft0(W)
        W = fft1(W); self.phase_shearX(W); W = ifft1(W)
        W = ifft0(W)
        self.sign_flip(W)
        self.wignerfunction = W
        return W

    def rho2wigner_blackman(self):
        W = self.rho.copy()
        self.sign_flip(W)
        self.blackmanX(W); W = fft1(W); self.phase_shearX(W); W = ifft1(W)
        self.blackmanY(W); W = fft0(W); self.phase_shearY(W); W = ifft0(W)
        self.blackmanX(W); W = fft1(W); self.phase_shearX(W); W = ifft1(W)
        self.blackmanY(W); W = ifft0(W)
        self.sign_flip(W)
        self.wignerfunction = W
        return W

    def rho2wigner(self):
        return self.rho2wigner_()

    # ---------------------------------------------------------------- propagation wm:543-622
    def single_step_propagation(self):
        rho = self.rho
        self.expV(rho, self.t)
        rho = ifft0(rho)
        rho = fft1(rho)
        self.expK(rho, self.t)
        rho = fft0(rho)
        rho = ifft1(rho)
        rho /= rho.shape[0] * rho.shape[1]
        self.expV(rho, self.t)
        self.rho = rho
        return rho

    def propagate(self, steps=1):
        for _ in range(steps):
            self.t += self.dt
            self.single_step_propagation()
            self.get_Ehrenfest(self.t)
        if not self.isEhrenfest:
            self.normalize_rho_wigner()
        return self.wignerfunction

    def get_Ehrenfest(self, t):
        if self.isEhrenfest:
            self.normalize_rho_wigner()
            self.X_average.append(self.get_average("X"))
            self.X_average_RHS.append(self.get_average(self.diff_K))
            self.P_average.append(self.get_average("P"))
            self.P_average_RHS.append(-self.get_average(self.diff_V))
            self.hamiltonian_average.append(self.get_average(self.hamiltonian))

    def normalize_rho_wigner(self):
        self.rho2wigner()
        norm = np.sum(self.wignerfunction).real * self.dXdP
        self.wignerfunction /= norm
        self.rho /= norm
        return self


# ======================================================================================
# Wigner-Bloch (wigner_bloch_cuda_1d.py)
# ======================================================================================

class WignerBlochOracle(WignerMoyalOracle):
    """wigner_bloch_cuda_1d.py:9-366, restated for the CPU."""

    def __init__(self, **kwargs):
        kwargs = dict(kwargs)
        if "t_initial" not in kwargs:
            kwargs.update(t_initial=0.0)
        self.kT = kwargs.pop("kT", 0.0)
        self.dbeta = kwargs.pop("dbeta", 0.01)
        if "dt" not in kwargs:
            kwargs.update(dt=self.dbeta)
        WignerMoyalOracle.__init__(self, **kwargs)
        t0 = self.defines["t_initial"]
        # wb:70-92, fill kernels wb:343-365
        self.V_min = define_value(np.min(self._V(X=self.kXX, t=t0) + self._V(X=self.kXX_prime, t=t0)))
        self.K_min = define_value(np.min(self._K(P=self.kPP, t=t0) + self._K(P=self.kPP_prime, t=t0)))

    # wb:276-316
    def bloch_expK(self, W, dbeta):
        t0 = self.defines["t_initial"]
        phase = -0.5 * dbeta * (self._K(P=self.kPP, t=t0) + self._K(P=self.kPP_prime, t=t0) - self.K_min)
        W *= np.exp(phase)

    def bloch_expV(self, W, dbeta):
        t0 = self.defines["t_initial"]
        phase = -0.25 * dbeta * (self._V(X=self.kXX, t=t0) + self._V(X=self.kXX_prime, t=t0) - self.V_min)
        W *= self.sign * np.exp(phase)

    get_dbeta_num_beta_steps = staticmethod(dbeta_num_beta_steps)

    def bloch_single_step_propagation(self, dbeta):
        rho = self.rho
        self.bloch_expV(rho, dbeta)
        rho = ifft0(rho)
        rho = fft1(rho)
        self.bloch_expK(rho, dbeta)
        rho = fft0(rho)
        rho = ifft1(rho)
        self.bloch_expV(rho, dbeta)
        self.rho = rho
        self.normalize_rho_wigner()

    def get_gibbs_state(self, kT=None, dbeta=None):
        if dbeta is None:
            dbeta = self.dbeta
        if kT is None:
            kT = self.kT
        dbeta, num_beta_steps = self.get_dbeta_num_beta_steps(kT, dbeta)
        dbeta = np.float64(dbeta)
        self.set_wignerfunction(1.0 / np.prod(self.wignerfunction.shape))
        self.gibbs_steps_done = 0
        k = 0
        while k < num_beta_steps:
            self.bloch_single_step_propagation(dbeta)
            self.gibbs_steps_done = k + 1
            if not self.get_purity() < 1.0:
                break
            k += 1
        return self.wignerfunction

    def get_ground_state(self, dbeta=None, abs_tol_purity=1e-12):
        previous_energy = current_energy = np.inf
        previous_purity = current_purity = 0.0
        if dbeta is None:
            dbeta = self.dbeta
        dbeta = np.float64(dbeta)
        self.set_wignerfunction(1.0 / np.prod(self.wignerfunction.shape))
        previous_rho = self.rho.copy()
        while current_purity < (1.0 - abs_tol_purity) and dbeta > 1e-11:
            self.bloch_single_step_propagation(dbeta)
            try:
                current_purity = self.get_purity()
                assert current_purity <= 1.0
                current_energy = self.get_average(self.hamiltonian)
                assert current_energy < previous_energy
                assert self.get_sigma_x_sigma_p() >= 0.5
                previous_energy = current_energy
                previous_purity = current_purity
                previous_rho[:] = self.rho
            except AssertionError:
                self.rho[:] = previous_rho
                dbeta *= 0.5
                current_energy = previous_energy
                current_purity = previous_purity
        self.rho2wigner()
        return self.wignerfunction


# ======================================================================================
# von Neumann (rho_vneumann_cuda_1d.py)
# ======================================================================================

class RhoVNeumannOracle(_Base):
    """rho_vneumann_cuda_1d.py:15-822, restated for the CPU."""

    def __init__(self, **kwargs):
        kwargs = dict(kwargs)
        self._store_kwargs(kwargs)
        if not hasattr(self, "X_gridDIM"):
            raise AttributeError("Coordinate grid size (X_gridDIM) was not specified")
        assert _is_pow2(self.X_gridDIM), "Coordinate grid size (X_gridDIM) must be a power of two"
        for name, msg in (
            ("X_amplitude", "Coordinate grid range (X_amplitude) was not specified"),
            ("V", "Potential energy (V) was not specified"),
            ("K", "Momentum dependence (K) was not specified"),
            ("dt", "Time-step (dt) was not specified"),
        ):
            if not hasattr(self, name):
                raise AttributeError(msg)
        if "t" in kwargs:
            del kwargs["t"]
        else:
            self.t = 0.0
        kwargs.update(t_initial=self.t)  # vn:94 (overrides a caller's t_initial)
        self.t = np.float64(self.t)

        N = self.X_gridDIM
        self.dX = 2.0 * self.X_amplitude / N
        self.X = np.linspace(-self.X_amplitude, self.X_amplitude - self.dX, N)
        self.P = np.arange(N, dtype=float) - N // 2
        self.P *= 2.0 * np.pi / (N * self.dX)
        self.dP = self.P[1] - self.P[0]
        self.wigner_padding = N // 2
        self.XX_gridDIM = N + 2 * self.wigner_padding
        XW = np.arange(self.XX_gridDIM, dtype=float) - self.XX_gridDIM // 2
        XW *= self.dX / np.sqrt(2.0)
        self.dX_wigner = XW[1] - XW[0]
        PP = np.arange(self.XX_gridDIM, dtype=float) - self.XX_gridDIM // 2
        PP *= 2.0 * np.pi / (self.XX_gridDIM * self.dX)
        self.dPP = PP[1] - PP[0]
        PW = PP / np.sqrt(2.0)
        self.dP_wigner = PW[1] - PW[0]
        self.dXdP_wigner = self.dX_wigner * self.dP_wigner
        self.X_wigner = XW[np.newaxis, :]
        self.P_wigner = PW[:, np.newaxis]

        kwargs.update(dX=self.dX, dP=self.dP, XX_gridDIM=self.XX_gridDIM, dXX=self.dX, dPP=self.dPP,
                      P_max=self.P.max(), X_max=self.X.max())
        self._kwargs_for_defines = kwargs
        self.defines = make_defines(kwargs)
        if not hasattr(self, "abs_boundary_x"):
            self.abs_boundary_x = "1."
        if not hasattr(self, "abs_boundary_p"):
            self.abs_boundary_p = "1."

        d = self.defines
        self.i = np.arange(N)[:, None]
        self.j = np.arange(N)[None, :]
        self.kX = d["dX"] * (self.j - 0.5 * N)
        self.kX_prime = d["dX"] * (self.i - 0.5 * N)
        self.kP = d["dP"] * (self.j - 0.5 * N)
        self.kP_prime = d["dP"] * (self.i - 0.5 * N)
        M = self.XX_gridDIM
        self.wi = np.arange(M)[:, None]
        self.wj = np.arange(M)[None, :]
        self._V = self._expr(self.V)
        self._K = self._expr(self.K)
        self._absx = self._expr(self.abs_boundary_x)
        self._absp = self._expr(self.abs_boundary_p)
        self.sign = 1.0 - 2.0 * ((self.i + self.j) % 2)

        self.wignerfunction = np.zeros((M, M), np.complex128)
        self.rho = np.zeros((N, N), np.complex128)
        self._compiled_observable = {}
        if hasattr(self, "diff_K") and hasattr(self, "diff_V"):
            self.X_average, self.P_average = [], []
            self.X_average_RHS, self.P_average_RHS = [], []
            self.hamiltonian_average = []
            self.wigner_time = []
            self.isEhrenfest = True
        else:
            self.isEhrenfest = False

    # kernels vn:608-770
    def phase_shearX(self, W):
        d, M = self.defines, self.XX_gridDIM
        PP = d["dPP"] * (self.wj - 0.5 * M)
        XX_prime = d["dXX"] * (self.wi - 0.5 * M)
        phase = -np.tan(np.pi / 8.0) * PP * XX_prime
        W *= (np.cos(phase) + 1j * np.sin(phase)) / float(M)

    def phase_shearY(self, W):
        d, M = self.defines, self.XX_gridDIM
        XX = d["dXX"] * (self.wj - 0.5 * M)
        PP_prime = d["dPP"] * (self.wi - 0.5 * M)
        phase = np.sin(np.pi / 4.0) * PP_prime * XX
        W *= (np.cos(phase) + 1j * np.sin(phase)) / float(M)

    def sign_flip_rho(self, rho):
        rho *= 1 - 2 * ((self.i + self.j) % 2)

    def sign_flip_wigner(self, W):
        W *= 1 - 2 * ((self.wi + self.wj) % 2)

    def _absp_of(self, P):
        return self._absp(P=P, t=self.t)

    def _absx_of(self, X):
        return self._absx(X=X, t=self.t)

    def expK(self, rho, t):
        dt = self.defines["dt"]
        tt = t + 0.5 * dt
        phase = -dt * (self._K(P=self.kP, t=tt) - self._K(P=self.kP_prime, t=tt))
        rho *= (np.cos(phase) + 1j * np.sin(phase)) * self._absp_of(self.kP) * self._absp_of(self.kP_prime)

    def expV(self, rho, t):
        dt = self.defines["dt"]
        tt = t + 0.5 * dt
        phase = -0.5 * dt * (self._V(X=self.kX, t=tt) - self._V(X=self.kX_prime, t=tt))
        rho *= self.sign * (np.cos(phase) + 1j * np.sin(phase)) * self._absx_of(self.kX) * self._absx_of(self.kX_prime)

    def _trace(self, a):
        return np.trace(a)

    # vn:348-427
    def set_rho(self, new):
        if isinstance(new, np.ndarray):
            assert new.shape == self.rho.shape, "The grid sizes does not match"
            self.rho[:] = new.astype(np.complex128)
        elif callable(new):
            self.rho[:] = new(self, self.X[:, None], self.X[None, :])
        elif isinstance(new, str):
            f = self._expr(new)
            self.rho[:] = f(X=self.kX, X_prime=self.kX_prime, i=self.i, j=self.j)
        elif isinstance(new, (float, complex, np.floating, np.complexfloating)):
            self.rho.fill(np.complex128(new))
        else:
            raise NotImplementedError("new_rho must be either function or numpy.array")
        self.rho /= self._trace(self.rho).real * self.dX
        return self

    def get_wignerfunction(self):
        N, pad = self.X_gridDIM, self.wigner_padding
        W = np.zeros_like(self.wignerfunction)
        W[pad:pad + N, pad:pad + N] = self.rho
        self.sign_flip_wigner(W)
        W = fft1(W); self.phase_shearX(W); W = ifft1(W)
        W = fft0(W); self.phase_shearY(W); W = ifft0(W)
        W = fft1(W); self.phase_shearX(W); W = ifft1(W)
        W = ifft0(W)
        self.sign_flip_wigner(W)
        W /= np.sum(W).real * self.dXdP_wigner
        self.wignerfunction = W
        return W

    # vn:429-468
    def propagate(self, steps=1):
        for _ in range(steps):
            self.t += self.dt
            self.single_step_propagation()
            self.rho /= self._trace(self.rho).real * self.dX
            self.get_Ehrenfest(self.t)
        return self

    def single_step_propagation(self):
        rho = self.rho
        self.expV(rho, self.t)
        rho = ifft0(rho)
        rho = fft1(rho)
        self.expK(rho, self.t)
        rho = fft0(rho)
        rho = ifft1(rho)
        self.expV(rho, self.t)
        self.rho = rho
        return rho

    def get_Ehrenfest(self, t):
        if self.isEhrenfest:
            self.X_average.append(self.get_average(("X",)))
            self.X_average_RHS.append(self.get_average((None, self.diff_K)))
            self.P_average.append(self.get_average((None, "P")))
            self.P_average_RHS.append(-self.get_average((self.diff_V,)))
            self.hamiltonian_average.append(self.get_average((None, self.K)) + self.get_average((self.V,)))

    def _apply_observable(self, tmp, obs):
        f = self._compiled_observable.get(obs)
        if f is None:
            f = self._compiled_observable[obs] = self._expr(obs)
        tmp *= f(X=self.kX, P=self.kP, t=self.t, i=self.i, j=self.j)

    # vn:503-591
    def get_average(self, observable):
        is_x = False
        tmp = self.rho.copy()
        for obs in observable:
            is_x = not is_x
            if obs:
                if is_x:
                    self._apply_observable(tmp, obs)
                else:
                    self.sign_flip_rho(tmp)
                    tmp = fft1(tmp)
                    tmp /= tmp.shape[1]
                    self._apply_observable(tmp, obs)
                    tmp = ifft1(tmp)
                    self.sign_flip_rho(tmp)
        return self._trace(tmp).real * self.dX

    def get_purity(self):
        return np.sum(np.abs(self.rho) ** 2) * self.dX ** 2

    def get_sigma_x_sigma_p(self):
        return np.sqrt(
            (self.get_average(("X * X",)) - self.get_average(("X",)) ** 2)
            * (self.get_average((None, "P * P")) - self.get_average((None, "P")) ** 2)
        )


# ======================================================================================
# rho-Bloch (rho_bloch_cuda_1d.py)
# ======================================================================================

class RhoBlochOracle(RhoVNeumannOracle):
    """rho_bloch_cuda_1d.py:10-372, restated for the CPU."""

    def __init__(self, **kwargs):
        kwargs = dict(kwargs)
        if "t_initial" not in kwargs:
            kwargs.update(t_initial=0.0)
        self.kT = kwargs.pop("kT", 0.0)
        self.dbeta = kwargs.pop("dbeta", 0.01)
        if "dt" not in kwargs:
            kwargs.update(dt=self.dbeta)
        RhoVNeumannOracle.__init__(self, **kwargs)
        t0 = self.defines["t_initial"]
        self.V_min = define_value(np.min(self._V(X=self.kX, t=t0) + self._V(X=self.kX_prime, t=t0)))
        # rb:360-371: fill_K multiplies a zeroed array, so K_min is 0 (or NaN for non-finite K)
        zeros = np.zeros((self.X_gridDIM, self.X_gridDIM))
        with np.errstate(invalid="ignore"):
            kmin = np.min(zeros * (self._K(P=self.kP, t=t0) + self._K(P=self.kP_prime, t=t0)))
        self.K_min = define_value(kmin)

    get_dbeta_num_beta_steps = staticmethod(dbeta_num_beta_steps)

    # rb:276-315
    def bloch_expK(self, rho, dbeta):
        t0 = self.defines["t_initial"]
        phase = -0.5 * dbeta * (self._K(P=self.kP, t=t0) + self._K(P=self.kP_prime, t=t0) - self.K_min)
        rho *= np.exp(phase)

    def bloch_expV(self, rho, dbeta):
        t0 = self.defines["t_initial"]
        phase = -0.25 * dbeta * (self._V(X=self.kX, t=t0) + self._V(X=self.kX_prime, t=t0) - self.V_min)
        rho *= self.sign * np.exp(phase)

    def bloch_single_step_propagation(self, dbeta):
        rho = self.rho
        self.bloch_expV(rho, dbeta)
        rho = ifft0(rho)
        rho = fft1(rho)
        self.bloch_expK(rho, dbeta)
        rho = fft0(rho)
        rho = ifft1(rho)
        self.bloch_expV(rho, dbeta)
        rho /= self._trace(rho) * self.dX  # complex trace (rb:244)
        self.rho = rho
        return rho

    def get_gibbs_state(self, kT=None, dbeta=None):
        if dbeta is None:
            dbeta = self.dbeta
        if kT is None:
            kT = self.kT
        dbeta, num_beta_steps = self.get_dbeta_num_beta_steps(kT, dbeta)
        dbeta = np.float64(dbeta)
        self.set_rho("double(i == j)")
        self.gibbs_steps_done = 0
        k = 0
        while k < num_beta_steps:
            self.bloch_single_step_propagation(dbeta)
            self.gibbs_steps_done = k + 1
            if not self.get_purity() < 1.0:
                break
            k += 1
        return self.rho

    def get_ground_state(self, dbeta=None, abs_tol_purity=1e-12):
        previous_energy = current_energy = np.inf
        previous_purity = current_purity = 0.0
        if dbeta is None:
            dbeta = self.dbeta
        dbeta = np.float64(dbeta)
        self.set_rho("double(i == j)")
        previous_rho = self.rho.copy()
        while current_purity < (1.0 - abs_tol_purity) and dbeta > 1e-12:
            self.bloch_single_step_propagation(dbeta)
            try:
                current_purity = self.get_purity()
                assert current_purity <= 1.0
                current_energy = self.get_average((None, self.K)) + self.get_average((self.V,))
                assert current_energy < previous_energy
                previous_energy = current_energy
                previous_purity = current_purity
                previous_rho[:] = self.rho
            except AssertionError:
                self.rho[:] = previous_rho
                dbeta *= 0.5
                current_energy = previous_energy
                current_purity = previous_purity
        return self.rho


# ======================================================================================
# Schrodinger-Wigner (schrodinger_wigner_cuda_1d.py)
# ======================================================================================

class SchrodingerWignerOracle(_Base):
    """schrodinger_wigner_cuda_1d.py:16-902, restated for the CPU.

    ``get_wigner`` allocates the N x N buffer that the reference leaves
    commented out (sw:244, sw:255-256) and otherwise follows sw:593-625.
    """

    def __init__(self, **kwargs):
        kwargs = dict(kwargs)
        self._store_kwargs(kwargs)
        if not hasattr(self, "X_gridDIM"):
            raise AttributeError("Coordinate grid size (X_gridDIM) was not specified")
        assert _is_pow2(self.X_gridDIM), "Coordinate grid size (X_gridDIM) must be a power of two"
        for name, msg in (
            ("X_amplitude", "Coordinate grid range (X_amplitude) was not specified"),
            ("V", "Potential energy (V) was not specified"),
            ("K", "Momentum dependence (K) was not specified"),
            ("dt", "Time-step (dt) was not specified"),
        ):
            if not hasattr(self, name):
                raise AttributeError(msg)
        if "t" in kwargs:
            del kwargs["t"]
        else:
            self.t = 0.0
        kwargs.update(t_initial=self.t)
        self.t = np.float64(self.t)
        N = self.X_gridDIM
        self.dX = 2.0 * self.X_amplitude / N
        self.X = np.linspace(-self.X_amplitude, self.X_amplitude - self.dX, N)
        self.P = np.fft.fftshift(np.fft.fftfreq(N, self.dX / (2.0 * np.pi)))
        self.dP = self.P[1] - self.P[0]
        self.X_wigner = self.X / np.sqrt(2.0)
        self.dXX = self.X_wigner[1] - self.X_wigner[0]
        self.P_wigner = self.P / np.sqrt(2.0)
        self.dPP = self.P_wigner[1] - self.P_wigner[0]
        self.wigner_dXdP = self.dX * self.dP
        kwargs.update(dX=self.dX, dP=self.dP, P_max=self.P.max())
        self._kwargs_for_defines = kwargs
        self.defines = make_defines(kwargs)
        if not hasattr(self, "abs_boundary_x"):
            self.abs_boundary_x = "1."
        if not hasattr(self, "abs_boundary_p"):
            self.abs_boundary_p = "1."
        d = self.defines
        self.j1 = np.arange(N)
        self.kX1 = d["dX"] * (self.j1 - 0.5 * N)
        self.kP1 = d["dP"] * ((self.j1 + N // 2) % N - 0.5 * N)
        self.i = np.arange(N)[:, None]
        self.j = np.arange(N)[None, :]
        self._V = self._expr(self.V)
        self._K = self._expr(self.K)
        self._absx = self._expr(self.abs_boundary_x)
        self._absp = self._expr(self.abs_boundary_p)
        self.wavefunction = np.zeros((1, N), np.complex128)
        self.wignerfunction = np.zeros((N, N), np.complex128)
        self._compiled_observable = {}
        if hasattr(self, "diff_K") and hasattr(self, "diff_V"):
            self.X_average, self.P_average = [], []
            self.X_average_RHS, self.P_average_RHS = [], []
            self.hamiltonian_average = []
            self.isEhrenfest = True
        else:
            self.isEhrenfest = False

    @staticmethod
    def _norm(a):
        return np.sqrt(np.sum(np.abs(a) ** 2))

    # kernels sw:798-854
    def expK(self, psi, t):
        phase = -self.defines["dt"] * self._K(P=self.kP1, t=t)
        psi *= (np.cos(phase) + 1j * np.sin(phase)) * self._absp(j=self.j1, P=self.kP1, t=t)

    def expV(self, psi, t):
        phase = -0.5 * self.defines["dt"] * self._V(X=self.kX1, t=t)
        psi *= (np.cos(phase) + 1j * np.sin(phase)) * self._absx(j=self.j1, X=self.kX1, t=t)

    def bloch_expK(self, psi):
        phase = -self.defines["dt"] * self._K(P=self.kP1, t=self.defines["t_initial"])
        psi *= np.exp(phase)

    def bloch_expV(self, psi):
        phase = -0.5 * self.defines["dt"] * self._V(X=self.kX1, t=self.defines["t_initial"])
        psi *= np.exp(phase)

    def _fft(self, psi):
        return fft1(psi)

    def _ifft(self, psi):
        return ifft1(psi)

    # sw:316-503
    def set_wavefunction(self, new):
        if isinstance(new, np.ndarray):
            assert new.shape == self.wavefunction.shape, "The grid sizes does not match with the wave function"
            self.wavefunction[:] = new.astype(np.complex128)
        elif callable(new):
            self.wavefunction[:] = new(self, self.X)
        elif isinstance(new, str):
            f = self._expr(new)
            self.wavefunction[0, :] = f(X=self.kX1, j=self.j1)
        elif isinstance(new, (float, complex, np.floating, np.complexfloating)):
            self.wavefunction.fill(np.complex128(new))
        else:
            raise NotImplementedError("new_wave_func must be either function or numpy.array")
        self.wavefunction /= self._norm(self.wavefunction) * np.sqrt(self.dX)
        return self

    def single_step_propagation(self):
        psi = self.wavefunction
        self.expV(psi[0], self.t)
        psi = self._fft(psi)
        self.expK(psi[0], self.t)
        psi = self._ifft(psi)
        self.expV(psi[0], self.t)
        self.wavefunction = psi
        return psi

    def propagate(self, steps=1):
        for _ in range(steps):
            self.t += self.dt
            self.single_step_propagation()
            self.get_Ehrenfest(self.t)
            self.wavefunction /= self._norm(self.wavefunction) * np.sqrt(self.dX)
        return self

    def get_average(self, observable):
        f = self._compiled_observable.get(observable)
        if f is None:
            f = self._compiled_observable[observable] = self._expr(observable)
        w = np.abs(self.wavefunction[0]) ** 2 * f(X=self.kX1, P=self.kP1, t=self.t, j=self.j1)
        return np.sum(w)

    def get_Ehrenfest(self, t):
        if self.isEhrenfest:
            self.wavefunction /= self._norm(self.wavefunction)
            self.X_average.append(self.get_average("X"))
            self.P_average_RHS.append(-self.get_average(self.diff_V))
            self.hamiltonian_average.append(self.get_average(self.V))
            self.wavefunction = self._fft(self.wavefunction)
            self.wavefunction /= self._norm(self.wavefunction)
            self.X_average_RHS.append(self.get_average(self.diff_K))
            self.P_average.append(self.get_average("P"))
            self.hamiltonian_average[-1] += self.get_average(self.K)
            self.wavefunction = self._ifft(self.wavefunction)

    def get_energy(self):
        self.wavefunction /= self._norm(self.wavefunction)
        av_V = self.get_average(self.V)
        self.wavefunction = self._fft(self.wavefunction)
        self.wavefunction /= self._norm(self.wavefunction)
        av_K = self.get_average(self.K)
        self.wavefunction = self._ifft(self.wavefunction)
        return av_V + av_K

    def _bloch_step(self):
        psi = self.wavefunction
        self.bloch_expV(psi[0])
        psi = self._fft(psi)
        self.bloch_expK(psi[0])
        psi = self._ifft(psi)
        self.bloch_expV(psi[0])
        self.wavefunction = psi

    def set_ground_state(self, nsteps=10000):
        self.set_wavefunction(1.0)
        for _ in range(nsteps):
            self._bloch_step()
            self.wavefunction /= self._norm(self.wavefunction) * np.sqrt(self.dX)
        return self

    def projectout_stationary_states(self, wavefunction):
        wavefunction /= self._norm(wavefunction)
        projs = [np.sum(np.conj(psi) * wavefunction) for psi in self.stationary_states]
        for psi, proj in zip(self.stationary_states, projs):
            wavefunction -= proj * psi
        wavefunction /= self._norm(wavefunction)
        return wavefunction

    def get_stationary_states(self, nstates, nsteps=10000):
        self.stationary_states = []
        even = True
        for _ in range(nstates):
            if even:
                self.set_wavefunction(1.0)
            else:
                self.set_wavefunction("atan(X)")
            even = not even
            for _ in range(nsteps):
                self._bloch_step()
                self.projectout_stationary_states(self.wavefunction)
            self.stationary_states.append(self.wavefunction.copy())
        return self

    # sw:680-771
    def _shearX(self, W):
        d, N = self.defines, self.X_gridDIM
        P = d["dP"] * ((self.j + N // 2) % N - 0.5 * N)
        X_prime = d["dX"] * (self.i - 0.5 * N)
        phase = -np.tan(np.pi / 8.0) * P * X_prime
        W *= (np.cos(phase) + 1j * np.sin(phase)) / float(N)

    def _shearY(self, W):
        d, N = self.defines, self.X_gridDIM
        X = d["dX"] * (self.j - 0.5 * N)
        P_prime = d["dP"] * ((self.i + N // 2) % N - 0.5 * N)
        phase = np.sin(np.pi / 4.0) * P_prime * X
        W *= (np.cos(phase) + 1j * np.sin(phase)) / float(N)

    def _sign_flip(self, W):
        W *= 1 - 2 * (self.i % 2)

    def _blackmanX(self, W):
        Cj = self.j * 2.0 * np.pi / (self.X_gridDIM - 1.0)
        W *= 0.42 - 0.5 * np.cos(Cj) + 0.08 * np.cos(2.0 * Cj)

    def _blackmanY(self, W):
        Ci = self.i * 2.0 * np.pi / (self.X_gridDIM - 1.0)
        W *= 0.42 - 0.5 * np.cos(Ci) + 0.08 * np.cos(2.0 * Ci)

    def get_wigner(self, blackman=False):
        psi = self.wavefunction[0]
        W = psi[None, :] * np.conj(psi[:, None])
        if blackman:
            self._blackmanX(W)
        W = fft1(W); self._shearX(W); W = ifft1(W)
        if blackman:
            self._blackmanY(W)
        W = fft0(W); self._shearY(W); W = ifft0(W)
        if blackman:
            self._blackmanX(W)
        W = fft1(W); self._shearX(W); W = ifft1(W)
        if blackman:
            self._blackmanY(W)
        self._sign_flip(W)
        W = ifft0(W)
        self._sign_flip(W)
        W /= np.sum(W).real * self.wigner_dXdP
        self.wignerfunction = W
        return W

    def get_wigner_blackman(self):
        return self.get_wigner(blackman=True)
