"""The oracle with its kernel arithmetic taken from the reference's own CUDA-C.

TEST INFRASTRUCTURE ONLY (golden-vector generation, tests/golden/make_golden.py).

Each class below is the corresponding oracle class of oracle/propagators.py
(which restates the reference's Python-level control flow) with every kernel
call -- phase multiplies, shears, sign flips, Blackman windows, initial
conditions, observables, Bloch exponentials, V_min / K_min fills -- replaced
by the reference's own kernel source, compiled for the CPU by
oracle/ref_build.py.  cuFFT is replaced by pocketfft, as in the oracle.
"""
import numpy as np

from . import ref_build
from .propagators import (RhoBlochOracle, RhoVNeumannOracle, SchrodingerWignerOracle, WignerBlochOracle,
                          WignerMoyalOracle, define_value)

WM = "wigner_moyal_cuda_1d.py"
WB = "wigner_bloch_cuda_1d.py"
VN = "rho_vneumann_cuda_1d.py"
RB = "rho_bloch_cuda_1d.py"
SW = "schrodinger_wigner_cuda_1d.py"


def _consts(obj):
    """cuda_consts exactly as the reference assembles it (wm:169-182, wm:233-237)."""
    out = ""
    for name, value in obj._kwargs_for_defines.items():
        if isinstance(value, (bool, int, np.integer)):
            out += "#define %s %d\n" % (name, int(value))
        elif isinstance(value, (float, np.floating)):
            out += "#define %s %.15e\n" % (name, value)
    out += getattr(obj, "consts", "")
    out += getattr(obj, "functions", "")
    return out


def _c(a):
    return np.ascontiguousarray(a)


class _RotatedKernels:
    """Kernel calls of wigner_moyal_cuda_1d.py (and the Bloch kernels of wigner_bloch_cuda_1d.py)."""

    def _ref_setup(self):
        self.cuda_consts = _consts(self)
        self._mod = ref_build.RefModule(ref_build.template(WM, "wigner_cuda_source").format(
            cuda_consts=self.cuda_consts, K=self.K, V=self.V,
            abs_boundary_x=self.abs_boundary_x, abs_boundary_p=self.abs_boundary_p))
        self._grid = (1, self.P_gridDIM)
        self._obs_mods = {}

    def _run(self, name, arr, *args):
        self._mod.call(name, self._grid, self.X_gridDIM, arr, *args)

    def phase_shearX(self, rho):
        self._run("phase_shearX", rho)

    def phase_shearY(self, rho):
        self._run("phase_shearY", rho)

    def blackmanX(self, rho):
        self._run("blackmanX", rho)

    def blackmanY(self, rho):
        self._run("blackmanY", rho)

    def sign_flip(self, rho):
        self._run("sign_flip", rho)

    def expK(self, rho, t):
        self._run("expK", rho, t)

    def expV(self, rho, t):
        self._run("expV", rho, t)

    def get_average(self, observable):
        mod = self._obs_mods.get(observable)
        if mod is None:
            mod = self._obs_mods[observable] = ref_build.RefModule(
                ref_build.template(WM, "weighted_func_cuda_code").format(cuda_consts=self.cuda_consts, func=observable))
        weighted = np.zeros(self.wignerfunction.shape)
        W = _c(self.wignerfunction)
        mod.call("Kernel", self._grid, self.X_gridDIM, W, weighted, float(self.t))
        return np.sum(weighted) * self.dXdP

    def set_wignerfunction(self, new):
        if isinstance(new, str):
            mod = ref_build.RefModule(ref_build.template(WM, "init_wigner_cuda_source").format(
                cuda_consts=self.cuda_consts, new_wigner_func=new))
            W = np.zeros((self.P_gridDIM, self.X_gridDIM), np.complex128)
            mod.call("Kernel", self._grid, self.X_gridDIM, W)
            new = W
        return WignerMoyalOracle.set_wignerfunction(self, new)


class RefWignerMoyal(_RotatedKernels, WignerMoyalOracle):
    def __init__(self, **kwargs):
        WignerMoyalOracle.__init__(self, **kwargs)
        self._ref_setup()


class RefWignerBloch(_RotatedKernels, WignerBlochOracle):
    def __init__(self, **kwargs):
        WignerBlochOracle.__init__(self, **kwargs)
        self._ref_setup()
        # wb:70-92: fill kernels, then the minima become #defines (wb:55-56)
        fill = ref_build.RefModule(ref_build.template(WB, "fill_V_K").format(
            cuda_consts=self.cuda_consts, K=self.K, V=self.V))
        tmp = np.zeros((self.P_gridDIM, self.X_gridDIM))
        fill.call("fill_V", self._grid, self.X_gridDIM, tmp)
        self.V_min = define_value(tmp.min())
        tmp = np.zeros((self.P_gridDIM, self.X_gridDIM))
        fill.call("fill_K", self._grid, self.X_gridDIM, tmp)
        self.K_min = define_value(tmp.min())
        consts = self.cuda_consts + "#define V_min %.15e \n" % self.V_min + "#define K_min %.15e \n" % self.K_min
        self._bloch = ref_build.RefModule(ref_build.template(WB, "bloch_cuda_source").format(
            cuda_consts=consts, K=self.K, V=self.V,
            abs_boundary_p=self.abs_boundary_p, abs_boundary_x=self.abs_boundary_x))

    def bloch_expK(self, W, dbeta):
        self._bloch.call("bloch_expK", self._grid, self.X_gridDIM, W, dbeta)

    def bloch_expV(self, W, dbeta):
        self._bloch.call("bloch_expV", self._grid, self.X_gridDIM, W, dbeta)


class _RhoKernels:
    """Kernel calls of rho_vneumann_cuda_1d.py."""

    def _ref_setup(self):
        self.cuda_consts = _consts(self)
        self._mod = ref_build.RefModule(ref_build.template(VN, "wigner_cuda_source").format(
            cuda_consts=self.cuda_consts, K=self.K, V=self.V,
            abs_boundary_x=self.abs_boundary_x, abs_boundary_p=self.abs_boundary_p))
        self._obs_mods = {}

    def _rho(self, name, arr, *args):
        self._mod.call(name, (1, self.X_gridDIM), self.X_gridDIM, arr, *args)

    def _wig(self, name, arr, *args):
        self._mod.call(name, (1, self.XX_gridDIM), self.XX_gridDIM, arr, *args)

    def phase_shearX(self, W):
        self._wig("phase_shearX", W)

    def phase_shearY(self, W):
        self._wig("phase_shearY", W)

    def sign_flip_rho(self, rho):
        self._rho("sign_flip_rho", rho)

    def sign_flip_wigner(self, W):
        self._wig("sign_flip_wigner", W)

    def expK(self, rho, t):
        self._rho("expK", rho, t)

    def expV(self, rho, t):
        self._rho("expV", rho, t)

    def _apply_observable(self, tmp, obs):
        mod = self._obs_mods.get(obs)
        if mod is None:
            mod = self._obs_mods[obs] = ref_build.RefModule(ref_build.template(VN, "apply_observable_rho_cuda_source")
                                                            .format(cuda_consts=self.cuda_consts, observable=obs))
        mod.call("Kernel", (1, self.X_gridDIM), self.X_gridDIM, tmp, float(self.t))

    def set_rho(self, new):
        if isinstance(new, str):
            mod = ref_build.RefModule(ref_build.template(VN, "init_rho_source").format(
                cuda_consts=self.cuda_consts, new_rho_func=new))
            rho = np.zeros((self.X_gridDIM, self.X_gridDIM), np.complex128)
            mod.call("Kernel", (1, self.X_gridDIM), self.X_gridDIM, rho)
            new = rho
        return RhoVNeumannOracle.set_rho(self, new)


class RefRhoVNeumann(_RhoKernels, RhoVNeumannOracle):
    def __init__(self, **kwargs):
        RhoVNeumannOracle.__init__(self, **kwargs)
        self._ref_setup()


class RefRhoBloch(_RhoKernels, RhoBlochOracle):
    def __init__(self, **kwargs):
        RhoBlochOracle.__init__(self, **kwargs)
        self._ref_setup()
        # rb:70-98 (fill_K multiplies its zeroed array, rb:370)
        fill = ref_build.RefModule(ref_build.template(RB, "fill_V_K").format(
            cuda_consts=self.cuda_consts, K=self.K, V=self.V))
        N = self.X_gridDIM
        tmp = np.zeros((N, N))
        fill.call("fill_V", (1, N), N, tmp)
        self.V_min = define_value(tmp.min())
        tmp = np.zeros((N, N))
        fill.call("fill_K", (1, N), N, tmp)
        self.K_min = define_value(tmp.min())
        consts = self.cuda_consts + "#define V_min %.15e\n" % self.V_min + "#define K_min %.15e\n" % self.K_min
        self._bloch = ref_build.RefModule(ref_build.template(RB, "bloch_expK_expV_cuda_source").format(
            cuda_consts=consts, K=self.K, V=self.V))

    def bloch_expK(self, rho, dbeta):
        self._bloch.call("bloch_expK", (1, self.X_gridDIM), self.X_gridDIM, rho, dbeta)

    def bloch_expV(self, rho, dbeta):
        self._bloch.call("bloch_expV", (1, self.X_gridDIM), self.X_gridDIM, rho, dbeta)


class RefSchrodingerWigner(SchrodingerWignerOracle):
    """Kernel calls of schrodinger_wigner_cuda_1d.py."""

    def __init__(self, **kwargs):
        SchrodingerWignerOracle.__init__(self, **kwargs)
        self.cuda_consts = _consts(self)
        self._mod = ref_build.RefModule(ref_build.template(SW, "schrodinger_wigner_cuda_source").format(
            cuda_consts=self.cuda_consts, K=self.K, V=self.V,
            abs_boundary_x=self.abs_boundary_x, abs_boundary_p=self.abs_boundary_p))
        self._obs_mods = {}

    def _psi(self, name, psi, *args):
        self._mod.call(name, (1, 1), self.X_gridDIM, psi, *args)

    def _w(self, name, W, *args):
        self._mod.call(name, (1, self.X_gridDIM), self.X_gridDIM, W, *args)

    def expK(self, psi, t):
        self._psi("expK", psi, t)

    def expV(self, psi, t):
        self._psi("expV", psi, t)

    def bloch_expK(self, psi):
        self._psi("bloch_expK", psi)

    def bloch_expV(self, psi):
        self._psi("bloch_expV", psi)

    def _shearX(self, W):
        self._w("phase_shearX", W)

    def _shearY(self, W):
        self._w("phase_shearY", W)

    def _sign_flip(self, W):
        self._w("sign_flip", W)

    def _blackmanX(self, W):
        self._w("blackmanX", W)

    def _blackmanY(self, W):
        self._w("blackmanY", W)

    def get_average(self, observable):
        mod = self._obs_mods.get(observable)
        if mod is None:
            mod = self._obs_mods[observable] = ref_build.RefModule(
                ref_build.template(SW, "weighted_func_cuda_code").format(cuda_consts=self.cuda_consts, func=observable))
        weighted = np.zeros(self.X_gridDIM)
        psi = _c(self.wavefunction[0])
        mod.call("Kernel", (1, 1), self.X_gridDIM, psi, weighted, float(self.t))
        return np.sum(weighted)

    def set_wavefunction(self, new):
        if isinstance(new, str):
            mod = ref_build.RefModule(ref_build.template(SW, "init_wavefunction_cuda_source").format(
                cuda_consts=self.cuda_consts, new_wave_func=new))
            psi = np.zeros((1, self.X_gridDIM), np.complex128)
            mod.call("Kernel", (1, 1), self.X_gridDIM, psi)
            new = psi
        return SchrodingerWignerOracle.set_wavefunction(self, new)

    def get_wigner(self, blackman=False):
        psi = _c(self.wavefunction[0])
        W = np.zeros((self.X_gridDIM, self.X_gridDIM), np.complex128)
        self._mod.call("psi2rho", (1, self.X_gridDIM), self.X_gridDIM, psi, W)
        return self._wigner_from(W, blackman)

    def _wigner_from(self, W, blackman):
        from .propagators import fft0, fft1, ifft0, ifft1

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
