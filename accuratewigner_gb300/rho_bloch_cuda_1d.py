"""RhoBlochCUDA1D on GB300: drop-in for rho_bloch_cuda_1d.py:10-372.

Gibbs states of rho(x, x') by imaginary-time split-operator propagation of the
Bloch equation (Bondar et al., Phys. Rev. E 93, 063304 (2016)).
"""
import ctypes

import numpy as np

from . import _lib
from .rho_vneumann_cuda_1d import RhoVNeumannCUDA1D
from .wigner_bloch_cuda_1d import _round_half_away

_c = ctypes


class RhoBlochCUDA1D(RhoVNeumannCUDA1D):
    """
    Find the density matrix of the Boltzmann-Gibbs canonical state [rho = exp(-H/kT)]
    by second-order split-operator propagation of the Bloch equation.
    The Hamiltonian should be of the form H = K(p) + V(x).

    Keywords in addition to RhoVNeumannCUDA1D's (rb:20-28): kT, dbeta, t_initial.
    """

    _kind = _lib.AW_RHO_BLOCH

    def __init__(self, **kwargs):
        kwargs = dict(kwargs)
        if "t_initial" not in kwargs:
            kwargs.update(t_initial=0.0)
            print("Warning: Initial time (t_initial) was not specified. So the default value was used t_initial = 0.")
        self.kT = kwargs.pop("kT", 0.0)
        self.dbeta = kwargs.pop("dbeta", 0.01)
        if "dt" not in kwargs:
            kwargs.update(dt=self.dbeta)
        RhoVNeumannCUDA1D.__init__(self, **kwargs)
        vmin, kmin = _c.c_double(), _c.c_double()
        _lib.check(_lib.load().aw_bloch_min(self._h, _c.byref(vmin), _c.byref(kmin)))
        self.V_min, self.K_min = vmin.value, kmin.value
        self.cuda_consts += "#define V_min %.15e\n" % self.V_min
        self.cuda_consts += "#define K_min %.15e\n" % self.K_min

    def _slots(self, table):
        RhoVNeumannCUDA1D._slots(self, table)
        # energy checked by get_ground_state (rb:194)
        self._energy_slot = table.add_slot([(self.K, 1.0), (self.V, 1.0)])

    def get_V_min(self):
        return self.V_min

    def get_K_min(self):
        return self.K_min

    @classmethod
    def get_dbeta_num_beta_steps(cls, kT, dbeta):
        """rb:100-123."""
        if kT > 0:
            num_beta_steps = 1.0 / (kT * dbeta)
            if _round_half_away(num_beta_steps) != num_beta_steps:
                num_beta_steps = _round_half_away(num_beta_steps)
                dbeta = 1.0 / (kT * num_beta_steps)
            num_beta_steps = int(num_beta_steps)
        else:
            num_beta_steps = np.inf
        return dbeta, num_beta_steps

    def get_gibbs_state(self, kT=None, dbeta=None):
        """rb:125-161."""
        if dbeta is None:
            dbeta = self.dbeta
        if kT is None:
            kT = self.kT
        dbeta, num_beta_steps = self.get_dbeta_num_beta_steps(kT, dbeta)
        dbeta = np.float64(dbeta)
        self.set_rho("double(i == j)")
        if not np.isfinite(num_beta_steps):
            raise ValueError("get_gibbs_state needs kT > 0 (use get_ground_state for kT = 0)")
        done, purity = _c.c_int64(), _c.c_double()
        _lib.check(_lib.load().aw_gibbs(self._h, float(dbeta), int(num_beta_steps), _c.byref(done), _c.byref(purity)))
        self.gibbs_steps_done = int(done.value)
        if num_beta_steps > 0 and not purity.value < 1.0:
            k = self.gibbs_steps_done - 1
            print("Warning: Gibbs state calculations interupted because purity = %.10f > 1."
                  "Current kT = %.6f" % (purity.value, 1 / (k * dbeta) if k > 0 else np.inf))
        return self.rho

    def bloch_single_step_propagation(self, dbeta):
        """rb:225-246 (trace normalisation included)."""
        self._last_bloch = np.empty(self._n_slots + 2)
        _lib.check(_lib.load().aw_bloch_step(self._h, float(dbeta), self._last_bloch.ctypes.data_as(_c.c_void_p)))
        return self.rho

    def get_ground_state(self, dbeta=None, abs_tol_purity=1e-12):
        """rb:163-223."""
        lib = _lib.load()
        previous_energy = current_energy = np.inf
        previous_purity = current_purity = 0.0
        if dbeta is None:
            dbeta = self.dbeta
        dbeta = np.float64(dbeta)
        self.set_rho("double(i == j)")
        _lib.check(lib.aw_copy_buffer(self._h, _lib.AW_BUF_RHO, _lib.AW_BUF_SNAPSHOT))
        while current_purity < (1.0 - abs_tol_purity) and dbeta > 1e-12:
            self.bloch_single_step_propagation(dbeta)
            r = self._last_bloch
            try:
                current_purity = r[self._n_slots]
                assert current_purity <= 1.0
                current_energy = r[self._energy_slot]
                assert current_energy < previous_energy
                previous_energy = current_energy
                previous_purity = current_purity
                _lib.check(lib.aw_copy_buffer(self._h, _lib.AW_BUF_RHO, _lib.AW_BUF_SNAPSHOT))
                print("Current energy: %.5f; purity: 1 - %.2e; dbeta: %.2e"
                      % (current_energy, 1 - current_purity, dbeta))
            except AssertionError:
                _lib.check(lib.aw_copy_buffer(self._h, _lib.AW_BUF_SNAPSHOT, _lib.AW_BUF_RHO))
                dbeta *= 0.5
                current_energy = previous_energy
                current_purity = previous_purity
        return self.rho
