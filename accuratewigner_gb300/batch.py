"""Batches of independent propagators stepped together on one GPU.

No reference counterpart: this is the batched form of the reference's
propagators (one launch per pass covers every instance of the batch).  A batch
holds ``n_inst`` instances of one propagator class on one grid; each instance
has its own state, phase tables, per-instance constants (``params``), norm,
stop flag and observable rows, and no instance reads another's data, so an
instance's results do not depend on which others share the batch.

    b = PropagatorBatch(WignerBlochCUDA1D, 64, params=("a", "b"), init="1.",
                        X_gridDIM=512, P_gridDIM=512, X_amplitude=10., P_amplitude=8.,
                        V="a * X * X * X * X - b * X * X", K="0.5 * P * P", dt=0.01, kT=1.)
    b.set_params(k, [a_k, b_k])          # per instance
    b.gibbs(kT=[...], dbeta=0.01)        # per-instance temperature
    w = b.wigner(k)                      # host copy of instance k's Wigner function
"""
import ctypes

import numpy as np

from . import _lib
from .rho_bloch_cuda_1d import RhoBlochCUDA1D
from .rho_vneumann_cuda_1d import RhoVNeumannCUDA1D
from .wigner_bloch_cuda_1d import WignerBlochCUDA1D, _round_half_away
from .wigner_moyal_cuda_1d import WignerMoyalCUDA1D

_c = ctypes


def dbeta_num_beta_steps(kT, dbeta):
    """Step count round(1 / (kT dbeta)) and dbeta re-fit to it (wigner_bloch_cuda_1d.py:94-117)."""
    n = 1.0 / (kT * dbeta)
    if _round_half_away(n) != n:
        n = _round_half_away(n)
        dbeta = 1.0 / (kT * n)
    return float(dbeta), int(n)


class PropagatorBatch:
    """n_inst instances of `cls` (WignerMoyalCUDA1D, WignerBlochCUDA1D, RhoVNeumannCUDA1D or
    RhoBlochCUDA1D) with per-instance constants `params` and initial state `init`
    (W(X, P) for the Wigner classes, rho(X, X_prime) for the density-matrix classes)."""

    def __init__(self, cls, n_inst, params=(), init="", **kwargs):
        if cls not in (WignerMoyalCUDA1D, WignerBlochCUDA1D, RhoVNeumannCUDA1D, RhoBlochCUDA1D):
            raise TypeError("batches exist for the Wigner-Moyal, Wigner-Bloch, von Neumann and rho-Bloch classes")
        self.cls = cls
        self.n_inst = int(n_inst)
        self.params = tuple(params)
        self.rotated = issubclass(cls, WignerMoyalCUDA1D)
        self.prop = cls(**kwargs, n_inst=self.n_inst, batch_params=list(self.params), batch_init=init)
        self._h = self.prop._h
        self.t = np.full(self.n_inst, np.float64(getattr(self.prop, "t", 0.0)))
        self._view = (0, self.n_inst)

    # ------------------------------------------------------------------ instances
    def close(self):
        self.prop._handle.close()

    def set_view(self, first=0, count=None):
        count = self.n_inst - first if count is None else count
        if (first, count) != self._view:
            _lib.check(_lib.load().aw_set_view(self._h, int(first), int(count)))
            self._view = (first, count)

    def set_params(self, inst, values):
        v = np.ascontiguousarray(values, dtype=np.float64)
        assert v.size == len(self.params), "one value per parameter"
        _lib.check(_lib.load().aw_set_params(self._h, int(inst), v.ctypes.data_as(_c.POINTER(_c.c_double))))

    def set_active(self, flags):
        f = np.ascontiguousarray(np.asarray(flags, dtype=bool).astype(np.int32))
        assert f.size == self.n_inst
        _lib.check(_lib.load().aw_set_active(self._h, f.ctypes.data_as(_c.POINTER(_c.c_int32))))

    def init_state(self, first=0, count=None):
        """Evaluate the initial-state expression for instances [first, first + count) and normalise it."""
        self.set_view(first, count)
        _lib.check(_lib.load().aw_init_state(self._h))

    # ------------------------------------------------------------------ stepping
    def propagate(self, steps, first=0, count=None):
        """`steps` real-time steps of every active instance of [first, first + count)."""
        self.set_view(first, count)
        first, count = self._view
        t = _c.c_double(float(self.t[first]))
        _lib.check(_lib.load().aw_propagate(self._h, int(steps), _c.byref(t)))
        self.t[first:first + count] += steps * self.prop.dt
        return self

    def gibbs_steps(self, dbeta, steps, first=0, count=None):
        """`steps` Bloch steps of dbeta[k] on instances first + k; returns (steps done, purity) per instance."""
        self.set_view(first, count)
        first, count = self._view
        db = np.ascontiguousarray(np.broadcast_to(np.asarray(dbeta, dtype=np.float64), (count,)))
        done = np.zeros(count, np.int64)
        pur = np.zeros(count, np.float64)
        _lib.check(_lib.load().aw_gibbs_batch(self._h, db.ctypes.data_as(_c.POINTER(_c.c_double)), int(steps),
                                              done.ctypes.data_as(_c.POINTER(_c.c_int64)),
                                              pur.ctypes.data_as(_c.POINTER(_c.c_double))))
        return done, pur

    def gibbs(self, kT, dbeta=None):
        """Gibbs states of every instance at its own temperature kT[k] (get_gibbs_state,
        wigner_bloch_cuda_1d.py:119-155 / rho_bloch_cuda_1d.py:125-161).

        Instance k runs round(1 / (kT[k] dbeta)) steps of its re-fitted dbeta and stops early once
        its purity reaches 1.  The instances must be ordered by step count (non-decreasing), so
        that the instances still running always form the tail of the batch.
        Returns (steps done, last purity) per instance; self.energy holds the last <H> of each
        Wigner-Bloch instance.
        """
        dbeta = self.prop.dbeta if dbeta is None else dbeta
        kT = np.broadcast_to(np.asarray(kT, dtype=np.float64), (self.n_inst,))
        fit = [dbeta_num_beta_steps(k, dbeta) for k in kT]
        db = np.array([f[0] for f in fit])
        nsteps = np.array([f[1] for f in fit], dtype=np.int64)
        if np.any(np.diff(nsteps) < 0):
            raise ValueError("order the instances by step count (non-decreasing)")
        self.set_active(np.ones(self.n_inst, bool))
        self.init_state()
        done = np.zeros(self.n_inst, np.int64)
        purity = np.zeros(self.n_inst)
        # Wigner-Bloch records <H> every step (first Bloch observable slot)
        h_slot = self.prop._bloch_slots[0] if hasattr(self.prop, "_bloch_slots") else None
        self.energy = np.full(self.n_inst, np.nan)
        running = np.ones(self.n_inst, bool)
        ran_before = 0
        first = 0
        while first < self.n_inst:
            chunk = int(nsteps[first] - ran_before)
            if chunk > 0:
                self.set_active(running)
                d, p = self.gibbs_steps(db[first:], chunk, first)
                for k in range(first, self.n_inst):
                    if not running[k]:
                        continue
                    done[k] += d[k - first]
                    if d[k - first] > 0:
                        purity[k] = p[k - first]
                        if h_slot is not None:
                            self.energy[k] = self.history(k)[d[k - first] - 1, h_slot]
                    if d[k - first] < chunk:
                        running[k] = False  # stopped at purity >= 1
                ran_before = int(nsteps[first])
            while first < self.n_inst and nsteps[first] <= ran_before:
                first += 1
        self.set_active(np.ones(self.n_inst, bool))
        self.set_view(0, self.n_inst)
        self.gibbs_steps_done = done
        return done, purity

    # ------------------------------------------------------------------ results
    def history(self, inst):
        """Observable rows of instance `inst` from the last propagation (n_slots + 2 columns)."""
        lib = _lib.load()
        rows, cols = _c.c_int64(), _c.c_int32()
        _lib.check(lib.aw_history_of(self._h, int(inst), None, 0, _c.byref(rows), _c.byref(cols)))
        out = np.empty((int(rows.value), int(cols.value)), np.float64)
        if rows.value:
            _lib.check(lib.aw_history_of(self._h, int(inst), out.ctypes.data_as(_c.c_void_p), int(rows.value), None,
                                         None))
        return out

    def _buffer(self, which, inst):
        self.set_view(inst, 1)
        lib = _lib.load()
        p, r, c, e = _c.c_void_p(), _c.c_int64(), _c.c_int64(), _c.c_int32()
        _lib.check(lib.aw_buffer(self._h, which, _c.byref(p), _c.byref(r), _c.byref(c), _c.byref(e)))
        out = np.empty((int(r.value), int(c.value)), np.complex128)
        _lib.check(lib.aw_get_buffer(self._h, which, out.ctypes.data_as(_c.c_void_p), 0))
        return out

    def wigner(self, inst):
        """Host copy of instance `inst`'s Wigner function (Wigner classes: the propagated W;
        density-matrix classes: get_wignerfunction of its rho)."""
        if not self.rotated:
            self.set_view(inst, 1)
            _lib.check(_lib.load().aw_rho2wigner(self._h, 0))
        return self._buffer(_lib.AW_BUF_WIGNER, inst)

    def rho(self, inst):
        return self._buffer(_lib.AW_BUF_RHO, inst)

    def set_rho(self, inst, arr):
        self.set_view(inst, 1)
        a = np.ascontiguousarray(arr, dtype=np.complex128)
        _lib.check(_lib.load().aw_set_buffer(self._h, _lib.AW_BUF_RHO, a.ctypes.data_as(_c.c_void_p), 0))

    def purity(self, inst):
        self.set_view(inst, 1)
        out = _c.c_double()
        _lib.check(_lib.load().aw_purity(self._h, _c.byref(out)))
        return out.value


def propagate_group(members, steps):
    """Advance von Neumann propagators of different grid sizes together by `steps` real-time steps.

    `members`: up to 8 RhoVNeumannCUDA1D propagators or PropagatorBatch batches of them (each batch over
    its current view), one arithmetic form, no per-step observables, V and K independent of t.  Members
    of side up to 128 (complex64: 256) step together, every pass of a step one persistent launch over
    all their tiles; larger members run their own step loop on their own streams meanwhile
    (aw_group_propagate).  No counterpart in the reference, which runs one propagator per script.  Each
    member's time advances.
    """
    members = list(members)
    handles = (_c.c_void_p * len(members))()
    times = (_c.c_double * len(members))()
    for k, m in enumerate(members):
        handles[k] = m._h
        if isinstance(m, PropagatorBatch):
            if m.cls is not RhoVNeumannCUDA1D:
                raise TypeError("grouped propagation takes von Neumann propagators")
            times[k] = float(m.t[m._view[0]])
        else:
            times[k] = float(m.t)
    _lib.check(_lib.load().aw_group_propagate(handles, len(members), int(steps), times))
    for k, m in enumerate(members):
        if isinstance(m, PropagatorBatch):
            first, count = m._view
            m.t[first:first + count] += steps * m.prop.dt
        else:
            m.t = np.float64(times[k])
    return members
