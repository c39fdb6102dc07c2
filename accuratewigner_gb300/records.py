"""On-disk records of a propagation run: ground-state cache, frames, Ehrenfest series.

Counterpart of the file output of strong_field_physics_cuda_1d.py (the driver
of the strong-field workflow: a Bloch ground state, then a driven run):

* the ground-state cache (sfp:202-214, a pickle of rho) is an ``.npz`` holding
  rho and a fingerprint of the grid and Hamiltonian;
* the HDF5 file's groups (sfp:113-125, :247-257, :368-373) become a directory:

      settings.npz      every number, string or array among the run parameters,
                        X_wigner, P_wigner                     (group "settings")
      frames/<n>.npz    wigner (real part of W), t, prob (diagonal of rho)
                                                               (group "frames/<n>")
      ehrenfest.npz     X_average, P_average, X_average_RHS, P_average_RHS,
                        hamiltonian_average                    (group "ehrenfest")

  (h5py is not part of this environment; the names and contents are those of
  the reference's groups);
* the high-harmonic spectrum of <p> (sfp:336-351).

Frames are written without stalling the propagation: ``save_frame`` copies W
and rho device-to-device into a staging slot (ordered on the propagator's
stream), a side stream moves the slot to pinned host memory, and a writer
thread saves the file, while the caller's next ``propagate`` already runs.
Two slots are in flight at most; a third frame waits for the oldest write.
"""
import ctypes
import hashlib
import os
import queue
import threading

import numpy as np

from . import _lib

_c = ctypes

EHRENFEST_NAMES = ("X_average", "P_average", "X_average_RHS", "P_average_RHS", "hamiltonian_average")


# ---------------------------------------------------------------------------- ground-state cache
def fingerprint(prop):
    """Grid sizes, amplitudes, time step, expressions and #define constants of a propagator."""
    parts = []
    for name in ("X_gridDIM", "P_gridDIM", "X_amplitude", "P_amplitude", "dt", "K", "V", "abs_boundary_x",
                 "abs_boundary_p", "functions"):
        parts.append("%s=%r" % (name, getattr(prop, name, None)))
    parts.append(getattr(prop, "cuda_consts", ""))
    return hashlib.sha256("\n".join(parts).encode()).hexdigest()


def ground_state(prop, path, abs_tol_purity=1e-10):
    """The ground state of `prop` (a Wigner-Bloch propagator) from the cache file at `path`, or
    computed by get_ground_state and stored there (sfp:202-214).

    The reference reuses whatever pickle it finds; here a cache made for another grid or
    Hamiltonian (fingerprint mismatch) is recomputed and replaced.  After a load W is recomputed
    from rho, so that wignerfunction matches the loaded state."""
    key = fingerprint(prop)
    try:
        with np.load(path) as f:
            if str(f["fingerprint"]) != key:
                raise ValueError("cache made for another propagator")
            prop.rho.set(f["rho"])
        prop.rho2wigner()
        return "loaded"
    except (OSError, KeyError, ValueError):
        prop.get_ground_state(abs_tol_purity=abs_tol_purity)
        tmp = path + ".tmp.npz"
        np.savez(tmp, rho=prop.rho.get(), fingerprint=np.array(key))
        os.replace(tmp, path)
        return "computed"


# ---------------------------------------------------------------------------- run directory
def _storable(value):
    """The HDF5 writes of sfp:115-119 keep numbers, strings and arrays and skip the rest."""
    if callable(value):
        return None
    try:
        a = np.asarray(value)
    except Exception:
        return None
    return a if a.dtype.kind in "biufcU" else None


class _Slot:
    def __init__(self, torch, rows, cols, diag):
        self.dev_w = torch.empty((rows, cols), dtype=torch.complex128, device="cuda")
        self.dev_rho = torch.empty((rows, cols), dtype=torch.complex128, device="cuda")
        self.host_w = torch.empty((rows, cols), dtype=torch.float64, pin_memory=True)
        self.host_prob = torch.empty(diag, dtype=torch.complex128, pin_memory=True)
        self.free = threading.Event()
        self.free.set()


class RunRecord:
    """Directory record of one run of a Wigner-Moyal / Wigner-Bloch propagator.

        with RunRecord("run_dir", prop, sys_params) as rec:
            for _ in range(num_frames):
                prop.propagate(100)
                rec.save_frame(prop)
        # ehrenfest.npz is written on exit from prop's observable lists
    """

    def __init__(self, path, prop, params=None):
        import torch

        self.path = path
        self.prop = prop
        os.makedirs(os.path.join(path, "frames"), exist_ok=True)
        settings = {}
        for key, val in (params or {}).items():
            a = _storable(val)
            if a is not None:
                settings[key] = a
        settings["X_wigner"] = np.asarray(prop.X)
        settings["P_wigner"] = np.asarray(prop.P)
        np.savez(os.path.join(path, "settings.npz"), **settings)
        self.frame_num = 0
        self._torch = torch
        rows, cols = prop.wignerfunction.shape
        self._slots = [_Slot(torch, rows, cols, min(rows, cols)) for _ in range(2)]
        self._next = 0
        self._copy = torch.cuda.Stream()
        self._queue = queue.Queue()
        self._error = None
        self._writer = threading.Thread(target=self._write_loop, daemon=True)
        self._writer.start()

    # frames -----------------------------------------------------------------
    def save_frame(self, prop=None):
        """Record W (real part), t and the diagonal of rho of the propagator's current state as
        frame `frame_num` (sfp:243-257); returns at once, the file appears when its write ends."""
        prop = prop or self.prop
        if self._error:
            raise self._error
        slot = self._slots[self._next]
        self._next = (self._next + 1) % len(self._slots)
        slot.free.wait()
        slot.free.clear()
        lib = _lib.load()
        # device-to-device into the slot; these calls return after the handle's stream has drained
        _lib.check(lib.aw_get_buffer(prop._h, _lib.AW_BUF_WIGNER, _c.c_void_p(slot.dev_w.data_ptr()), 1))
        _lib.check(lib.aw_get_buffer(prop._h, _lib.AW_BUF_RHO, _c.c_void_p(slot.dev_rho.data_ptr()), 1))
        torch = self._torch
        with torch.cuda.stream(self._copy):
            slot.host_w.copy_(slot.dev_w.real, non_blocking=True)
            slot.host_prob.copy_(torch.diagonal(slot.dev_rho), non_blocking=True)
            done = torch.cuda.Event()
            done.record(self._copy)
        self._queue.put((self.frame_num, float(prop.t), slot, done))
        self.frame_num += 1

    def _write_loop(self):
        while True:
            item = self._queue.get()
            if item is None:
                return
            n, t, slot, done = item
            try:
                done.synchronize()
                tmp = os.path.join(self.path, "frames", "%d.tmp.npz" % n)
                np.savez(tmp, wigner=slot.host_w.numpy(), t=np.float64(t), prob=slot.host_prob.numpy())
                os.replace(tmp, os.path.join(self.path, "frames", "%d.npz" % n))
            except Exception as e:  # surfaced by the next save_frame / close
                self._error = e
            finally:
                slot.free.set()

    # end of run --------------------------------------------------------------
    def close(self):
        """Wait for the frames in flight and write the Ehrenfest series (sfp:368-373)."""
        if self._writer is None:
            return
        self._queue.put(None)
        self._writer.join()
        self._writer = None
        series = {k: np.asarray(getattr(self.prop, k)) for k in EHRENFEST_NAMES if hasattr(self.prop, k)}
        np.savez(os.path.join(self.path, "ehrenfest.npz"), **series)
        if self._error:
            raise self._error

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def read_record(path):
    """The record as nested dicts: {"settings": {...}, "frames": {n: {...}}, "ehrenfest": {...}}."""
    def load(p):
        with np.load(p) as f:
            return {k: f[k] for k in f.files}

    out = {"settings": load(os.path.join(path, "settings.npz")), "frames": {}}
    fdir = os.path.join(path, "frames")
    for name in os.listdir(fdir):
        if name.endswith(".npz") and not name.endswith(".tmp.npz"):
            out["frames"][int(name[:-4])] = load(os.path.join(fdir, name))
    e = os.path.join(path, "ehrenfest.npz")
    if os.path.exists(e):
        out["ehrenfest"] = load(e)
    return out


# ---------------------------------------------------------------------------- analysis
def hhg_spectrum(p_average, dt, omega):
    """High-harmonic spectrum of <p>(t) (sfp:336-351): |FFT(blackman * <p>)|^2, centred and
    normalised to its maximum, against frequency in units of the laser frequency omega."""
    j = np.asarray(p_average, dtype=np.float64)
    n = j.size
    spectrum = np.abs(np.fft.fftshift(np.fft.fft(np.blackman(n) * j))) ** 2
    omegas = np.fft.fftshift(np.fft.fftfreq(n, dt / (2 * np.pi))) / omega
    return omegas, spectrum / spectrum.max()
