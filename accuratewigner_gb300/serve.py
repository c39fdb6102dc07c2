"""A request loop that serves Wigner-Moyal, von Neumann and rho-Bloch (Gibbs-state) requests on
one GPU with continuous batching.

No reference counterpart (the reference runs one propagator per script).  Requests are grouped
by (kind, grid side) into pools; a pool is one batched handle (PropagatorBatch) with a fixed
number of slots whose states stay resident in device memory.  Each pool has a worker thread:
between chunks of steps it admits waiting requests into free slots (setting the slot's
parameters and initial state), advances every occupied slot by the next chunk, reads back the
per-step observables, and retires the slots whose requests are complete.  Pools run on their
own CUDA streams, so the work of different pools overlaps on the device.  A pool is created
only when the free device memory covers it (admission by free HBM); idle pools are released
when memory is needed.

Every request's computation is independent of the others in its pool, so a result is the same
alone and in a mix up to the rounding of its chunk boundaries (a chunk ends with the state
normalised, as propagate() does).

Precision: an engine runs every request in complex128 ("c128"), in complex64 ("c64"), or picks per
request ("auto"): complex64 when the error model below keeps the request's relative L2 error within
its tolerance, complex128 (the FP64-accurate form) otherwise.
"""
import collections
import threading
import time

import numpy as np

from .batch import PropagatorBatch
from .rho_bloch_cuda_1d import RhoBlochCUDA1D
from .rho_vneumann_cuda_1d import RhoVNeumannCUDA1D
from .wigner_moyal_cuda_1d import WignerMoyalCUDA1D

# potential sum_k c_k x^k (k = 2..4) and its derivative, per-request constants
V_EXPR = "c2 * X * X + c3 * X * X * X + c4 * X * X * X * X"
DV_EXPR = "2. * c2 * X + 3. * c3 * X * X + 4. * c4 * X * X * X"
PARAMS = ("c2", "c3", "c4", "x0", "p0")
INIT = {
    "wm": "exp(-pow(X - x0, 2) - pow(P - p0, 2))",
    "vn": "exp(-0.5 * pow(X - x0, 2) - 0.5 * pow(X_prime - x0, 2)) * "
          "exp(cuda_complex(0., p0) * (X - X_prime))",
    "rb": "double(i == j)",
}
CLASSES = {"wm": WignerMoyalCUDA1D, "vn": RhoVNeumannCUDA1D, "rb": RhoBlochCUDA1D}


# Relative L2 error of a complex64 propagation after `steps` steps on an n x n grid, against the FP64
# result: the FP32 rounding of each FFT stage of the 4 propagation transforms a step adds up like a
# random walk, err = C eps32 sqrt(4 steps log2 n).  C = 3 bounds the measured values (anharmonic
# Wigner-Moyal 256^2, 1000 steps: 1.4e-5, C = 1.3; strong-field 1024^2, 1000 steps: 3.2e-5, C = 2.7).
C64_ERROR_C = 3.0
EPS32 = 2.0 ** -24


def c64_error(n, steps):
    return C64_ERROR_C * EPS32 * np.sqrt(4.0 * steps * np.log2(n))


def amplitude(n):
    """Grid amplitude of side n: dX dP = 2 pi / n with X_amplitude = P_amplitude."""
    return float(np.sqrt(np.pi * n / 2.0))


class Request:
    """One propagation: kind 'wm' (real-time Wigner-Moyal with Ehrenfest observables), 'vn'
    (real-time von Neumann) or 'rb' (rho-Bloch Gibbs state after `steps` steps of dbeta)."""

    def __init__(self, rid, kind, n, steps, coeffs, x0=0.0, p0=0.0, arrival=0.0, keep_state=False, tol=1e-5):
        self.rid = rid
        self.tol = float(tol)    # relative L2 error the request accepts ("auto" engines)
        self.precision = None    # the form it ran in
        self.kind = kind
        self.n = int(n)
        self.steps = int(steps)
        self.coeffs = tuple(float(c) for c in coeffs)
        self.x0 = float(x0)
        self.p0 = float(p0)
        self.arrival = float(arrival)
        self.keep_state = keep_state
        self.start = None
        self.done = None
        self.steps_done = 0
        self.history = []      # per-step observable rows (wm)
        self.purity = None
        self.state = None      # host copy of the final W (wm) or rho (vn, rb) when keep_state

    @property
    def latency(self):
        return None if self.done is None else self.done - self.arrival

    @property
    def work(self):
        return self.n * self.n * self.steps_done


def pool_bytes(kind, n, slots):
    """Device memory of a pool: state arrays per slot plus scratch (complex128)."""
    per = 16 * n * n
    arrays = 4 if kind == "wm" else 8  # wm: rho, W, scratch, snapshot; vn/rb: rho, (2n)^2 W, scratch, snapshot
    return slots * arrays * per + (64 << 20)


class Pool(threading.Thread):
    """Slots of one (kind, side) and the worker that steps them."""

    def __init__(self, engine, kind, n, slots, precision, chunk, dt, dbeta):
        super().__init__(daemon=True)
        self.engine = engine
        self.kind = kind
        self.n = n
        self.slots = slots
        self.chunk = chunk
        self.dbeta = dbeta
        a = amplitude(n)
        common = dict(t=0.0, dt=dt, X_gridDIM=n, X_amplitude=a, K="0.5 * P * P", V=V_EXPR, precision=precision)
        if kind == "wm":
            kw = dict(common, P_gridDIM=n, P_amplitude=a, diff_K="P", diff_V=DV_EXPR)
        elif kind == "vn":
            kw = dict(common)
        else:
            kw = dict(common, kT=1.0, dbeta=dbeta, t_initial=0.0)
        self.batch = PropagatorBatch(CLASSES[kind], slots, params=PARAMS, init=INIT[kind], **kw)
        self.queue = collections.deque()
        self.cv = threading.Condition()
        self.occupant = [None] * slots
        self.left = [0] * slots
        self.closing = False
        self.error = None
        self.last_busy = time.perf_counter()

    def submit(self, req):
        with self.cv:
            self.queue.append(req)
            self.cv.notify()

    def idle(self):
        with self.cv:
            return not self.queue and all(o is None for o in self.occupant)

    def close(self):
        with self.cv:
            self.closing = True
            self.cv.notify()

    def _admit(self):
        for s in range(self.slots):
            if self.occupant[s] is not None:
                continue
            with self.cv:
                if not self.queue:
                    return
                req = self.queue.popleft()
            c2, c3, c4 = req.coeffs
            self.batch.set_params(s, [c2, c3, c4, req.x0, req.p0])
            self.batch.init_state(s, 1)
            req.start = time.perf_counter()
            self.occupant[s] = req
            self.left[s] = req.steps

    def _step(self):
        active = [o is not None for o in self.occupant]
        self.batch.set_active(active)
        k = min(self.chunk, min(self.left[s] for s in range(self.slots) if active[s]))
        if self.kind == "rb":
            done, pur = self.batch.gibbs_steps(self.dbeta, k, 0, self.slots)
        else:
            self.batch.propagate(k, 0, self.slots)
            done, pur = np.full(self.slots, k), None
        now_finished = []
        for s in range(self.slots):
            req = self.occupant[s]
            if req is None:
                continue
            req.steps_done += int(done[s])
            self.left[s] -= k
            if self.kind == "wm":
                req.history.append(self.batch.history(s)[:k])
            if pur is not None and done[s] > 0:
                req.purity = float(pur[s])
            if self.left[s] <= 0 or int(done[s]) < k:
                now_finished.append(s)
        for s in now_finished:
            req = self.occupant[s]
            if req.keep_state:
                req.state = self.batch.wigner(s) if self.kind == "wm" else self.batch.rho(s)
            if self.kind != "rb":
                req.purity = self.batch.purity(s)
            req.done = time.perf_counter()
            self.occupant[s] = None
            self.engine._finished(req)

    def run(self):
        try:
            while True:
                with self.cv:
                    while not self.closing and not self.queue and all(o is None for o in self.occupant):
                        self.cv.wait()
                    if self.closing and not self.queue and all(o is None for o in self.occupant):
                        break
                self._admit()
                if any(o is not None for o in self.occupant):
                    self._step()
                    self.last_busy = time.perf_counter()
        except Exception as e:  # surfaced by Engine.run
            self.error = e
            self.engine._failed(e)
        finally:
            self.batch.close()


class Engine:
    """Continuous-batching request loop on one GPU."""

    def __init__(self, precision="c128", chunk=200, dt=0.01, dbeta=0.01, slots=None, reserve_bytes=2 << 30):
        assert precision in ("c128", "c64", "auto", "c128-fp64")
        self.precision = precision
        self.chunk = chunk
        self.dt = dt
        self.dbeta = dbeta
        self.slots = slots or {128: 8, 256: 8, 512: 8, 1024: 4, 2048: 2}
        self.reserve = reserve_bytes
        self.pools = {}
        self.lock = threading.Lock()
        self.done_cv = threading.Condition()
        self.finished = []
        self.errors = []

    # pools ----------------------------------------------------------------
    def _free_bytes(self):
        import torch

        free, _ = torch.cuda.mem_get_info()
        return free

    def precision_for(self, req):
        if self.precision != "auto":
            return self.precision
        return "c64" if c64_error(req.n, req.steps) <= req.tol else "c128"

    def pool(self, kind, n, precision=None):
        """The pool of (kind, n, precision), created when the free device memory covers it."""
        precision = precision or (self.precision if self.precision != "auto" else "c128")
        key = (kind, n, precision)
        with self.lock:
            p = self.pools.get(key)
            if p is not None:
                return p
            need = pool_bytes(kind, n, self.slots[n]) // (2 if precision == "c64" else 1) + self.reserve
            while self._free_bytes() < need:
                # release an idle pool, or wait for one to become idle
                idle = [k for k, q in self.pools.items() if q.idle()]
                if idle:
                    q = self.pools.pop(min(idle, key=lambda k: self.pools[k].last_busy))
                    q.close()
                    q.join()
                    continue
                if not self.pools:
                    raise MemoryError("not enough device memory for a %s pool of side %d (%s)" % key)
                time.sleep(0.01)
            p = Pool(self, kind, n, self.slots[n], precision, self.chunk, self.dt, self.dbeta)
            self.pools[key] = p
            p.start()
            return p

    def warm(self, kinds=("wm", "vn", "rb"), sides=(128, 256, 512, 1024, 2048)):
        """Create the pools ahead of the first request (JIT compile, buffers), as a server starts."""
        precs = ("c128", "c64") if self.precision == "auto" else (self.precision,)
        for k in kinds:
            for n in sides:
                for p in precs:
                    self.pool(k, n, p)

    # requests ---------------------------------------------------------------
    def submit(self, req):
        req.precision = self.precision_for(req)
        self.pool(req.kind, req.n, req.precision).submit(req)

    def _finished(self, req):
        with self.done_cv:
            self.finished.append(req)
            self.done_cv.notify_all()

    def _failed(self, e):
        with self.done_cv:
            self.errors.append(e)
            self.done_cv.notify_all()

    def run(self, requests, realtime=True):
        """Submit `requests` at their arrival times (seconds from now) and wait for all of them."""
        t0 = time.perf_counter()
        with self.done_cv:
            target = len(self.finished) + len(requests)  # an engine serves one stream after another
        for r in sorted(requests, key=lambda r: r.arrival):
            if realtime:
                wait = t0 + r.arrival - time.perf_counter()
                if wait > 0:
                    time.sleep(wait)
            r.arrival = time.perf_counter()
            self.submit(r)
        with self.done_cv:
            while len(self.finished) < target and not self.errors:
                self.done_cv.wait(timeout=1.0)
        if self.errors:
            raise self.errors[0]
        return time.perf_counter() - t0

    def close(self):
        with self.lock:
            for p in self.pools.values():
                p.close()
            for p in self.pools.values():
                p.join()
            self.pools.clear()


def make_stream(n_requests, rate, seed=0, sides=(128, 256, 512, 1024, 2048), steps=(100, 5000),
                kinds=("wm", "vn", "rb")):
    """Poisson stream: kind and side uniform, steps ~ U(steps), c2 > 0, c3, c4 >= 0, x0, p0 random."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n_requests):
        t += rng.exponential(1.0 / rate)
        kind = kinds[rng.integers(len(kinds))]
        n = int(sides[rng.integers(len(sides))])
        st = int(rng.integers(steps[0], steps[1] + 1))
        c2 = float(rng.uniform(0.1, 1.0))
        c3 = float(rng.uniform(-0.02, 0.02))
        c4 = float(rng.uniform(0.0, 0.05))
        x0 = float(rng.uniform(-1.5, 1.5))
        p0 = float(rng.uniform(-1.5, 1.5))
        out.append(Request(i, kind, n, st, (c2, c3, c4), x0, p0, arrival=t))
    return out
