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

Precision: an engine runs every request in complex128 ("c128" double-float or "c128-fp64" native
FP64), in complex64 ("c64"), or picks per request ("auto") from a measurement: the request's first
PROBE_STEPS steps run twice, in complex64 and in complex128, from the same initial state; the
relative L2 distance of the two states is the measured complex64 error of the probe window, which is
extrapolated to the request's full step count (FP32 rounding grows between a random walk, steps^0.5,
and a drift, steps^1: the exponent C64_GROWTH bounds both).  A request whose estimate is within its
tolerance continues in complex64 from the complex64 probe's state; otherwise it falls back and
continues in complex128 from the complex128 probe's state, so that no step is run twice more than
the probe window.  Every auto request records the estimate (est_error) and whether it fell back.
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


# Measured complex64 error of the probe window, extrapolated to the whole request:
#   est = err(probe) * (steps / probe) ** C64_GROWTH
# FP32 rounding of the butterflies adds up between a random walk (exponent 0.5) and a drift (1.0);
# measured on the anharmonic 256^2 Wigner-Moyal run against FP64: 2.9e-6 after 100 steps, 7.0e-6
# after 300, 1.5e-5 after 1000 (exponent 0.71), so 0.8 errs on the side of falling back.
PROBE_STEPS = 200
C64_GROWTH = 0.8
EPS32 = 2.0 ** -24
# a tolerance below this is out of complex64's reach whatever the step count (a few FP32 roundings)
C64_MIN_TOL = 8.0 * EPS32


def c64_estimate(probe_err, probe_steps, steps):
    """Estimated relative L2 error after `steps` steps from the error measured after `probe_steps`."""
    if steps <= probe_steps:
        return float(probe_err)
    return float(probe_err) * (steps / float(probe_steps)) ** C64_GROWTH


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
        self.init_rho = None   # start from this rho (host array) instead of the initial-state expression
        self.est_error = None  # auto engines: estimated complex64 error of the whole request (measured)
        self.fell_back = False  # auto engines: the estimate exceeded tol and the request finished in complex128
        self.on_done = None    # internal requests of an auto engine: callback instead of the finished list

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
            if req.init_rho is None:
                self.batch.init_state(s, 1)
            else:
                self.batch.set_rho(s, req.init_rho)
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
                if req.on_done is not None:
                    req.rho = self.batch.rho(s)  # the continuation starts from rho
            if self.kind != "rb":
                req.purity = self.batch.purity(s)
            req.done = time.perf_counter()
            self.occupant[s] = None
            if req.on_done is not None:
                req.on_done(req)
            else:
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

    def __init__(self, precision="c128", chunk=200, dt=0.01, dbeta=0.01, slots=None, reserve_bytes=2 << 30,
                 fallback="c128"):
        """precision: the form of every request, or "auto": complex64 while its measured error allows,
        else `fallback`, a complex128 form ("c128", double-float, or "c128-fp64", native FP64)."""
        assert precision in ("c128", "c64", "auto", "c128-fp64")
        assert fallback in ("c128", "c128-fp64")
        self.precision = precision
        self.fallback = fallback
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
        """The form a request starts in (auto: complex64 unless its tolerance is out of its reach)."""
        if self.precision != "auto":
            return self.precision
        return "c64" if req.tol >= C64_MIN_TOL else self.fallback

    def pool(self, kind, n, precision=None):
        """The pool of (kind, n, precision), created when the free device memory covers it."""
        precision = precision or (self.precision if self.precision != "auto" else self.fallback)
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
        precs = (self.fallback, "c64") if self.precision == "auto" else (self.precision,)
        for k in kinds:
            for n in sides:
                for p in precs:
                    self.pool(k, n, p)

    # requests ---------------------------------------------------------------
    def submit(self, req):
        req.precision = self.precision_for(req)
        if self.precision == "auto" and req.precision == "c64":
            self._probe(req)
            return
        self.pool(req.kind, req.n, req.precision).submit(req)

    # auto: the measured complex64 error and the fallback -------------------------
    def _sub(self, req, steps, precision, init_rho, on_done):
        r = Request(req.rid, req.kind, req.n, steps, req.coeffs, req.x0, req.p0, arrival=req.arrival,
                    keep_state=True, tol=req.tol)
        r.precision = precision
        r.init_rho = init_rho
        r.on_done = on_done
        self.pool(r.kind, r.n, precision).submit(r)
        return r

    def _probe(self, req):
        """Run the first PROBE_STEPS steps of `req` in complex64 and in complex128; when both are done,
        continue in the form the measured error allows (see the module docstring)."""
        probe = min(PROBE_STEPS, req.steps)
        lock = threading.Lock()
        got = {}

        def probe_done(r):
            with lock:
                got[r.precision] = r
                if len(got) < 2:
                    return
            lo, hi = got["c64"], got[self.fallback]
            ref = hi.state
            err = float(np.linalg.norm(lo.state - ref) / max(np.linalg.norm(ref), 1e-300))
            # a Gibbs run that stopped early (purity 1) ends with its probe
            stopped = hi.steps_done < probe or lo.steps_done < probe
            req.est_error = c64_estimate(err, probe, probe if stopped else req.steps)
            keep = lo if req.est_error <= req.tol else hi
            req.fell_back = keep is hi
            req.precision = keep.precision
            req.history = list(keep.history)
            req.steps_done = keep.steps_done
            req.start = min(lo.start, hi.start)
            left = req.steps - probe
            if stopped or left <= 0:
                self._complete(req, keep, continued=False)
                return
            self._sub(req, left, keep.precision, keep.rho, lambda c: self._complete(req, c, continued=True))

        self._sub(req, probe, "c64", None, probe_done)
        self._sub(req, probe, self.fallback, None, probe_done)

    def _complete(self, req, last, continued):
        """Finish an auto request from its last internal request: the probe it kept, or the
        continuation after it (whose steps and observable rows follow the probe's)."""
        if continued:
            req.history.extend(last.history)
            req.steps_done += last.steps_done
        req.purity = last.purity
        if req.keep_state:
            req.state = last.state
        req.done = time.perf_counter()
        self._finished(req)

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
