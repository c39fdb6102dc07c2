"""Throughput of the strong-field Wigner-Moyal split step on GB300.

Workload (the headline configuration): Wigner-Moyal propagation on a
1024 x 1024 (x, p) grid, X_amplitude = 60, P_amplitude = 6, soft-core
V = -1/sqrt(x^2 + 2) + x E(t), E(t) = 0.04 sin^2(pi t / T) sin(0.057 t) over
T = 5 cycles, K = p^2 / 2, dt = 0.05, cos^(1/8) absorbing boundary on the
outer 10 % of x, Ehrenfest observables (<x>, <p>, dipole acceleration,
energy) recorded every step.  The initial state is a Wigner-Bloch Gibbs state
of the field-free Hamiltonian (synthetic: timing does not depend on it).

A "step" is one split step including its per-step Wigner transform,
normalisation and observables.  The metric is grid-point * steps / s.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--precision c128|c128-fp64|c64]

Other workloads (one JSON line each, not the headline):
  --workload plain          Wigner-Moyal 256 x 256, anharmonic, Ehrenfest every step, 1000 steps
  --workload batched-gibbs  64 Wigner-Bloch Gibbs states of 512 x 512 in one batch, per-instance
                            double well and temperature; purity and energy against complex128
  --workload served         Poisson stream of Wigner-Moyal / von Neumann / rho-Bloch requests through
                            the continuous-batching loop: p50 / p99 latency and aggregate throughput
  --workload served-sweep   the served stream at several arrival rates (--rates): achieved vs offered
                            load, p50 / p99 per rate and the knee rate
  --workload large-vn       von Neumann 4096 x 4096, driven Morse potential, 2000 steps
  --workload precision      the headline workload in complex128 (double-float), complex64 and native
                            FP64 side by side: errors of W and of <x>, <p>, dipole acceleration per step
  --workload frames         the headline workload writing a frame (W, t, diagonal of rho) every 100
                            steps through the asynchronous run record, against no frames
  --workload group          five von Neumann propagators of sides 128 to 2048 stepped as one group
                            (one persistent launch per pass), against one after another
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

E_FIELD_C = """
__device__ double E(double t)
{
    const double T = ncyc * 2. * M_PI / omega;
    return E0 * pow(sin(M_PI * t / T), 2) * sin(omega * t);
}
__device__ double cosmask(double x, double xmax)
{
    const double a = fabs(x) - 0.9 * xmax;
    return a > 0. ? pow(fabs(cos(0.5 * M_PI * fmin(a / (0.1 * xmax), 1.))), 0.125) : 1.;
}
"""


def e_field(t, E0=0.04, omega=0.057, ncyc=5):
    T = ncyc * 2 * np.pi / omega
    return E0 * np.sin(np.pi * t / T) ** 2 * np.sin(omega * t)


def cosmask(x, xmax):
    a = np.abs(x) - 0.9 * xmax
    r = np.minimum(np.maximum(a, 0.0) / (0.1 * xmax), 1.0)
    return np.where(a > 0, np.power(np.abs(np.cos(0.5 * np.pi * r)), 0.125), 1.0)


N_GRID = 1024
PARAMS = dict(
    t=0.0, dt=0.05, X_gridDIM=N_GRID, X_amplitude=60.0, P_gridDIM=N_GRID, P_amplitude=6.0,
    E0=0.04, omega=0.057, ncyc=5,
    functions=E_FIELD_C,
    K="0.5 * P * P",
    V="-1. / sqrt(X * X + 2.) + X * E(t)",
    diff_K="P",
    diff_V="X / pow(X * X + 2., 1.5) + E(t)",
    abs_boundary_x="cosmask(XX, XX_max) * cosmask(XX_prime, XX_prime_max)",
)
INIT = "exp(-X * X - P * P) / M_PI"
CHUNK = 50  # steps per propagate() call, as the reference's own driver loop (wigner_moyal_cuda_1d.py:954)

STATE_BYTES_PER_PT = {"c128": 16, "c128-fp64": 16, "c64": 8}
METRIC = "grid-pt*steps/s (Wigner-Moyal split step with per-step Wigner transform and Ehrenfest observables)"
# arithmetic of the passes per precision
DTYPE = {"c128": "f32x2 (double-float pairs; complex128 state)", "c128-fp64": "f64", "c64": "f32 (FP64 tables and sums)",
         "auto": "per request: c64 (f32+f64) within the error bound, else c128"}
ALG_BYTES_FACTOR = 10  # bytes per grid point per step = 10 * S (propagation 4 S + per-step Wigner transform 6 S)


def _rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


class ClockSampler:
    """nvidia-smi samples during the timed region, kept as a CSV in $AW_CLOCKS_DIR (default: the
    temporary directory)."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = os.path.join(os.environ.get("AW_CLOCKS_DIR") or tempfile.gettempdir(),
                                 "clocks_bench_%d.csv" % os.getpid())

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        try:
            rows = [l.split(",") for l in open(self.path).read().strip().splitlines() if l.strip()]
        except Exception:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if len(r) >= 9]
        mx = [float(r[2]) for r in rows if len(r) >= 9]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            if len(r) < 9:
                continue
            for name, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_propagator(precision, init=None):
    """The headline propagator on the headline initial state (or on `init`, a Wigner function)."""
    from accuratewigner_gb300 import WignerMoyalCUDA1D

    prop = WignerMoyalCUDA1D(**PARAMS, precision=precision)
    prop.set_wignerfunction(INIT if init is None else init)
    return prop


def flush_l2(buf):
    buf.add_(1.0)


def headline_config(world):
    """The `config` of the headline line: the same dictionary for both arms."""
    return {
        "workload": "strong-field Wigner-Moyal, 1024x1024 (x,p), X_amplitude=60, P_amplitude=6, soft-core V + "
                    "x E(t), dt=0.05, cos^(1/8) absorber, Ehrenfest every step",
        "grid": [N_GRID, N_GRID],
        "precision": "complex128 state, FP64 arithmetic",
        "steps_per_call": CHUNK,
        "initial_state": "exp(-x^2 - p^2)/pi (synthetic, in place of the beta=100 Wigner-Bloch ground state)",
        "l2": "flushed (256 MB write) before every timed propagate() call; the 48 MB working set (state and two "
              "branch buffers) stays L2-resident within a call",
        "parallelism": "replicas" if world > 1 else "single GPU",
        "algorithmic_bytes_per_pt_step": ALG_BYTES_FACTOR * 16,
    }


DATA = ("synthetic: the 1024x1024 strong-field configuration with the Gaussian exp(-x^2-p^2)/pi as initial "
        "state in place of the beta=100 Wigner-Bloch ground state (timing does not depend on the state)")
# per launch of each pass kind, bytes read + written per grid point in units of S (the element size):
# the row pass reads and writes the state and writes the branch output; the column pass reads and
# writes the state; the marginal pass reads the branch output only
PASS_UNITS = {"row_pass": 3, "column_pass": 2, "marginal_pass": 1}
CLASS_OF = {"row_pass": 0, "column_pass": 1, "marginal_pass": 4}


def kernel_profile(lib, h, precision, peak):
    """One extra propagate() of CHUNK steps with CUDA events around every launch, the overlapped side
    stream folded into the handle's stream so that every event pair times one kernel alone; per pass
    kind: launches, mean duration, algorithmic bytes per launch and the achieved fraction of `peak`."""
    from accuratewigner_gb300 import _lib

    ncls = _lib.AW_PROF_CLASSES
    _lib.check(lib.aw_profile(h, 2))
    t = ctypes.c_double(0.0)
    _lib.check(lib.aw_propagate(h, CHUNK, ctypes.byref(t)))
    ms = (ctypes.c_double * ncls)()
    by = (ctypes.c_double * ncls)()
    nl = (ctypes.c_int64 * ncls)()
    _lib.check(lib.aw_profile_read(h, ms, by, nl))
    _lib.check(lib.aw_profile(h, 0))
    S = STATE_BYTES_PER_PT[precision]
    out = {}
    for name, cls in CLASS_OF.items():
        n = int(nl[cls])
        if not n:
            continue
        mean_ms = ms[cls] / n
        alg = PASS_UNITS[name] * S * N_GRID * N_GRID
        gbs = alg / (mean_ms / 1e3) / 1e9
        out[name] = {"launches": n, "mean_us": mean_ms * 1e3, "total_ms": ms[cls], "alg_bytes_per_launch": alg,
                     "achieved_gbs": gbs, "frac": gbs / peak}
    other = {"expression": 2, "helper": 3}
    out["other"] = {k: {"launches": int(nl[c]), "total_ms": ms[c]} for k, c in other.items()}
    return out


def roofline_of(prof, precision, peak, peaks):
    """The roofline object of the dominant kernel (largest total time among the passes)."""
    passes = {k: v for k, v in prof.items() if k in PASS_UNITS}
    dom = max(passes, key=lambda k: passes[k]["total_ms"])
    d = passes[dom]
    return {
        "bound": "hbm",
        "kernel": dom,
        "achieved": d["achieved_gbs"],
        "peak": peak,
        "unit": "GB/s",
        "frac": d["frac"],
        "traffic": load_traffic(dom, precision),
        "alg_bytes_per_launch": d["alg_bytes_per_launch"],
        "mean_launch_us": d["mean_us"],
        "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback 6800 GB/s",
        "per_kernel": {k: {"mean_us": v["mean_us"], "achieved_gbs": v["achieved_gbs"], "frac": v["frac"],
                           "alg_bytes_per_launch": v["alg_bytes_per_launch"], "launches": v["launches"],
                           "traffic": load_traffic(k, precision)} for k, v in passes.items()},
        "timing": "CUDA events around every launch of one extra %d-step propagate() after the timed region, "
                  "the overlapping side stream folded into the handle's stream (each event pair times one "
                  "kernel alone)" % CHUNK,
        "note": "the 48 MB working set stays in L2 within a call; the passes are bound by the FP64 pipe "
                "(native FP64) or by FP32 issue and latency (double-float), not by HBM: see fp64_pipe",
    }


def time_chunks(lib, h, prop, chunks, l2buf, stream):
    """CUDA-event time of each propagate() call on the library's stream, L2 flushed before each."""
    import torch

    times = []
    for n in chunks:
        flush_l2(l2buf)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        t = ctypes.c_double(prop.t)
        from accuratewigner_gb300 import _lib

        _lib.check(lib.aw_propagate(h, int(n), ctypes.byref(t)))
        prop.t = np.float64(t.value)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    return times


def accuracy_vs_fp64(steps=1000):
    """W relative L2 after `steps` steps and the largest error of <x>, <p> and the dipole acceleration
    over the steps (relative to max(|FP64|, 1)) of the double-float and complex64 forms against the
    native FP64 form, all three from the headline initial state."""
    runs = {}
    for prec in ("c128-fp64", "c128", "c64"):
        g = make_propagator(prec)
        for _ in range(steps // CHUNK):
            g.propagate(CHUNK)
        runs[prec] = (g.wignerfunction.get(), {k: np.array(getattr(g, k)) for k in ("X_average", "P_average",
                                                                                    "P_average_RHS")})
        g.close()
    w_ref, o_ref = runs["c128-fp64"]
    out = {}
    for prec in ("c128", "c64"):
        w, o = runs[prec]
        err = {k: float(np.max(np.abs(o[k] - o_ref[k]) / np.maximum(np.abs(o_ref[k]), 1.0))) for k in o}
        out[prec] = {"steps": steps, "W_rel_l2": float(np.linalg.norm(w - w_ref) / np.linalg.norm(w_ref)),
                     "x": err["X_average"], "p": err["P_average"], "dipole_acceleration": err["P_average_RHS"]}
    return out


def run_ours(args):
    import torch

    from accuratewigner_gb300 import _lib

    rank, world, local = _rank()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    lib = _lib.load()
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    l2buf = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > 129 MB L2
    npts = N_GRID * N_GRID
    chunks = []
    left = args.steps
    while left > 0:
        chunks.append(min(CHUNK, left))
        left -= chunks[-1]

    def measure(precision, clocked):
        prop = make_propagator(precision)
        h = prop._h
        st = ctypes.c_void_p()
        _lib.check(lib.aw_stream(h, ctypes.byref(st)))
        stream = torch.cuda.ExternalStream(st.value)
        t = ctypes.c_double(prop.t)
        _lib.check(lib.aw_propagate(h, max(args.warmup, 3), ctypes.byref(t)))  # warm-up
        prop.t = np.float64(t.value)
        torch.cuda.synchronize()
        launches0 = _lib.launch_count()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        if clocked:
            with ClockSampler(local) as clk:
                times = time_chunks(lib, h, prop, chunks, l2buf, stream)
            clocks = clk.summary()
        else:
            times, clocks = time_chunks(lib, h, prop, chunks, l2buf, stream), None
        torch.cuda.synchronize()
        launches = _lib.launch_count() - launches0
        from accuratewigner_gb300.replicas import job_throughput

        total, _, value = job_throughput(float(sum(times)), npts * args.steps, device="cuda")
        if dist:
            dist.barrier()
        prof = kernel_profile(lib, h, precision, peak)
        return prop, {"value": value, "ms_per_step": total / args.steps * 1e3, "launches": int(launches),
                      "clocks": clocks, "profile": prof, "roofline": roofline_of(prof, precision, peak, peaks)}

    prop, main = measure(args.precision, True)

    # end-to-end through the public API with host buffers: per chunk upload rho from pinned host memory,
    # propagate, read back the Wigner function (into pinned host memory) and the observables
    host_rho = torch.empty((N_GRID, N_GRID), dtype=torch.complex128, pin_memory=True).numpy()
    host_w = torch.empty((N_GRID, N_GRID), dtype=torch.complex128, pin_memory=True).numpy()
    host_rho[:] = prop.rho.get()
    e2e_times = []
    for n in chunks:
        flush_l2(l2buf)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        prop.rho.set(host_rho)
        prop.propagate(n)
        prop.wignerfunction.get(host_w)
        _ = prop.X_average[-n:], prop.P_average[-n:], prop.P_average_RHS[-n:]
        torch.cuda.synchronize()
        e2e_times.append(time.perf_counter() - t0)
    prop.close()
    from accuratewigner_gb300.replicas import job_throughput

    e2e_total, _, e2e_value = job_throughput(float(sum(e2e_times)), npts * args.steps, device="cuda")
    h2d = npts * 16 * len(chunks) / args.steps
    d2h = (npts * 16 + CHUNK * 7 * 8) * len(chunks) / args.steps

    # the other two arithmetic forms of the same step, each with its own time and roofline, and their
    # errors against native FP64
    forms = {}
    if not args.no_forms:
        for prec in ("c128-fp64", "c128", "c64"):
            if prec == args.precision:
                continue
            p2, m = measure(prec, False)
            p2.close()
            forms[prec] = {"dtype": DTYPE[prec], "value": m["value"], "ms_per_step": m["ms_per_step"],
                           "roofline": {k: m["roofline"][k] for k in ("kernel", "achieved", "frac", "per_kernel")}}
        if world == 1:
            acc = accuracy_vs_fp64()
            for prec, e in acc.items():
                if prec in forms:
                    forms[prec]["error_vs_fp64"] = e

    if rank == 0:
        cpu = cpu_baseline(args) if world == 1 and not args.no_cpu else None
        line = {
            "metric": METRIC,
            "value": main["value"],
            "unit": "grid-pt*steps/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": main["ms_per_step"],
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": DTYPE[args.precision],
            "data": DATA,
            "config": headline_config(world),
            "e2e": {"value": e2e_value, "unit": "grid-pt*steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": main["launches"],
            "roofline": main["roofline"],
            "fp64_pipe": fp64_pipe_note(args.precision),
            "fp64_roofline": fp64_roofline(args.precision, main["value"], main["clocks"]),
            "kernel_profile": main["profile"],
            "forms": forms,
            "clocks": main["clocks"],
        }
        if args.precision != "c128-fp64":
            line["config"]["precision"] = DTYPE[args.precision]
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def fp64_pipe_note(precision):
    """FP64-pipe figures of the passes from the committed ncu capture, for the native FP64 form."""
    if precision != "c128-fp64":
        return None
    path = os.path.join(ROOT, "profiles", "traffic_per_launch.json")
    try:
        return json.load(open(path)).get("fp64_pipe")
    except Exception:
        return None


def fp64_roofline(precision, value, clocks, sms=None):
    """The native FP64 step against the FP64 pipe: the passes' FP64 instructions a point (committed ncu
    counts; the per-call launches left out) times grid-pt*steps/s, over 2 FP64 lanes a clock a SM at the
    SM clock sampled during the run (sms: the SM count, by default the device's)."""
    note = fp64_pipe_note(precision)
    if not note or "fp64_instructions_per_point" not in note:
        return None
    per = note["fp64_instructions_per_point"]
    inst = sum(v for k, v in per.items() if isinstance(v, (int, float)))
    mhz = (clocks or {}).get("sm_mhz") or (clocks or {}).get("sm_max_mhz")
    if not mhz:
        return None
    if sms is None:
        import torch

        sms = torch.cuda.get_device_properties(0).multi_processor_count
    peak = 2.0 * sms * mhz * 1e6
    achieved = inst * value
    return {"bound": "fp64 pipe", "fp64_inst_per_point_step": inst, "achieved_inst_per_s": achieved,
            "peak_inst_per_s": peak, "frac": achieved / peak, "sm_mhz": mhz,
            "note": "FP64 lane instructions of the row, column and marginal passes a grid point a step "
                    "(profiles/traffic_per_launch.json) x the measured grid-pt*steps/s"}


def load_traffic(kernel, precision):
    """DRAM bytes per launch of a pass kind, from the committed ncu summary (or None)."""
    path = os.path.join(ROOT, "profiles", "traffic_per_launch.json")
    try:
        return json.load(open(path)).get("%s/%s" % (kernel, precision))
    except Exception:
        return None


def cpu_baseline(args, steps=2):
    """The oracle (NumPy + pocketfft, all host cores) on a bounded sample of the workload."""
    from oracle import propagators as orc

    params = {k: v for k, v in PARAMS.items() if k != "functions"}
    o = orc.WignerMoyalOracle(**params, py_functions={"E": e_field, "cosmask": cosmask})
    o.set_wignerfunction(INIT)
    o.propagate(1)
    t0 = time.perf_counter()
    o.propagate(steps)
    dt = time.perf_counter() - t0
    return {"value": N_GRID * N_GRID * steps / dt, "unit": "grid-pt*steps/s", "cores": orc.WORKERS, "kind": "port",
            "sample": "%d steps of the same 1024x1024 workload (oracle, scipy.fft workers=%d)" % (steps, orc.WORKERS)}


def run_reference(args):
    rank, world, _ = _rank()
    if rank != 0:
        return
    from oracle import propagators as orc

    params = {k: v for k, v in PARAMS.items() if k != "functions"}
    o = orc.WignerMoyalOracle(**params, py_functions={"E": e_field, "cosmask": cosmask})
    o.set_wignerfunction(INIT)
    o.propagate(max(1, min(args.warmup, 1)))
    sample = 1  # each step is a bounded sample of the workload (one full split step on the 1024^2 grid)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        o.propagate(sample)
        times.append(time.perf_counter() - t0)
    total = float(sum(times))
    value = N_GRID * N_GRID * sample * args.steps / total
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": "grid-pt*steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": total / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": DATA,
        "config": headline_config(world),
        "cpu_baseline": {"value": value, "unit": "grid-pt*steps/s", "cores": orc.WORKERS, "kind": "port",
                         "sample": "one split step per timed step (NumPy restatement of the reference, scipy.fft "
                                   "workers=%d)" % orc.WORKERS},
        "e2e": {"value": value, "unit": "grid-pt*steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


# ------------------------------------------------------------------------ other workloads
def _timed(fn):
    import torch

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = fn()
    torch.cuda.synchronize()
    return time.perf_counter() - t0, out


def _line(workload, metric, value, unit, seconds, args, config, extra=None, higher=True):
    line = {"workload": workload, "metric": metric, "value": value, "unit": unit, "n_gpus": 1,
            "seconds": seconds, "higher_is_better": higher, "dtype": DTYPE[args.precision],
            "data": "synthetic, seeded", "config": config}
    line.update(extra or {})
    print(json.dumps(line))


def plain_propagator(precision):
    """Wigner-Moyal 256 x 256, Xa = 8, Pa = 7, V = x^2 / 2 + 0.05 x^4, dt = 0.01, Ehrenfest observables."""
    from accuratewigner_gb300 import WignerMoyalCUDA1D

    p = dict(t=0.0, dt=0.01, X_gridDIM=256, X_amplitude=8.0, P_gridDIM=256, P_amplitude=7.0, K="0.5 * P * P",
             V="0.5 * X * X + 0.05 * X * X * X * X", diff_K="P", diff_V="X + 0.2 * X * X * X",
             precision=precision)
    g = WignerMoyalCUDA1D(**p)
    g.set_wignerfunction("exp(-pow(X - 1., 2) - P * P) / M_PI")
    return g


def run_plain(args):
    """The plain 256 x 256 propagator (plain_propagator), 1000 steps in calls of CHUNK."""
    g = plain_propagator(args.precision)
    for _ in range(2):  # warm-up calls of the timed length (their step-window graphs are captured here)
        g.propagate(CHUNK)
    steps = 1000
    with ClockSampler(0) as clk:
        sec, _ = _timed(lambda: [g.propagate(CHUNK) for _ in range(steps // CHUNK)])
    _line("plain", "grid-pt*steps/s", 256 * 256 * steps / sec, "grid-pt*steps/s", sec, args,
          {"grid": [256, 256], "steps": steps, "steps_per_call": CHUNK, "precision": args.precision},
          {"ms_per_step": sec / steps * 1e3, "clocks": clk.summary()})


def run_batched_gibbs(args):
    """64 Wigner-Bloch instances of 512 x 512 (Xa = 10, Pa = 8), V = a x^4 - b x^2 with a ~ U(0.02, 0.1),
    b ~ U(0.2, 1.0), beta ~ LogU(0.5, 20), dbeta = 0.01, all in one batch."""
    from accuratewigner_gb300 import WignerBlochCUDA1D
    from accuratewigner_gb300.batch import PropagatorBatch, dbeta_num_beta_steps

    n_inst, n = 64, 512
    rng = np.random.default_rng(0)
    a = rng.uniform(0.02, 0.1, n_inst)
    b = rng.uniform(0.2, 1.0, n_inst)
    beta = np.exp(rng.uniform(np.log(0.5), np.log(20.0), n_inst))
    kT = 1.0 / beta
    steps = np.array([dbeta_num_beta_steps(k, 0.01)[1] for k in kT])
    order = np.argsort(steps, kind="stable")  # instances ordered by step count
    base = dict(t=0.0, X_gridDIM=n, P_gridDIM=n, X_amplitude=10.0, P_amplitude=8.0, K="0.5 * P * P",
                V="a * X * X * X * X - b * X * X", dt=0.01, dbeta=0.01, kT=1.0, t_initial=0.0)

    def run(prec):
        bt = PropagatorBatch(WignerBlochCUDA1D, n_inst, params=("a", "b"), init="1.", precision=prec, **base)
        for slot, k in enumerate(order):
            bt.set_params(slot, [a[k], b[k]])
        bt.gibbs(kT[order])  # warm-up (JIT, buffers)
        sec, (done, pur) = _timed(lambda: bt.gibbs(kT[order]))
        e = bt.energy.copy()
        bt.close()
        return sec, done, pur, e

    with ClockSampler(0) as clk:
        sec, done, pur, e = run(args.precision)
    ref = run("c128") if args.precision != "c128" else None
    work = float(np.sum(done)) * n * n
    extra = {"ms_total": sec * 1e3, "instances": n_inst, "steps_total": int(np.sum(done)),
             "purity_range": [float(pur.min()), float(pur.max())], "clocks": clk.summary()}
    if ref:
        extra["vs_c128"] = {"max_abs_purity_err": float(np.max(np.abs(pur - ref[2]))),
                            "max_rel_energy_err": float(np.max(np.abs(e - ref[3]) / np.abs(ref[3])))}
    _line("batched-gibbs", "grid-pt*steps/s", work / sec, "grid-pt*steps/s", sec, args,
          {"instances": n_inst, "grid": [n, n], "X_amplitude": 10.0, "P_amplitude": 8.0, "dbeta": 0.01,
           "beta": "LogU(0.5, 20), seed 0", "potential": "a x^4 - b x^2, a ~ U(0.02, 0.1), b ~ U(0.2, 1.0)",
           "precision": args.precision}, extra)


def run_precision(args):
    """The headline workload run in native FP64 (the reference), double-float complex128 and complex64:
    relative L2 error of W every 50 steps and the largest error of <x>, <p> and the dipole
    acceleration over the steps."""
    from accuratewigner_gb300 import WignerMoyalCUDA1D

    steps = args.steps if args.steps != 200 else 1000
    w0 = make_propagator("c128").wignerfunction.get()

    def run(prec):
        g = WignerMoyalCUDA1D(**PARAMS, precision=prec)
        g.set_wignerfunction(w0)
        ws = []
        for _ in range(steps // CHUNK):
            g.propagate(CHUNK)
            ws.append(g.wignerfunction.get())
        obs = {k: np.array(getattr(g, k)) for k in ("X_average", "P_average", "P_average_RHS")}
        g._handle.close()
        return ws, obs

    ref_w, ref_o = run("c128-fp64")
    out = {}
    for prec in ("c128", "c64"):
        ws, obs = run(prec)
        w_err = [float(np.linalg.norm(a - b) / np.linalg.norm(b)) for a, b in zip(ws, ref_w)]
        o_err = {k: float(np.max(np.abs(obs[k] - ref_o[k]) / np.maximum(np.abs(ref_o[k]), 1.0))) for k in obs}
        out[prec] = {"W_rel_l2_every_50_steps": w_err, "W_rel_l2_final": w_err[-1],
                     "max_scaled_err": {"x": o_err["X_average"], "p": o_err["P_average"],
                                        "dipole_acceleration": o_err["P_average_RHS"]}}
    _line("precision", "relative L2 error of W vs native FP64 after %d steps (c64)" % steps,
          out["c64"]["W_rel_l2_final"], "relative L2", 0.0, args,
          {"workload": "strong-field Wigner-Moyal 1024x1024 (the headline)", "steps": steps,
           "reference": "c128-fp64 (native FP64 passes)", "observable_scale": "max(|ref|, 1)"},
          {"errors": out}, higher=False)


def run_served(args):
    """Poisson stream of Wigner-Moyal / von Neumann / rho-Bloch requests, sides {128 .. 2048},
    steps ~ U(100, 5000), through the continuous-batching request loop."""
    from accuratewigner_gb300.serve import Engine, make_stream

    eng = Engine(precision=args.precision, chunk=200, fallback=args.fallback)
    eng.warm()
    reqs = make_stream(args.requests, args.rate, seed=0)
    for r in reqs:
        r.tol = args.tol
    with ClockSampler(0) as clk:
        wall = eng.run(reqs)
    eng.close()
    lat = np.array([r.latency for r in reqs])
    work = float(sum(r.work for r in reqs))
    by_kind = {k: float(np.percentile([r.latency for r in reqs if r.kind == k], 50))
               for k in ("wm", "vn", "rb") if any(r.kind == k for r in reqs)}
    _line("served", "grid-pt*steps/s (aggregate) with p50/p99 request latency", work / wall, "grid-pt*steps/s",
          wall, args,
          {"requests": args.requests, "rate_per_s": args.rate, "seed": 0, "sides": [128, 256, 512, 1024, 2048],
           "steps": "U(100, 5000)", "kinds": ["wigner-moyal (Ehrenfest)", "von Neumann", "rho-Bloch Gibbs"],
           "potential": "c2 x^2 + c3 x^3 + c4 x^4, c2 ~ U(0.1, 1), c3 ~ U(-0.02, 0.02), c4 ~ U(0, 0.05)",
           "amplitude": "X_amplitude = P_amplitude = sqrt(pi N / 2)", "chunk_steps": 200,
           "precision": args.precision, "tolerance": args.tol, "fallback": args.fallback},
          dict({"p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
                "mean_latency_s": float(lat.mean()), "p50_latency_by_kind_s": by_kind, "clocks": clk.summary()},
               **auto_summary(reqs)))


def auto_summary(reqs):
    """Requests of an auto engine: how many ran in each form and the measured complex64 error estimates."""
    est = [r.est_error for r in reqs if r.est_error is not None]
    if not est:
        return {}
    return {"auto": {"complex64": sum(1 for r in reqs if r.precision == "c64"),
                     "fell_back_to_complex128": sum(1 for r in reqs if r.fell_back),
                     "complex128_from_the_start": sum(1 for r in reqs if r.est_error is None),
                     "est_error_p50": float(np.percentile(est, 50)), "est_error_max": float(np.max(est)),
                     "tolerance": float(reqs[0].tol)}}


def run_served_sweep(args):
    """The served stream at several Poisson rates (one warmed engine, the same seeded requests at each
    rate, arrival times scaled by 1/rate): offered and delivered load, p50/p99 latency per rate.
    The knee is the highest rate whose p50 latency stays within twice the p50 of the lowest rate."""
    from accuratewigner_gb300.serve import Engine, make_stream

    rates = sorted(float(r) for r in args.rates.split(","))
    eng = Engine(precision=args.precision, chunk=200, fallback=args.fallback)
    eng.warm()
    sweep = []
    with ClockSampler(0) as clk:
        for rate in rates:
            reqs = make_stream(args.requests, rate, seed=0)
            for r in reqs:
                r.tol = args.tol
            span = max(r.arrival for r in reqs)
            asked = float(sum(r.n * r.n * r.steps for r in reqs))  # rho-Bloch requests may stop early
            wall = eng.run(reqs)
            lat = np.array([r.latency for r in reqs])
            sweep.append({"rate_per_s": rate, "offered": asked / span, "delivered": asked / wall,
                          "executed": float(sum(r.work for r in reqs)) / wall, "wall_s": wall,
                          "p50_latency_s": float(np.percentile(lat, 50)),
                          "p99_latency_s": float(np.percentile(lat, 99))})
    eng.close()
    base = sweep[0]["p50_latency_s"]
    knee = max(s["rate_per_s"] for s in sweep if s["p50_latency_s"] <= 2.0 * base)
    best = max(s["executed"] for s in sweep)
    _line("served-sweep", "grid-pt*steps/s (executed, best over the rate sweep) with the knee rate", best,
          "grid-pt*steps/s", sum(s["wall_s"] for s in sweep), args,
          {"requests_per_rate": args.requests, "rates_per_s": rates, "seed": 0, "sides": [128, 256, 512, 1024, 2048],
           "steps": "U(100, 5000)", "kinds": ["wigner-moyal (Ehrenfest)", "von Neumann", "rho-Bloch Gibbs"],
           "chunk_steps": 200, "precision": args.precision,
           "knee": "highest rate whose p50 latency is <= 2 x the p50 latency at the lowest rate",
           "offered / delivered": "requested grid-pt*steps over the arrival span / over the wall time"},
          {"knee_rate_per_s": knee, "sweep": sweep, "clocks": clk.summary()})


def run_frames(args):
    """The headline run with its on-disk record: a frame (W, t, diagonal of rho) saved every 100 steps
    through the asynchronous writer, against the same steps without frames."""
    import shutil

    import torch

    from accuratewigner_gb300.records import RunRecord

    prop = make_propagator(args.precision)
    chunk, frames = 100, 10
    prop.propagate(chunk)  # warm-up

    def plain():
        for _ in range(frames):
            prop.propagate(chunk)
        torch.cuda.synchronize()

    d = tempfile.mkdtemp(prefix="aw_frames_")
    try:
        with ClockSampler(0) as clk:
            t_plain, _ = _timed(plain)
            rec = RunRecord(d, prop, PARAMS)  # staging slots and pinned buffers: set up once per run

            def recorded():
                for _ in range(frames):
                    prop.propagate(chunk)
                    rec.save_frame()
                torch.cuda.synchronize()
                t_loop = time.perf_counter()
                rec.close()  # waits for the last frames' writes
                return t_loop

            t0 = time.perf_counter()
            t_rec, t_loop = _timed(recorded)
            t_loop -= t0
        frame_bytes = os.path.getsize(os.path.join(d, "frames", "0.npz"))
    finally:
        shutil.rmtree(d, ignore_errors=True)
    work = float(N_GRID * N_GRID * chunk * frames)
    _line("frames", "grid-pt*steps/s with a frame written every 100 steps", work / t_rec, "grid-pt*steps/s", t_rec,
          args, {"workload": "strong-field Wigner-Moyal 1024x1024 (the headline)", "steps": chunk * frames,
                 "frame_every_steps": chunk, "frame": "W real part, t, diagonal of rho (.npz)",
                 "precision": args.precision},
          {"without_frames": work / t_plain, "overhead_fraction": t_rec / t_plain - 1.0,
           "propagation_with_capture_s": t_loop, "propagation_alone_s": t_plain,
           "drain_after_last_frame_s": t_rec - t_loop, "bytes_per_frame": frame_bytes,
           "note": "frames go to a temporary directory; once the host file system's write rate is below "
                   "the frame rate the drain, not the capture, sets the time",
           "clocks": clk.summary()})


def _group_sets(spec):
    """'128,256,512;128x8' -> [[128, 256, 512], [128] * 8]"""
    out = []
    for part in spec.split(";"):
        sides = []
        for tok in part.split(","):
            n, _, k = tok.strip().partition("x")
            sides += [int(n)] * (int(k) if k else 1)
        out.append(sides)
    return out


def group_member_params(n, k, precision):
    """Member k (side n) of a group workload: its own harmonic-plus-quartic potential."""
    return dict(t=0.0, dt=0.01, X_gridDIM=n, X_amplitude=float(np.sqrt(np.pi * n / 2.0)), x0=0.3 * k, p0=-0.2 * k,
                c2=0.2 + 0.1 * k, K="0.5 * P * P", V="c2 * X * X + 0.01 * X * X * X * X", precision=precision)


def run_group(args):
    """Von Neumann propagators of the given sides (default one each of 128, 256, 512, 1024 and 2048; their
    own potentials), 200 steps: grouped (one persistent launch per pass of a step for all of them) against
    the same propagators stepped one after another through propagate().  One line per set of sides."""
    import torch

    from accuratewigner_gb300 import RhoVNeumannCUDA1D
    from accuratewigner_gb300.batch import propagate_group

    steps = 200
    init = ("exp(-0.5 * pow(X - x0, 2) - 0.5 * pow(X_prime - x0, 2)) * "
            "exp(cuda_complex(0., p0) * (X - X_prime))")

    for sides in _group_sets(args.sides):
        props = []
        for k, n in enumerate(sides):
            g = RhoVNeumannCUDA1D(**group_member_params(n, k, args.precision))
            g.set_rho(init)
            props.append(g)
        work = float(sum(n * n for n in sides)) * steps
        # warm-up calls of the timed length (step-window graphs are captured per call length)
        for _ in range(2):
            propagate_group(props, CHUNK)
        with ClockSampler(0) as clk:
            t_group, _ = _timed(lambda: [propagate_group(props, CHUNK) for _ in range(steps // CHUNK)])
        for _ in range(2):
            for g in props:
                g.propagate(CHUNK)
        # each member through its own propagate(); the members' streams overlap on the device
        t_streams, _ = _timed(lambda: [[g.propagate(CHUNK) for g in props] for _ in range(steps // CHUNK)])

        def serial():
            for _ in range(steps // CHUNK):
                for g in props:
                    g.propagate(CHUNK)
                    torch.cuda.synchronize()

        t_serial, _ = _timed(serial)  # one member at a time
        for g in props:
            g.close()
        _line("group", "grid-pt*steps/s (von Neumann propagators of sides %s stepped as one group)"
              % ",".join(map(str, sides)), work / t_group, "grid-pt*steps/s", t_group, args,
              {"sides": sides, "steps": steps, "steps_per_call": CHUNK, "precision": args.precision},
              {"own_streams": work / t_streams, "vs_own_streams": t_streams / t_group,
               "one_at_a_time": work / t_serial, "vs_one_at_a_time": t_serial / t_group, "clocks": clk.summary()})


def large_vn_config(n=4096):
    """Parameters and initial state of the 4096^2 von Neumann workload.  The Morse wall is capped at 1e4
    (it reaches 9e69 at x = -80, where kick phases would depend on the last bits of V); states in the
    well move as under the uncapped wall."""
    morse = "D * pow(1. - exp(-alpha * (X - xm)), 2)"
    p = dict(t=0.0, dt=0.02, X_gridDIM=n, X_amplitude=80.0, D=0.18, alpha=1.0, xm=1.4, Vcap=1e4, K="0.5 * P * P",
             V="fmin(%s, Vcap) + X * 0.02 * sin(0.01 * t)" % morse, diff_K="P",
             diff_V="2. * D * alpha * exp(-alpha * (X - xm)) * (1. - exp(-alpha * (X - xm))) * (%s < Vcap)"
                    " + 0.02 * sin(0.01 * t)" % morse)
    rng = np.random.default_rng(0)
    centres = rng.uniform(0.5, 4.0, 8)
    w = rng.uniform(0.2, 1.0, 8)
    w /= w.sum()
    x = np.linspace(-80.0, 80.0 - 160.0 / n, n)

    def rho0():
        r = np.zeros((n, n))
        for c, wk in zip(centres, w):
            g = np.exp(-0.5 * (x - c) ** 2)
            r += wk * np.outer(g, g)
        return r

    return p, rho0


def run_large_vn(args):
    """von Neumann 4096 x 4096, X_amplitude = 80, Morse V = D (1 - exp(-alpha (x - x0)))^2 + x 0.02 sin(0.01 t)
    (D = 0.18, alpha = 1, x0 = 1.4), dt = 0.02, 2000 steps; rho0 = sum of 8 seeded Gaussian pure states."""
    from accuratewigner_gb300 import RhoVNeumannCUDA1D

    n, steps = 4096, args.steps if args.steps != 200 else 2000
    p, rho0 = large_vn_config()

    def run(prec, k):
        g = RhoVNeumannCUDA1D(precision=prec, **p)
        g.set_rho(rho0())
        g.propagate(3)
        sec, _ = _timed(lambda: [g.propagate(min(CHUNK, k - i)) for i in range(0, k, CHUNK)])
        out = (sec, g.rho.get(), np.array(g.X_average), g.get_purity())
        g._handle.close()
        return out

    with ClockSampler(0) as clk:
        sec, rho, xav, pur = run(args.precision, steps)
    bytes_per_pt = 4 * STATE_BYTES_PER_PT[args.precision]
    extra = {"ms_per_step": sec / steps * 1e3, "achieved_gbs": bytes_per_pt * n * n * steps / sec / 1e9,
             "algorithmic_bytes_per_pt_step": bytes_per_pt, "trace": float(np.trace(rho).real * 160.0 / n),
             "purity": float(pur), "x_final": float(xav[-1]), "clocks": clk.summary()}
    if args.precision != "c128-fp64":
        # against the native FP64 form (held to the FP64 oracle at 1e-10 by the 4096^2 parity test)
        _, rref, xref, pref = run("c128-fp64", steps)
        tr = float(np.trace(rho).real * 160.0 / n)
        tref = float(np.trace(rref).real * 160.0 / n)
        extra["vs_fp64"] = {"rho_rel_l2": float(np.linalg.norm(rho - rref) / np.linalg.norm(rref)),
                            "trace_err": abs(tr - tref), "purity_err": float(abs(pur - pref)),
                            "x_max_abs_err": float(np.max(np.abs(xav - xref)))}
    _line("large-vn", "grid-pt*steps/s", n * n * steps / sec, "grid-pt*steps/s", sec, args,
          {"grid": [n, n], "X_amplitude": 80.0, "dt": 0.02, "steps": steps, "potential": "Morse capped at 1e4",
           "initial": "8 Gaussians, centres U(0.5, 4), seed 0",
           "precision": args.precision}, extra)


def run_profile_window(args):
    """The headline (or the 4096^2 von Neumann, or the plain 256^2) workload with `--profile-steps` steps
    inside a profiler range: the launches an ncu capture with --profile-from-start off sees are those
    steps' alone."""
    import torch

    torch.cuda.init()
    if args.workload == "plain":
        g = plain_propagator(args.precision)
    elif args.workload == "large-vn":
        from accuratewigner_gb300 import RhoVNeumannCUDA1D

        p, rho0 = large_vn_config()
        g = RhoVNeumannCUDA1D(precision=args.precision, **p)
        g.set_rho(rho0())
    else:
        g = make_propagator(args.precision)
    g.propagate(max(args.warmup, 3))
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    t0 = time.perf_counter()
    g.propagate(args.profile_steps)
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    print(json.dumps({"profile_window": args.workload, "precision": args.precision, "steps": args.profile_steps,
                      "ms_per_step": (time.perf_counter() - t0) / args.profile_steps * 1e3}))
    g.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="c128-fp64", choices=["c128", "c128-fp64", "c64", "auto"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-forms", action="store_true", help="headline: skip the other arithmetic forms")
    ap.add_argument("--profile-steps", type=int, default=0,
                    help="set up the workload (headline, plain or large-vn), warm up, run this many steps inside a "
                         "cudaProfilerStart/Stop range (for ncu --profile-from-start off) and exit")
    ap.add_argument("--workload", default="strong-field",
                    choices=["strong-field", "plain", "batched-gibbs", "served", "served-sweep", "large-vn",
                             "precision", "frames", "group"])
    ap.add_argument("--requests", type=int, default=60, help="served: number of requests (per rate for the sweep)")
    ap.add_argument("--rate", type=float, default=4.0, help="served: Poisson arrival rate per second")
    ap.add_argument("--rates", default="1,1.5,2,3,4", help="served-sweep: comma-separated arrival rates per second")
    ap.add_argument("--fallback", default="c128", choices=["c128", "c128-fp64"],
                    help="served with --precision auto: the complex128 form a request falls back to")
    ap.add_argument("--tol", type=float, default=1e-5,
                    help="served: each request's relative error tolerance (precision auto runs complex64 within it)")
    ap.add_argument("--sides", default="128,256,512,1024,2048",
                    help="group: sets of grid sides separated by ';', each a comma list ('NxK' = K members of side N)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    other = {"plain": run_plain, "batched-gibbs": run_batched_gibbs, "served": run_served,
             "served-sweep": run_served_sweep, "large-vn": run_large_vn, "precision": run_precision,
             "frames": run_frames, "group": run_group}
    if args.precision == "auto" and args.workload not in ("served", "served-sweep"):
        ap.error("--precision auto chooses per request: only the served workload has requests")
    if args.profile_steps:
        run_profile_window(args)
        return
    if args.workload in other:
        import torch

        torch.cuda.init()
        other[args.workload](args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
