"""Generate the golden vectors in tests/golden/ from the reference's own kernel code.

Runs only where the reference checkout exists (the build container):

    python tests/golden/make_golden.py          # the cases that have no file yet
    python tests/golden/make_golden.py --all    # every case

Each case runs a small configuration through oracle/ref_kernels.py, i.e. the
reference's CUDA-C kernels compiled for the CPU by oracle/ref_build.py, driven
in the reference's op order with pocketfft standing in for cuFFT, and stores
the parameters and results in <case>.npz.  The tests compare both the NumPy
oracle and the GPU library against these files.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from oracle import ref_build, ref_kernels  # noqa: E402
from golden_cases import CASES  # noqa: E402


def run_case(name, spec):
    kind = spec["kind"]
    params = dict(spec["params"])
    cls = {"wm": ref_kernels.RefWignerMoyal, "wb": ref_kernels.RefWignerBloch, "vn": ref_kernels.RefRhoVNeumann,
           "rb": ref_kernels.RefRhoBloch, "sw": ref_kernels.RefSchrodingerWigner}[kind]
    obj = cls(**params)
    out = {}
    for op in spec["ops"]:
        verb, arg = op[0], op[1] if len(op) > 1 else None
        if verb == "set_wigner":
            obj.set_wignerfunction(arg)
        elif verb == "set_rho":
            obj.set_rho(arg)
        elif verb == "set_psi":
            obj.set_wavefunction(arg)
        elif verb == "propagate":
            obj.propagate(arg)
        elif verb == "gibbs":
            obj.get_gibbs_state()
            out["gibbs_steps_done"] = obj.gibbs_steps_done
            out["V_min"] = obj.V_min
            out["K_min"] = obj.K_min
        elif verb == "ground":
            obj.set_ground_state(arg)
        elif verb == "ground_state":
            obj.get_ground_state(abs_tol_purity=arg)
        elif verb == "single_steps":
            for _ in range(arg):
                obj.t += obj.dt
                obj.single_step_propagation()
        elif verb == "save":
            what = arg
            if what == "rho_single":
                out["rho_single"] = np.array(obj.rho)
            elif what == "wigner":
                out["wigner"] = np.array(obj.wignerfunction)
            elif what == "rho":
                out["rho"] = np.array(obj.rho)
            elif what == "psi":
                out["psi"] = np.array(obj.wavefunction)
            elif what == "rho2wigner_blackman":
                out["wigner_blackman"] = np.array(obj.rho2wigner_blackman())
            elif what == "vn_wigner":
                out["vn_wigner"] = np.array(obj.get_wignerfunction())
            elif what == "sw_wigner":
                out["sw_wigner"] = np.array(obj.get_wigner())
                out["sw_wigner_blackman"] = np.array(obj.get_wigner(blackman=True))
            elif what == "ehrenfest":
                for k in ("X_average", "X_average_RHS", "P_average", "P_average_RHS", "hamiltonian_average"):
                    out[k] = np.array(getattr(obj, k))
            elif what == "purity":
                out["purity"] = obj.get_purity()
            elif what == "energy":
                out["energy"] = obj.get_energy()
            elif what == "t":
                out["t"] = float(obj.t)
        elif verb == "average":
            key, expr = arg
            out["avg_" + key] = obj.get_average(expr)
    return out


def main():
    if not ref_build.available():
        sys.exit("the reference checkout is needed to regenerate the golden vectors")
    redo = "--all" in sys.argv
    for name, spec in CASES.items():
        if not redo and os.path.exists(os.path.join(HERE, name + ".npz")):
            continue
        out = run_case(name, spec)
        meta = json.dumps({"kind": spec["kind"], "ops": spec["ops"]})
        np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=np.array(meta), **out)
        print(name, sorted(out))


if __name__ == "__main__":
    main()
