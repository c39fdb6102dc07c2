"""Small configurations whose reference results are stored in tests/golden/.

Expressions are plain CUDA-C arithmetic (no user `functions`), so that the
NumPy oracle, the GPU library and the reference's kernels all evaluate them.
"""
CASES = {
    # Wigner-Moyal, anharmonic, non-square grid, Ehrenfest every step (wm:543-606)
    "wm_anharmonic": dict(
        kind="wm",
        params=dict(t=0.0, dt=0.01, X_gridDIM=64, X_amplitude=6.0, P_gridDIM=32, P_amplitude=5.0,
                    K="0.5 * P * P", V="0.5 * X * X + 0.05 * X * X * X * X", diff_K="P", diff_V="X + 0.2 * X * X * X"),
        ops=[["set_wigner", "exp(-pow(X - 1., 2) - P * P) / M_PI"], ["propagate", 12], ["save", "wigner"],
             ["save", "rho"], ["save", "ehrenfest"], ["save", "purity"], ["save", "t"],
             ["average", ["xp", "X * P"]], ["save", "rho2wigner_blackman"]],
    ),
    # Wigner-Moyal with a time-dependent potential and both absorbing boundaries, no Ehrenfest
    "wm_driven_absorbing": dict(
        kind="wm",
        params=dict(t=0.3, dt=0.02, X_gridDIM=64, X_amplitude=8.0, P_gridDIM=64, P_amplitude=5.0, F=0.3,
                    K="0.5 * P * P", V="0.5 * X * X + X * F * sin(0.7 * t)",
                    abs_boundary_x="pow(abs(cos(0.5 * M_PI * XX / (XX_max + dXX)) * cos(0.5 * M_PI * XX_prime / (XX_prime_max + dXX_prime))), dt * 0.1)",
                    abs_boundary_p="exp(-0.001 * dt * (PP * PP + PP_prime * PP_prime))"),
        ops=[["set_wigner", "exp(-pow(X + 0.5, 2) - pow(P - 0.3, 2))"], ["propagate", 10], ["save", "wigner"],
             ["save", "rho"], ["save", "t"]],
    ),
    # Wigner-Bloch Gibbs state of the harmonic oscillator (wb:119-155)
    "wb_gibbs": dict(
        kind="wb",
        params=dict(t=0.0, dt=0.01, X_gridDIM=64, X_amplitude=6.0, P_gridDIM=64, P_amplitude=6.0, kT=0.7, omega=1.3,
                    K="0.5 * P * P", V="0.5 * omega * omega * X * X + 0.02 * X * X * X * X"),
        ops=[["gibbs"], ["save", "wigner"], ["save", "rho"], ["save", "purity"]],
    ),
    # von Neumann with absorbing boundaries and Ehrenfest (vn:429-591), then the padded Wigner transform
    "vn_ehrenfest": dict(
        kind="vn",
        params=dict(t=0.0, dt=0.01, X_gridDIM=64, X_amplitude=8.0, sigma=1.0, p0=0.4, x0=0.5,
                    K="0.5 * P * P", V="0.1 * X * X + 0.01 * X * X * X * X", diff_K="P",
                    diff_V="0.2 * X + 0.04 * X * X * X",
                    abs_boundary_x="pow(abs(cos(0.5 * M_PI * X / (X_max + dX))), 0.01)",
                    abs_boundary_p="exp(-0.0001 * P * P)"),
        ops=[["set_rho", "exp(-sigma * pow(X - x0, 2) + cuda_complex(0., p0) * X) * "
                         "exp(-sigma * pow(X_prime - x0, 2) - cuda_complex(0., p0) * X_prime)"],
             ["propagate", 10], ["save", "rho"], ["save", "ehrenfest"], ["save", "purity"], ["save", "vn_wigner"]],
    ),
    # rho-Bloch Gibbs state (rb:125-161), including the K_min = 0 quirk (rb:370)
    "rb_gibbs": dict(
        kind="rb",
        params=dict(t=0.0, dt=0.01, X_gridDIM=64, X_amplitude=8.0, kT=0.5, omega=1.1,
                    K="0.5 * P * P + 0.1", V="0.5 * omega * omega * X * X"),
        ops=[["gibbs"], ["save", "rho"], ["save", "purity"], ["save", "vn_wigner"]],
    ),
    # Schrodinger-Wigner: propagation with Ehrenfest, Wigner transforms, imaginary-time ground state
    "sw_propagate": dict(
        kind="sw",
        params=dict(t=0.0, dt=0.01, X_gridDIM=128, X_amplitude=8.0, K="0.5 * P * P",
                    V="0.5 * X * X + 0.05 * X * X * X * X", diff_K="P", diff_V="X + 0.2 * X * X * X",
                    abs_boundary_x="pow(abs(cos(0.5 * M_PI * X / (8. + dX))), 0.01)"),
        ops=[["set_psi", "exp(-pow(X - 1., 2) + cuda_complex(0., 0.5) * X)"], ["propagate", 15], ["save", "psi"],
             ["save", "ehrenfest"], ["save", "sw_wigner"], ["ground", 200], ["save", "energy"]],
    ),
    # Wigner-Moyal with absorbing boundaries that depend on t in both frames and a driven potential,
    # Ehrenfest every step, then single steps (wm:543-561) at the advanced times
    "wm_tdep_absorbers": dict(
        kind="wm",
        params=dict(t=0.1, dt=0.02, X_gridDIM=64, X_amplitude=8.0, P_gridDIM=32, P_amplitude=5.0, F=0.3,
                    K="0.5 * P * P", V="0.5 * X * X + X * F * sin(0.7 * t)", diff_K="P", diff_V="X + F * sin(0.7 * t)",
                    abs_boundary_x="pow(abs(cos(0.5 * M_PI * XX / (XX_max + dXX)) * cos(0.5 * M_PI * XX_prime / (XX_prime_max + dXX_prime))), dt * (0.1 + 0.05 * sin(t)))",
                    abs_boundary_p="exp(-0.001 * dt * (1. + cos(0.5 * t)) * (PP * PP + PP_prime * PP_prime))"),
        ops=[["set_wigner", "exp(-pow(X + 0.5, 2) - pow(P - 0.3, 2))"], ["propagate", 8], ["save", "wigner"],
             ["save", "rho"], ["save", "ehrenfest"], ["single_steps", 2], ["save", "rho_single"]],
    ),
    # von Neumann single steps (vn:450-468): not normalised
    "vn_single_steps": dict(
        kind="vn",
        params=dict(t=0.0, dt=0.01, X_gridDIM=64, X_amplitude=8.0, sigma=1.0, p0=0.4, x0=0.5,
                    K="0.5 * P * P", V="0.1 * X * X + 0.01 * X * X * X * X"),
        ops=[["set_rho", "exp(-sigma * pow(X - x0, 2) + cuda_complex(0., p0) * X) * "
                         "exp(-sigma * pow(X_prime - x0, 2) - cuda_complex(0., p0) * X_prime)"],
             ["single_steps", 3], ["save", "rho_single"]],
    ),
    # The cases below pin the oracle on the CPU only (gpu=False): the GPU library is checked against
    # the oracle for the same features by test_rho_schrodinger_gpu.py (ordered von Neumann averages)
    # and test_wigner_moyal_gpu.py / test_rho_schrodinger_gpu.py (ground states; their loops stop on
    # purities that may differ from the reference's in the last digits, so those checks use 1e-8).
    # von Neumann averages of ordered operator products (vn:520-563, kernel vn:811-821)
    "vn_ordered_averages": dict(
        kind="vn", gpu=False,
        params=dict(t=0.0, dt=0.01, X_gridDIM=64, X_amplitude=8.0, sigma=1.0, p0=0.4, x0=0.5,
                    K="0.5 * P * P", V="0.1 * X * X + 0.01 * X * X * X * X"),
        ops=[["set_rho", "exp(-sigma * pow(X - x0, 2) + cuda_complex(0., p0) * X) * "
                         "exp(-sigma * pow(X_prime - x0, 2) - cuda_complex(0., p0) * X_prime)"],
             ["propagate", 6], ["average", ["x", ["X"]]], ["average", ["p", [None, "P"]]],
             ["average", ["p2x", [None, "P * P", "X"]]], ["average", ["xpx", ["X", "P", "X"]]],
             ["save", "purity"]],
    ),
    # Wigner-Bloch ground state with the dbeta-halving rollback (wb:157-219)
    "wb_ground_state": dict(
        kind="wb", gpu=False,
        params=dict(t=0.0, dt=0.05, X_gridDIM=64, X_amplitude=6.0, P_gridDIM=64, P_amplitude=6.0, dbeta=0.05,
                    K="0.5 * P * P", V="0.5 * X * X + 0.05 * X * X * X * X"),
        ops=[["ground_state", 1e-8], ["save", "wigner"], ["save", "purity"]],
    ),
    # rho-Bloch ground state (rb:163-223)
    "rb_ground_state": dict(
        kind="rb", gpu=False,
        params=dict(t=0.0, dt=0.05, X_gridDIM=64, X_amplitude=8.0, dbeta=0.05,
                    K="0.5 * P * P", V="0.5 * X * X + 0.05 * X * X * X * X"),
        ops=[["ground_state", 1e-8], ["save", "rho"], ["save", "purity"]],
    ),
}


def _arr(x):
    import numpy as np

    return x.get() if hasattr(x, "get") and not isinstance(x, np.ndarray) else np.array(x)


def run_ops(obj, spec):
    """Apply a case's operations to an oracle or a GPU propagator; return the saved results."""
    import numpy as np

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
            if arg == "rho_single":
                out["rho_single"] = _arr(obj.rho)
            elif arg == "wigner":
                out["wigner"] = _arr(obj.wignerfunction)
            elif arg == "rho":
                out["rho"] = _arr(obj.rho)
            elif arg == "psi":
                out["psi"] = _arr(obj.wavefunction)
            elif arg == "rho2wigner_blackman":
                out["wigner_blackman"] = _arr(obj.rho2wigner_blackman())
            elif arg == "vn_wigner":
                out["vn_wigner"] = _arr(obj.get_wignerfunction())
            elif arg == "sw_wigner":
                out["sw_wigner"] = _arr(obj.get_wigner())
                out["sw_wigner_blackman"] = _arr(obj.get_wigner_blackman())
            elif arg == "ehrenfest":
                for k in ("X_average", "X_average_RHS", "P_average", "P_average_RHS", "hamiltonian_average"):
                    out[k] = np.array(getattr(obj, k))
            elif arg == "purity":
                out["purity"] = obj.get_purity()
            elif arg == "energy":
                out["energy"] = obj.get_energy()
            elif arg == "t":
                out["t"] = float(obj.t)
        elif verb == "average":
            key, expr = arg
            out["avg_" + key] = obj.get_average(expr)
    return out


def load_golden(name):
    import os

    import numpy as np

    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", name + ".npz")
    with np.load(path, allow_pickle=False) as z:
        return {k: z[k] for k in z.files if k != "meta"}


def compare(got, want, tol, scale=1.0):
    """Largest mismatch per key: relative L2 for arrays, scale-aware for scalars and histories."""
    import numpy as np

    bad = {}
    for k, w in want.items():
        g = np.asarray(got[k])
        w = np.asarray(w)
        if w.ndim >= 2:
            err = float(np.linalg.norm((g - w).ravel()) / np.linalg.norm(w.ravel()))
        elif w.dtype.kind in "iu":
            err = 0.0 if np.array_equal(g, w) else 1.0
        else:
            err = float(np.max(np.abs(g - w)) / max(float(np.max(np.abs(w))) if w.size else 0.0, scale))
        if not err <= tol:
            bad[k] = err
    return bad
