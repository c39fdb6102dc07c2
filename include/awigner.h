/* awigner.h -- C ABI of the GB300 split-operator propagators.
 *
 * The reference (dibondar/AccurateWigner) is Python 2 + PyCUDA: each propagator
 * class pastes CUDA-C expression strings into kernel templates, compiles them
 * with nvcc at construction and drives cuFFT through ctypes.  This library is
 * the native layer beneath drop-in Python classes with the same names; every
 * entry point below names the reference method it replaces.  Citations are
 * file:line inside the reference project.
 *
 * Conventions
 *   - Every call returns AW_OK (0) or a negative AW_E_* code; the message of the
 *     last failure on the calling thread is available from aw_last_error().
 *   - Complex buffers are interleaved (re, im) and C-ordered [row][column],
 *     rows = P / X' index, columns = X index, as in the reference.
 *   - A handle owns its device buffers and one CUDA stream; it is not
 *     thread-safe.  Calls are stream-ordered; calls that return data to the host
 *     synchronise the stream.
 */
#ifndef AWIGNER_H
#define AWIGNER_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AW_OK 0
#define AW_E_ARG -1      /* invalid argument (Python maps to AssertionError / ValueError) */
#define AW_E_CUDA -2     /* CUDA runtime failure */
#define AW_E_JIT -3      /* NVRTC compile error of a user expression (RuntimeError) */
#define AW_E_STATE -4    /* call not valid for this propagator kind or state */
#define AW_E_NOMEM -5    /* device allocation failed */

/* propagator kinds */
#define AW_WIGNER_MOYAL 0   /* WignerMoyalCUDA1D       wigner_moyal_cuda_1d.py:10 */
#define AW_WIGNER_BLOCH 1   /* WignerBlochCUDA1D       wigner_bloch_cuda_1d.py:9 */
#define AW_RHO_VNEUMANN 2   /* RhoVNeumannCUDA1D       rho_vneumann_cuda_1d.py:15 */
#define AW_RHO_BLOCH 3      /* RhoBlochCUDA1D          rho_bloch_cuda_1d.py:10 */
#define AW_SCHRODINGER 4    /* SchrodingerWignerCUDA1D schrodinger_wigner_cuda_1d.py:16 */

/* arithmetic of the state */
#define AW_C128 0           /* complex128 state, as the reference (wigner_moyal_cuda_1d.py:629); passes in
                               double-float arithmetic (FP32 hi + lo pairs, about 2^-48 per operation) */
#define AW_C64 1            /* complex64 butterflies and phases; FP64 tables and reductions */
#define AW_C128_FP64 2      /* complex128 state, passes in native FP64 arithmetic: the reference's
                               arithmetic, and what the Python classes use when not told otherwise */

/* device buffers */
#define AW_BUF_RHO 0        /* rho (WM/WB: Np x Nx in the rotated frame; VN/RB: N x N) */
#define AW_BUF_WIGNER 1     /* wignerfunction (WM/WB: Np x Nx; VN/RB: 2N x 2N; SW: N x N) */
#define AW_BUF_PSI 2        /* wavefunction (SW: 1 x N) */
#define AW_BUF_SNAPSHOT 3   /* copy of rho / psi used by ground-state rollback */

/* spatial classes of an observable term */
#define AW_TERM_X 0         /* expression of X (and t) only */
#define AW_TERM_P 1         /* expression of P (and t) only */

typedef struct aw_state_s* aw_handle;

typedef struct aw_config {
  int32_t kind;
  int32_t precision;
  int32_t x_grid_dim;        /* X_gridDIM */
  int32_t p_grid_dim;        /* P_gridDIM (WM/WB); ignored otherwise */
  /* kernel constants, already rounded through "%.15e" as the reference's
   * #defines round them (wigner_moyal_cuda_1d.py:171-176) */
  double dX, dP;
  double dXX, dXX_prime, dPP, dPP_prime;   /* WM/WB rotated grids (wm:122-134); VN: dXX = dX, dPP */
  double dt;
  double t_initial;
  double dXdP;               /* measure of the Wigner grid used by averages and norms */
  /* source of the user module: the reference's cuda_consts string (all
   * #defines + consts + functions) and the expression strings */
  const char* cuda_consts;
  const char* V;
  const char* K;
  const char* abs_boundary_x;
  const char* abs_boundary_p;
  int32_t v_time_dependent;  /* V mentions t: phase tables are rebuilt every step */
  int32_t k_time_dependent;
  int32_t absx_mode;         /* 0: identically one; 1: fixed in time; 2: depends on t */
  int32_t absp_mode;
  /* observables recorded every step (Ehrenfest theorems and energy,
   * wigner_moyal_cuda_1d.py:584-606) as sums of X-only and P-only terms */
  int32_t ehrenfest;
  int32_t n_obs_x;
  const char* const* obs_x;
  int32_t n_obs_p;
  const char* const* obs_p;
  int32_t n_terms;
  const int32_t* term_slot;
  const int32_t* term_kind;  /* AW_TERM_X / AW_TERM_P */
  const int32_t* term_index; /* index into obs_x / obs_p */
  const double* term_coef;
  int32_t n_slots;
  int32_t obs_p_time_dependent; /* a P-only observable mentions t */
  /* Batches (no reference counterpart: the batched and served forms).  n_inst > 1 makes the
   * handle hold n_inst independent instances of the same kind and grid, stepped together by
   * every call; each has its own state, tables, norm, stop flag and observable history.
   * param_names are per-instance constants usable in V, K, the absorbing boundaries, the
   * observables and init_expr; values are set per instance with aw_set_params.  init_expr is
   * the initial state of an instance (W(X, P) for Wigner-Moyal / Wigner-Bloch, rho(X, X_prime)
   * for von Neumann / rho-Bloch), evaluated by aw_init_state.  Batches require V and K that do
   * not depend on t.  n_inst = 0 or 1 with n_params = 0 is the plain single propagator. */
  int32_t n_inst;
  int32_t n_params;
  const char* const* param_names;
  const char* init_expr;
} aw_config;

/* Batches: the view [first, first + count) of instances that the following calls act on
 * (state buffers, fills, sums, transforms, propagation); the full range after aw_create.
 * aw_set_params writes instance `inst`'s parameter row (n_params values); aw_set_active marks
 * which instances of the view the step loops advance (inactive ones keep their state);
 * aw_init_state evaluates init_expr for the view and normalises it as set_wignerfunction /
 * set_rho do (wigner_moyal_cuda_1d.py:379-420, rho_vneumann_cuda_1d.py:348-385);
 * aw_history_of reads one instance's observable rows of the last propagation;
 * aw_gibbs_batch runs `steps` Bloch steps on the view with a step dbeta[k] per instance and
 * reports per-instance steps done and purity (wigner_bloch_cuda_1d.py:119-155,
 * rho_bloch_cuda_1d.py:125-161). */
int aw_set_view(aw_handle h, int32_t first, int32_t count);
int aw_set_params(aw_handle h, int32_t inst, const double* values);
int aw_set_active(aw_handle h, const int32_t* flags);
int aw_init_state(aw_handle h);
int aw_history_of(aw_handle h, int32_t inst, double* out, int64_t max_rows, int64_t* rows, int32_t* cols);
int aw_gibbs_batch(aw_handle h, const double* dbeta, int64_t steps, int64_t* done, double* purity);
int aw_bloch_min_of(aw_handle h, int32_t inst, double* v_min, double* k_min);

/* library */
int32_t aw_version(void);
const char* aw_last_error(void);
/* number of CUDA kernels this library has launched since load (all handles) */
int64_t aw_launch_count(void);

/* Timing of the handle's own launches with CUDA events (no counterpart in the
 * reference, which has no timers).  aw_profile(h, 1) clears and starts
 * recording with every launch on its usual stream; aw_profile(h, 2) does the
 * same but puts the work that normally overlaps the next step (the marginal
 * pass and observable reduction of Wigner-Moyal steps) on the handle's own
 * stream, so that each event pair times one kernel running alone;
 * aw_profile(h, 0) stops.  aw_profile_read fills, per launch class (0 row
 * passes, 1 column passes that store, 2 expression kernels, 3 helper kernels,
 * 4 reduction-only column passes), the summed device time in ms, the summed
 * algorithmic HBM bytes and the launch count: arrays of AW_PROF_CLASSES. */
/* Forms of the propagation passes (no counterpart in the reference; its axis-0
 * and axis-1 cuFFT plans, cufft.py:274-343, leave no such choice), as chosen by
 * the autotuner when the handle is created: form[0] columns per column-pass
 * block, form[1] whether the column tile is staged in shared memory by TMA
 * tensor copies instead of per-thread loads, form[2] elements a thread (and so
 * the FFT radix) of the column pass, 0 by the size rule or 1 the other choice,
 * form[3] the same for the row pass.  The column forms are timed per handle and
 * never change a result; the row shape is timed once per grid and form in the
 * process (the purity sum over row blocks follows it).  `set` (4 entries, < 0
 * keeps an entry; may be null) overrides, `get` (may be null) receives the
 * forms in force.  Columns per block: a power of two dividing the columns; TMA
 * needs rows of a multiple of 16 bytes. */
int aw_pass_form(aw_handle h, const int32_t* set, int32_t* get);

/* CUDA graphs of the Wigner-Moyal step loop (no counterpart in the reference,
 * whose propagate() launches every kernel from a Python loop,
 * wigner_moyal_cuda_1d.py:563-582).  With Ehrenfest observables, aw_propagate
 * runs windows of its steps (as many as fit, 16 to 248, an even count) from a
 * graph captured on first use per window length and replayed (the kick tables,
 * step times and history rows of a window live at fixed device addresses,
 * refreshed on the stream between windows); the first step, the last and any
 * remainder run on the streams.  Results are bit-identical with and without
 * graphs.  On by default for grids of at most 512 x 512 points, where launch
 * latency is a large part of a step; enable = 0 turns it off for the handle, 1
 * on. */
int aw_graph(aw_handle h, int32_t enable);

/* Grouped propagation (no counterpart in the reference, which runs one
 * propagator per script): `steps` real-time steps of `count` (1 to 8) von
 * Neumann handles of different square grid sizes (sides 64 to 2048, powers of
 * two; each handle a single propagator or a batch, over its current view), as
 * aw_propagate does for each (rho_vneumann_cuda_1d.py:429-448).  Members of
 * side up to 128 (complex64: 256) step together: every pass of a step is ONE
 * persistent launch over the tiles of all of them and the trace normalisation
 * one launch over all their instances; they compute with 8 elements a thread
 * (radix-8 FFT stages) in both passes, give the same bits alone (a group of
 * one) as in any group, and agree with their own aw_propagate with those
 * shapes (aw_pass_form) to rounding.  That work runs on the first grouped
 * member's stream; each grouped member's stream waits for it.  Larger members
 * fill the GPU with their own launches: each runs aw_propagate's step loop
 * (its bits) on its own stream, concurrently.  Members must share one
 * arithmetic form and record no per-step observables; V, K and absorbers must
 * not depend on t.  t[k] is member k's time, advanced on return. */
int aw_group_propagate(aw_handle* handles, int32_t count, int64_t steps, double* t);

#define AW_PROF_CLASSES 5
int aw_profile(aw_handle h, int32_t enable);
int aw_profile_read(aw_handle h, double* ms, double* bytes, int64_t* launches);

/* Construction: replaces the __init__ of each propagator class
 * (wigner_moyal_cuda_1d.py:17-327, wigner_bloch_cuda_1d.py:19-68,
 * rho_vneumann_cuda_1d.py:22-335, rho_bloch_cuda_1d.py:20-68,
 * schrodinger_wigner_cuda_1d.py:26-303): NVRTC compiles the expression
 * strings (SourceModule in the reference), device buffers are allocated and
 * the FFT twiddles and shear tables are built.  Bloch kinds also evaluate
 * V_min and K_min (wigner_bloch_cuda_1d.py:70-92, rho_bloch_cuda_1d.py:70-98).
 * Device memory: a few grid-sized complex buffers (state, Wigner function,
 * scratch); a single native FP64 Wigner-Moyal / Wigner-Bloch propagator of
 * up to 1024 x 1024 points also keeps full shear tables and, once it
 * propagates in real time, full K-kick and (for a V that does not depend on
 * t) V-kick tables: up to four more grid-sized complex128 arrays (16 MB each
 * at 1024 x 1024), which save FP64 products in its passes. */
int aw_create(const aw_config* cfg, aw_handle* out);
int aw_destroy(aw_handle h);
/* The checks of aw_create without a device: the configuration is validated and the expression
 * strings are compiled with NVRTC for `arch` ("sm_103a" when null or empty), which is where the
 * reference's constructors raise a CompileError (SourceModule in wigner_moyal_cuda_1d.py:241-247).
 * Nothing is allocated and no CUDA runtime call is made, so it runs on a machine without a GPU. */
int aw_check_config(const aw_config* cfg, const char* arch);
int aw_stream(aw_handle h, void** stream);
int aw_sync(aw_handle h);
int aw_bloch_min(aw_handle h, double* v_min, double* k_min);

/* Buffers: the device arrays the reference exposes as GPUArrays
 * (self.rho, self.wignerfunction, self.wavefunction) and their .get(). */
int aw_buffer(aw_handle h, int32_t which, void** dptr, int64_t* rows, int64_t* cols, int32_t* elem_bytes);
/* copy in/out as interleaved complex128 host or device memory */
int aw_set_buffer(aw_handle h, int32_t which, const void* src, int32_t src_on_device);
int aw_get_buffer(aw_handle h, int32_t which, void* dst, int32_t dst_on_device);
int aw_copy_buffer(aw_handle h, int32_t from, int32_t to);
/* initial conditions given as a CUDA-C string (init kernels of
 * wigner_moyal_cuda_1d.py:781-802, rho_vneumann_cuda_1d.py:773-794,
 * schrodinger_wigner_cuda_1d.py:857-875) or a constant (GPUArray.fill) */
int aw_fill_expr(aw_handle h, int32_t which, const char* expr);
int aw_fill_const(aw_handle h, int32_t which, double re, double im);
/* sum of a buffer (gpuarray.sum), trace of rho (skcuda linalg.trace),
 * multiplication by a complex scalar (GPUArray /=) */
int aw_sum(aw_handle h, int32_t which, double* re, double* im);
int aw_trace(aw_handle h, double* re, double* im);
int aw_scale(aw_handle h, int32_t which, double re, double im);

/* Phase-space transforms.
 *   WM/WB: aw_wigner2rho   = wigner_moyal_cuda_1d.py:422-469
 *          aw_rho2wigner   = wigner_moyal_cuda_1d.py:471-538 (blackman != 0: :503-538)
 *   VN/RB: aw_rho2wigner   = get_wignerfunction, rho_vneumann_cuda_1d.py:387-427 (normalised)
 *   SW:    aw_rho2wigner   = get_wigner / get_wigner_blackman, schrodinger_wigner_cuda_1d.py:593-663
 * aw_normalize_rho_wigner = wigner_moyal_cuda_1d.py:608-622 (WM/WB only). */
int aw_wigner2rho(aw_handle h);
int aw_rho2wigner(aw_handle h, int32_t blackman);
int aw_normalize_rho_wigner(aw_handle h);

/* Real-time propagation: `steps` repetitions of t += dt; single_step_propagation;
 * normalisation; Ehrenfest observables -- wigner_moyal_cuda_1d.py:563-582,
 * rho_vneumann_cuda_1d.py:429-448, schrodinger_wigner_cuda_1d.py:371-390.
 * *t holds the time before the call and receives the time after it, accumulated
 * step by step in FP64 exactly as the reference's `self.t += self.dt`. */
int aw_propagate(aw_handle h, int64_t steps, double* t);
/* One split step at time t exactly as single_step_propagation (wigner_moyal_cuda_1d.py:543-561,
 * rho_vneumann_cuda_1d.py:450-468, schrodinger_wigner_cuda_1d.py:356-369): not normalised, no
 * observables, the time left to the caller. */
int aw_single_step(aw_handle h, double t);
/* Observables recorded by the last aw_propagate: rows x (n_slots + 2) doubles,
 * columns = slots, purity, norm. */
int aw_history(aw_handle h, double* out, int64_t max_rows, int64_t* rows, int32_t* cols);

/* Expectation values.
 *   WM/WB: Sum Re W f(X,P,t) dXdP            wigner_moyal_cuda_1d.py:329-347
 *   SW:    Sum |psi|^2 f(X,P,t)              schrodinger_wigner_cuda_1d.py:392-410
 *   VN/RB: Tr[... f3(x) g2(p) f1(x) rho] dX  rho_vneumann_cuda_1d.py:520-563
 *          (ops = ordered tuple, NULL entries skip a factor) */
int aw_average(aw_handle h, const char* expr, double t, double* out);
int aw_average_ops(aw_handle h, const char* const* ops, int32_t n_ops, double t, double* out);
/* purity: WM/WB 2 pi Sum W^2 dXdP (wm:349-354); VN/RB Sum |rho|^2 dX^2 (vn:565-579) */
int aw_purity(aw_handle h, double* out);

/* Imaginary time.
 *   aw_bloch_step: one bloch_single_step_propagation including its
 *   normalisation (wigner_bloch_cuda_1d.py:221-240, rho_bloch_cuda_1d.py:225-246)
 *   followed by the recorded observables of one step: out[0..n_slots-1] slots,
 *   out[n_slots] purity (may be NULL).
 *   aw_gibbs: get_gibbs_state's loop (wigner_bloch_cuda_1d.py:119-155,
 *   rho_bloch_cuda_1d.py:125-161): up to `steps` Bloch steps of size dbeta,
 *   stopping after the first step whose purity is not below one.  *done
 *   receives the number of steps taken, *purity the last purity. */
int aw_bloch_step(aw_handle h, double dbeta, double* out);
int aw_gibbs(aw_handle h, double dbeta, int64_t steps, int64_t* done, double* purity);

/* Schrodinger imaginary time (schrodinger_wigner_cuda_1d.py:484-591):
 * `steps` Bloch steps, each followed by renormalisation (project != 0:
 * Gram-Schmidt against the stored stationary states instead). */
int aw_sw_imag_steps(aw_handle h, int64_t steps, int32_t project);
int aw_sw_store_state(aw_handle h);                 /* append psi to the stationary states */
int aw_sw_clear_states(aw_handle h);                /* forget the stored stationary states */
int aw_sw_get_state(aw_handle h, int32_t index, void* dst_host);
int aw_sw_energy(aw_handle h, double t, double* out); /* get_energy, sw:461-482 */
/* get_Ehrenfest, sw:412-459: the observable row (n_slots + 2 doubles) of the current wave function
 * at time t; the wave function is left unchanged */
int aw_sw_ehrenfest(aw_handle h, double t, double* row);

/* Buffer reduction that allocates nothing (no counterpart in the reference).
 * For callers that cannot allocate device memory: a host application that owns
 * the whole device memory budget and hands the library only pointers into its
 * own pool, or a latency-critical loop where cudaMalloc / cudaFree would
 * synchronise the device.  Same sums as aw_sum (mode 0: Sum a, complex),
 * aw_purity (mode 1: Sum Re(a*a)), |a|^2 (mode 2) and aw_trace (mode 3: Sum of
 * a[k * stride], k < n), over n complex128 (elem_bytes 16) or complex64 (8)
 * elements at `data`; writes out_device[0..1] = (re, im), stream-ordered on
 * `stream`.  For the trace the buffer must hold (n - 1) * stride + 1 elements
 * (an index that overflows 64 bits is rejected with AW_E_ARG).  Scratch is a
 * 16 KiB static device array: at most 67108864 elements per call (larger n is
 * rejected with AW_E_ARG).  The first call on a device looks up that array's
 * address; make it before any stream capture.  Later calls outside capture
 * look it up again (it moves after cudaDeviceReset); calls inside capture use
 * the address kept by the last call outside it.  Calls overlapping on the GPU
 * race on the shared array. */
int aw_reduce_noalloc(const void* data, int32_t elem_bytes, int64_t n, int64_t stride, int32_t mode,
                      double* out_device, void* stream);

#ifdef __cplusplus
}
#endif
#endif
