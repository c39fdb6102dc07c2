// C ABI of the GB300 split-operator propagators (declared in include/awigner.h).
//
// A handle owns the device state of one propagator: the grid buffers, the FFT
// twiddles, the shear tables of the Wigner transform, the phase tables built
// from the user's V and K, and the NVRTC module compiled from the user's
// strings.  The step loops run entirely on the device: every scalar the
// reference brings back to the host each step (norms, traces, observables,
// purity) stays in device memory and feeds the next pass directly.
#include <cuda_runtime.h>
#include <nvrtc.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "aw_jit.h"
#include "aw_pass.h"
#include "aw_util.h"
#include "awigner.h"

#define AW_VERSION 1

static thread_local std::string g_err;
static std::atomic<long long> g_launches{0};

static int fail(int code, const char* fmt, ...) {
  char buf[4096];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define CK(call)                                                                      \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess) return fail(AW_E_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)
#define TRY(call)        \
  do {                   \
    int r_ = (call);     \
    if (r_) return r_;   \
  } while (0)
#define KL(call)                                                                  \
  do {                                                                            \
    cudaEvent_t pe_ = prof_mark(h);                                               \
    int r_ = (call);                                                              \
    prof_done(h, PROF_UTIL, 0.0, pe_);                                            \
    ++g_launches;                                                                 \
    if (r_) return fail(AW_E_CUDA, "kernel launch failed (%d): %s", r_, #call);   \
  } while (0)

// ============================================================================ NVRTC
struct JitLib {
  cudaLibrary_t lib = nullptr;
};
static std::mutex g_jit_mu;
static std::unordered_map<std::string, cudaLibrary_t> g_jit_cache;

// NVRTC: `src` compiled for the option `arch` ("--gpu-architecture=sm_103a"); needs no device
static int nvrtc_cubin(const std::string& src, const char* arch, std::vector<char>* cubin) {
  nvrtcProgram prog;
  if (nvrtcCreateProgram(&prog, src.c_str(), "aw_user.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS)
    return fail(AW_E_JIT, "nvrtcCreateProgram failed");
  const char* opts[] = {arch, "--std=c++17", "-lineinfo"};
  nvrtcResult r = nvrtcCompileProgram(prog, 3, opts);
  if (r != NVRTC_SUCCESS) {
    size_t n = 0;
    nvrtcGetProgramLogSize(prog, &n);
    std::string log(n, '\0');
    nvrtcGetProgramLog(prog, &log[0]);
    nvrtcDestroyProgram(&prog);
    return fail(AW_E_JIT, "NVRTC could not compile the user expressions:\n%s", log.c_str());
  }
  size_t n = 0;
  nvrtcGetCUBINSize(prog, &n);
  cubin->resize(n);
  nvrtcGetCUBIN(prog, cubin->data());
  nvrtcDestroyProgram(&prog);
  return AW_OK;
}

static int jit_compile(const std::string& src, cudaLibrary_t* out) {
  int dev = 0, maj = 0, mnr = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&maj, cudaDevAttrComputeCapabilityMajor, dev));
  CK(cudaDeviceGetAttribute(&mnr, cudaDevAttrComputeCapabilityMinor, dev));
  char arch[64];
  snprintf(arch, sizeof arch, "--gpu-architecture=sm_%d%d%s", maj, mnr, maj >= 9 ? "a" : "");
  const std::string key = std::string(arch) + "\n" + src;
  {
    std::lock_guard<std::mutex> lk(g_jit_mu);
    auto it = g_jit_cache.find(key);
    if (it != g_jit_cache.end()) {
      *out = it->second;
      return AW_OK;
    }
  }
  std::vector<char> cubin;
  TRY(nvrtc_cubin(src, arch, &cubin));
  cudaLibrary_t lib;
  CK(cudaLibraryLoadData(&lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0));
  std::lock_guard<std::mutex> lk(g_jit_mu);
  g_jit_cache[key] = lib;
  *out = lib;
  return AW_OK;
}

static int jit_kernel(cudaLibrary_t lib, const char* name, cudaKernel_t* k) {
  CK(cudaLibraryGetKernel(k, lib, name));
  return AW_OK;
}

static int jit_launch(cudaKernel_t k, dim3 g, dim3 b, void** args, cudaStream_t st) {
  ++g_launches;
  CK(cudaLaunchKernel((const void*)k, g, b, args, 0, st));
  return AW_OK;
}
struct aw_state_s;
static int hjit(aw_state_s* h, cudaKernel_t k, dim3 g, dim3 b, void** args);

// ============================================================================ handle
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

// steps of one captured window of the Wigner-Moyal step loop: as many of a call's steps as fit (even,
// since the branch outputs alternate), from AW_GRAPH_MIN to AW_GRAPH_MAX (its tables and times fit
// the 256 slots of the time-dependent kick tables); AW_GRAPH_CACHE windows are kept per handle
#define AW_GRAPH_MIN 16
#define AW_GRAPH_MAX 248
#define AW_GRAPH_CACHE 4

struct aw_state_s {
  aw_config cfg;
  std::string consts, V, K, absx, absp;
  std::vector<std::string> obs_x, obs_p;
  std::vector<int> tslot, tkind, tidx;
  std::vector<double> tcoef;
  awjit::KindNames kn;
  int kind = 0, f32 = 0, esz = 16;
  int df = 0;                          // complex128 state, passes in double-float arithmetic
  // batches: ni instances (1 for a single propagator), np parameters each; calls act on the
  // view [v0, v0 + vc) and the step loops advance its active instances
  int ni = 1, np = 0, v0 = 0, vc = 1;
  std::vector<std::string> pnames;
  std::string init_expr;
  DevBuf params;                       // ni x np, row-major
  DevBuf bvec;                         // Bloch coefficients per instance: ca_V, shift_V, ca_K, shift_K (4 x ni)
  std::vector<int> active;             // per instance
  std::vector<double> vmin_i, kmin_i;  // Bloch minima per instance
  std::vector<char> minima_ok;
  int col_lines = 0;                   // columns per column-pass block of a batch (fixed, so that an
                                       // instance computes the same way whatever the view)
  int tuned_col_lines = 0;             // ... of the propagation column pass, chosen by timing (tune_col_lines)
  int tuned_col_tma = 0;               // ... and whether its tile is staged by TMA (chosen the same way)
  int tuned_col_shape = 0;             // ... and its elements a thread (AwPassArgs.shape)
  int tuned_row_shape = 0;             // elements a thread of the propagation row pass (tune_row_shape)
  int* err_host = nullptr;             // error word of the pass kernels' bounded waits (mapped pinned memory)
  // the Wigner-Moyal step loop replayed from CUDA graphs of windows of steps (rot_run), captured on
  // first use per (window length, parity of the call's step count), least recently used dropped
  bool graph_on = true;
  cudaGraphExec_t graph_exec[AW_GRAPH_CACHE] = {};
  long long graph_key[AW_GRAPH_CACHE] = {};
  long long graph_used[AW_GRAPH_CACHE] = {};
  long long graph_launches[AW_GRAPH_CACHE] = {};
  long long graph_clock = 0;
  DevBuf hwin;                         // history rows of one window
  // native FP64: tangent-form twiddle tables (aw_fft.cuh) of the lengths of tw_r, tw_c, tw_w, tw_l1, tw_l2
  DevBuf tt_r[2], tt_c[2], tt_w[2], tt_l1[2], tt_l2[2];
  DevBuf ctimes;                       // step times of the current call
  int* err_dev = nullptr;              // ... its device address
  cudaKernel_t k_binit = nullptr;
  // buffers currently holding double-float state (pointer, elements); plain complex128 at rest
  std::vector<std::pair<void*, long long>> df_live;
  int nr = 0, nc = 0;      // main grid rows x cols
  int wn = 0;              // Wigner grid side (VN: 2N; SW: N; WM: same as main)
  cudaStream_t st = nullptr;
  // side stream of the per-step observable reduction of real-time propagation, and its events
  cudaStream_t st2 = nullptr;
  cudaEvent_t ev_z[2] = {nullptr, nullptr}, ev_f[2] = {nullptr, nullptr};
  cudaLibrary_t lib = nullptr;
  cudaKernel_t k_tab = nullptr, k_values = nullptr, k_final = nullptr, k_mask2d = nullptr;
  cudaKernel_t k_final_rot = nullptr;
  std::unordered_map<std::string, cudaKernel_t> obs_kernels;
  // buffers
  DevBuf rho, W, snap, tmp, stage;
  DevBuf tw_r, tw_c, tw_w;            // twiddles: row length (nc), column length (nr), Wigner grid (wn)
  DevBuf shx_hi, shx_lo, shy_hi, shy_lo;
  // native FP64 on grids up to 1024 x 1024: the shear factors of the per-step Wigner transform as full
  // [lines][positions] tables (one complex product a point fewer on the FP64 pipe)
  DevBuf shx_full, shy_full;
  // ... and the column pass's K kick with its 1/N^2 (real time, K independent of t, one instance, no
  // momentum absorber) as one [column][row] table, rebuilt by each propagation call
  DevBuf kfull;
  DevBuf vfull;                        // ... and a V kick that does not change during the call, [row][column]
  DevBuf tabs;                         // phase tables, slots of (nc + nr) complex
  DevBuf vseq, vtimes;                 // time-dependent kick tables of a run of time points, their times
  DevBuf maskx, maskp;                 // 2-D masks (rotated frame)
  DevBuf maskx2;                       // second x mask of a time-dependent absorber (kicks at t_n, t_n+1)
  DevBuf masksep;                      // a separable x mask as column and row factors (nc + nr doubles)
  bool maskx_sep = false;              // ... folded into the V-kick tables instead of read per point
  double maskx_t[2] = {NAN, NAN};      // time of the x mask each buffer holds (time-dependent absorber)
  DevBuf red_line, red_cross, red_sq, rowsum, diag, abs2;
  DevBuf scal;                         // device scalars: [0..1] inv_norm (complex), [2..] misc
  DevBuf stop;                         // int
  DevBuf hist;
  DevBuf terms;                        // term tables for the finalize kernel
  DevBuf part;                         // reduction partials (double2 x 1024)
  DevBuf zbuf, altbuf;                 // rotated-frame marginal inputs (z | w, per-block partials of w)
  int z_lines = 0, z_blocks = 0;       // column pass of the marginals: columns per block, partial rows
  int z_cluster = 1;                   // ... and blocks per cluster
  DevBuf blk_tabs;                     // Blackman tables
  int shx_lo_n = 0, shy_lo_n = 0;
  DevBuf gdiag;                        // von Neumann: diagonal sums G_d of the branch point, then DFT scratch
  int sw_rows = 1;                     // Schrodinger: rows of the zero-padded psi tile
  // Schrodinger wave functions longer than one pass tile: psi read as an sw_n1 x sw_n2 matrix and
  // transformed by the four-step FFT (sw_run); 0 for the single-tile form
  int sw_n1 = 0, sw_n2 = 0;
  DevBuf tw_l1, tw_l2;                 // twiddles of the two factor lengths
  DevBuf swf_hi, swf_lo, swi_hi, swi_lo;  // exp(-+ 2 pi i n2 k1 / N) between the two stages
  int swt_lo_n = 0;
  int red_blocks = 0;                  // column blocks of the Wigner column pass
  long long hist_rows = 0, hist_cap = 0;
  int hist_cols = 0;
  double V_min = 0.0, K_min = 0.0;
  bool maskx_ready = false, maskp_ready = false;
  // Schrodinger stationary states
  std::vector<DevBuf> sw_states;
  // optional per-launch timing (aw_profile)
  struct ProfRec {
    int cls;
    double bytes;
    cudaEvent_t a, b;
  };
  bool prof_on = false;
  bool prof_serial = false;  // side-stream launches go to the handle's stream while profiling
  std::vector<ProfRec> prof;
  // the stream of the work that normally overlaps the next step (the handle's own while the profiler
  // serialises launches, so that every event pair times one kernel alone)
  cudaStream_t side() const { return prof_serial ? st : st2; }
};



// launch classes of the profiler (AW_PROF_CLASSES in awigner.h)
enum { PROF_ROW = 0, PROF_COL = 1, PROF_JIT = 2, PROF_UTIL = 3, PROF_RED = 4, PROF_NCLS = 5 };

static cudaEvent_t prof_mark(aw_state_s* h, cudaStream_t st = nullptr) {
  cudaEvent_t e = nullptr;
  if (!h->prof_on) return e;
  cudaEventCreate(&e);
  cudaEventRecord(e, st ? st : h->st);
  return e;
}
static void prof_done(aw_state_s* h, int cls, double bytes, cudaEvent_t a, cudaStream_t st = nullptr) {
  if (!h->prof_on || !a) return;
  cudaEvent_t b;
  cudaEventCreate(&b);
  cudaEventRecord(b, st ? st : h->st);
  h->prof.push_back({cls, bytes, a, b});
}
static void prof_clear(aw_state_s* h) {
  for (auto& r : h->prof) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  h->prof.clear();
}

// device scalars: [0, 2 ni) 1/norm of each instance (complex), then 16 spare, then the
// finalize partials of each instance (FIN_TV doubles apiece)
static constexpr int FIN_TV = 1088;
static double* dinv(aw_state_s* h, int inst = 0) { return (double*)h->scal.p + 2 * inst; }
static double* dmisc(aw_state_s* h, int k) { return (double*)h->scal.p + 2 * h->ni + k; }
static double* dtv(aw_state_s* h, int inst) { return (double*)h->scal.p + 2 * h->ni + 16 + (size_t)inst * FIN_TV; }
// per-instance stop flags and finalize counters
static int* dstop(aw_state_s* h, int inst = 0) { return (int*)h->stop.p + inst; }
static unsigned int* dcounter(aw_state_s* h, int inst) { return (unsigned int*)h->stop.p + h->ni + inst; }
static long long gsz(const aw_state_s* h) { return (long long)h->nr * h->nc; }
// rows per row-pass block and row-pass blocks per instance for a grid of nrows x ncols: chosen from
// the rows of all instances of the handle, so that every launch of a batch splits rows the same way
static int row_lines(const aw_state_s* h, int nrows, int ncols) {
  return aw_row_pass_lines_for(nrows * h->ni, ncols, h->f32);
}
static int row_blocks(const aw_state_s* h, int nrows, int ncols) { return nrows / row_lines(h, nrows, ncols); }
static void* at_inst(void* base, long long elems, int esz, int inst) {
  return base ? (char*)base + (size_t)inst * elems * esz : nullptr;
}
// scale every instance of the view of `buf` (elems per instance) by its 1/norm
static int vscale(aw_state_s* h, void* buf, long long elems) {
  KL(aw_k_scale_n(at_inst(buf, elems, h->esz, h->v0), h->f32, elems, h->vc, 1.0, 0.0, dinv(h, h->v0), h->st));
  return AW_OK;
}
// reset 1/norm of every instance of the view to 1
static int vinv_reset(aw_state_s* h) {
  KL(aw_k_fill(dinv(h, h->v0), 0, h->vc, 1.0, 0.0, h->st));
  return AW_OK;
}

static int hjit_on(aw_state_s* h, cudaKernel_t k, dim3 g, dim3 b, void** args, cudaStream_t st) {
  cudaEvent_t pe = nullptr;
  if (h->prof_on) {
    cudaEventCreate(&pe);
    cudaEventRecord(pe, st);
  }
  int r = jit_launch(k, g, b, args, st);
  if (pe) {
    cudaEvent_t pb;
    cudaEventCreate(&pb);
    cudaEventRecord(pb, st);
    h->prof.push_back({PROF_JIT, 0.0, pe, pb});
  }
  return r;
}
static int hjit(aw_state_s* h, cudaKernel_t k, dim3 g, dim3 b, void** args) { return hjit_on(h, k, g, b, args, h->st); }

extern "C" int aw_profile(aw_handle h, int32_t enable) {
  if (!h) return fail(AW_E_ARG, "null handle");
  if (enable < 0 || enable > 2) return fail(AW_E_ARG, "aw_profile: mode must be 0, 1 or 2");
  cudaStreamSynchronize(h->st);
  if (h->st2) cudaStreamSynchronize(h->st2);
  prof_clear(h);
  h->prof_on = enable != 0;
  h->prof_serial = enable == 2;
  return AW_OK;
}

extern "C" int aw_profile_read(aw_handle h, double* ms, double* bytes, int64_t* launches) {
  if (!h) return fail(AW_E_ARG, "null handle");
  CK(cudaStreamSynchronize(h->st));
  for (int c = 0; c < PROF_NCLS; ++c) {
    if (ms) ms[c] = 0.0;
    if (bytes) bytes[c] = 0.0;
    if (launches) launches[c] = 0;
  }
  for (auto& r : h->prof) {
    float t = 0.f;
    CK(cudaEventElapsedTime(&t, r.a, r.b));
    if (ms) ms[r.cls] += t;
    if (bytes) bytes[r.cls] += r.bytes;
    if (launches) launches[r.cls] += 1;
  }
  return AW_OK;
}

static void dfree(DevBuf& b) {
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.bytes = 0;
}

static int dalloc(DevBuf& b, size_t bytes) {
  if (b.bytes >= bytes && b.p) return AW_OK;
  dfree(b);
  if (bytes == 0) return AW_OK;
  cudaError_t e = cudaMalloc(&b.p, bytes);
  if (e != cudaSuccess) {
    b.p = nullptr;
    return fail(AW_E_NOMEM, "cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
  }
  b.bytes = bytes;
  return AW_OK;
}

static bool is_pow2(long long n) { return n >= 2 && (n & (n - 1)) == 0; }


static double define_round(double v) {
  // the value a kernel sees after '#define name %.15e' (wigner_moyal_cuda_1d.py:176)
  char buf[64];
  snprintf(buf, sizeof buf, "%.15e", v);
  return strtod(buf, nullptr);
}

// Element format of the tables the passes read: 0 FP64, 1 FP32, 2 double-float
// (each FP64 number as the FP32 pair hi = rn(v), lo = rn(v - hi); a complex entry as
// (re hi, im hi, re lo, im lo)).
static int tab_fmt(const aw_state_s* h) { return h->f32 ? 1 : (h->df ? 2 : 0); }

// Host-to-device copy that has landed when it returns: a pageable cudaMemcpy may return before its
// DMA completes, and the handle's non-blocking streams do not wait for the legacy stream.
static int h2d(void* dst, const void* src, size_t bytes) {
  CK(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
  CK(cudaStreamSynchronize(cudaStreamLegacy));
  return AW_OK;
}

// upload a complex table (interleaved re, im) in table format fmt
static int upload_reals(DevBuf& dst, const std::vector<double>& v, int fmt) {
  const size_t n = v.size();
  TRY(dalloc(dst, n * (fmt == 1 ? 4 : 8)));
  if (n == 0) return AW_OK;
  if (fmt == 0) {
    TRY(h2d(dst.p, v.data(), n * 8));
  } else if (fmt == 1) {
    std::vector<float> g(v.begin(), v.end());
    TRY(h2d(dst.p, g.data(), n * 4));
  } else {
    // complex entries (re, im) as (re hi, im hi, re lo, im lo)
    std::vector<float> g(2 * n);
    for (size_t k = 0; k + 1 < n; k += 2) {
      const float rh = (float)v[k], ih = (float)v[k + 1];
      g[2 * k] = rh;
      g[2 * k + 1] = ih;
      g[2 * k + 2] = (float)(v[k] - (double)rh);
      g[2 * k + 3] = (float)(v[k + 1] - (double)ih);
    }
    TRY(h2d(dst.p, g.data(), n * 8));
  }
  return AW_OK;
}

// twiddle table tw[m] = exp(-2 pi i m / n), built in extended precision
// Tangent-form twiddle table of length n for the native FP64 passes (layout: aw_fft.cuh, tan_off):
// for R in {2, 4, 8}, NS = 1 .. n / 2, k < NS, the entries of w = exp(-2 pi i k / (NS R)) listed there,
// each as t = i^e m (1 + i q) with |q| <= 1, computed in extended precision.
static int make_tan_twiddles(DevBuf* tt, int n) {
  const long double PI = 3.141592653589793238462643383279502884L;
  const size_t count = (size_t)7 * (n - 1);
  std::vector<double> mq(2 * count);
  std::vector<unsigned char> ee(count);
  size_t at = 0;
  for (int ri = 0; ri < 3; ++ri) {
    const int R = 2 << ri;
    for (long long ns = 1; ns < n; ns *= 2)
      for (long long k = 0; k < ns; ++k) {
        const long double base = (long double)k / (long double)(ns * R);  // w = exp(-2 pi i base)
        long double f[4];
        int nf = 0;
        if (R == 8) {
          f[nf++] = 4 * base;
          f[nf++] = 2 * base;
          f[nf++] = base;
          f[nf++] = base + 0.125L;
        } else if (R == 4) {
          f[nf++] = 2 * base;
          f[nf++] = base;
        } else {
          f[nf++] = base;
        }
        for (int j = 0; j < nf; ++j) {
          const long double a = 2.0L * PI * f[j];
          const long double c = cosl(a), sn = -sinl(a);
          long double m, q;
          int e;
          if (fabsl(c) >= fabsl(sn)) {
            m = c;
            q = sn / c;
            e = 0;
          } else {  // c + i s = i s (1 - i c / s)
            m = sn;
            q = -c / sn;
            e = 1;
          }
          mq[2 * at] = (double)m;
          mq[2 * at + 1] = (double)q;
          ee[at] = (unsigned char)e;
          ++at;
        }
      }
  }
  if (at != count) return fail(AW_E_STATE, "tangent twiddle table: %zu entries for %zu", at, count);
  TRY(dalloc(tt[0], mq.size() * sizeof(double)));
  TRY(dalloc(tt[1], ee.size()));
  TRY(h2d(tt[0].p, mq.data(), mq.size() * sizeof(double)));
  TRY(h2d(tt[1].p, ee.data(), ee.size()));
  return AW_OK;
}

static int make_twiddles(DevBuf& dst, int n, int fmt) {
  const long double PI = 3.141592653589793238462643383279502884L;
  std::vector<double> h(2 * (size_t)n);
  for (int m = 0; m < n; ++m) {
    // reduce to the first octant so that the exact points come out exact
    long double c, s;
    if (m == 0) {
      c = 1; s = 0;
    } else if (4LL * m == n) {
      c = 0; s = -1;
    } else if (2LL * m == n) {
      c = -1; s = 0;
    } else if (4LL * m == 3LL * n) {
      c = 0; s = 1;
    } else {
      long double a = 2.0L * PI * (long double)m / (long double)n;
      c = cosl(a);
      s = -sinl(a);
    }
    h[2 * m] = (double)c;
    h[2 * m + 1] = (double)s;
  }
  TRY(upload_reals(dst, h, fmt));
  return AW_OK;
}

// Two-level table of a bilinear phase exp(i alpha_line (q - npos/2)) * norm
// for q = 0..npos-1, split as hi[q / lo] * lo[q % lo].
static int make_shear(DevBuf& hi, DevBuf& lo, int* lo_n, const std::vector<double>& alpha, int npos, double norm,
                      int fmt, double offset = -1.0) {
  if (offset < 0) offset = 0.5 * npos;
  const int LO = npos < 32 ? npos : 32;
  const int nhi = npos / LO;
  const int lines = (int)alpha.size();
  std::vector<double> H(2 * (size_t)lines * nhi), L(2 * (size_t)lines * LO);
  for (int ln = 0; ln < lines; ++ln) {
    const double a = alpha[ln];
    for (int h = 0; h < nhi; ++h) {
      const double ph = a * ((double)(h * LO) - offset);
      H[2 * ((size_t)ln * nhi + h)] = cos(ph) * norm;
      H[2 * ((size_t)ln * nhi + h) + 1] = sin(ph) * norm;
    }
    for (int l = 0; l < LO; ++l) {
      const double ph = a * (double)l;
      L[2 * ((size_t)ln * LO + l)] = cos(ph);
      L[2 * ((size_t)ln * LO + l) + 1] = sin(ph);
    }
  }
  TRY(upload_reals(hi, H, fmt));
  TRY(upload_reals(lo, L, fmt));
  *lo_n = LO;
  return AW_OK;
}

// exp(2 pi i (line * q mod n) / n) / n split as hi[q / lo] * lo[q % lo], exact integer reduction
// exp(sign 2 pi i (line * q mod modulus) / modulus) for lines x npos, split as hi[q / lo] * lo[q % lo]
// (the four-step FFT's twiddles: line = n2, q = k1, modulus = N), exact integer reduction
static int make_twist4(DevBuf& hi, DevBuf& lo, int* lo_n, int lines, int npos, long long modulus, int sign, int fmt) {
  const int LO = npos < 32 ? npos : 32;
  const int nhi = npos / LO;
  const long double PI = 3.141592653589793238462643383279502884L;
  std::vector<double> H(2 * (size_t)lines * nhi), L(2 * (size_t)lines * LO);
  auto put = [&](std::vector<double>& v, size_t k, long long m) {
    const long double a = sign * 2.0L * PI * (long double)m / (long double)modulus;
    v[2 * k] = (double)cosl(a);
    v[2 * k + 1] = (double)sinl(a);
  };
  for (long long ln = 0; ln < lines; ++ln) {
    for (int hh = 0; hh < nhi; ++hh) put(H, (size_t)ln * nhi + hh, (ln * (long long)(hh * LO)) % modulus);
    for (int l = 0; l < LO; ++l) put(L, (size_t)ln * LO + l, (ln * (long long)l) % modulus);
  }
  TRY(upload_reals(hi, H, fmt));
  TRY(upload_reals(lo, L, fmt));
  *lo_n = LO;
  return AW_OK;
}

// ---------------------------------------------------------------- pass helpers
static AwFactor fnone() {
  AwFactor f;
  memset(&f, 0, sizeof f);
  f.scale = 1.0;
  return f;
}
static AwFactor fsign() {
  AwFactor f = fnone();
  f.sign = 1;
  f.active = 1;
  return f;
}
// phase table slots (a batch holds one set per instance)
enum { TAB_V1 = 0, TAB_V1B, TAB_V2, TAB_K, TAB_BV, TAB_BK, TAB_BLK, TAB_NSLOT };

// a pass over the main grid of every instance of the view
static AwPassArgs pnone(const aw_state_s* h) {
  AwPassArgs a;
  memset(&a, 0, sizeof a);
  a.f0 = a.f1 = a.f2 = a.f3 = a.fbr = fnone();
  a.nrows = h->nr;
  a.ncols = h->nc;
  a.batch_elems = (long long)h->nr * h->nc;
  a.batch_tab = (long long)TAB_NSLOT * (h->nc + h->nr);
  a.inst0 = h->v0;
  return a;
}

// algorithmic HBM bytes of one pass: every grid array it reads or writes once
static double pass_bytes(const aw_state_s* h, const AwPassArgs& a) {
  const double n = (double)a.nrows * a.ncols;
  double acc = 1.0 + (a.out ? 1.0 : 0.0) + (a.mid_out ? 1.0 : 0.0) + (a.br_out ? 1.0 : 0.0);
  return n * acc * h->esz;
}

// Double-float state tracking.  With h->df the passes read and write state in the double-float
// form; buffers are converted on their first use by a pass (in place, or into the pass's output
// when it writes elsewhere, so that an input buffer is never altered) and converted back to
// complex128 by settle() before any other kernel or the caller sees them.
static bool df_is_live(const aw_state_s* h, const void* p) {
  for (auto& e : h->df_live)
    if (e.first == p) return true;
  return false;
}
static void df_mark(aw_state_s* h, void* p, long long n) {
  if (!p) return;
  for (auto& e : h->df_live)
    if (e.first == p) {
      e.second = std::max(e.second, n);
      return;
    }
  h->df_live.push_back({p, n});
}
static int settle(aw_state_s* h) {
  for (auto& e : h->df_live) KL(aw_k_convert(e.first, 2, e.first, 0, e.second, h->st));
  h->df_live.clear();
  return AW_OK;
}
// converts back to complex128 when the scope ends (exported entry points that run passes)
struct Settled {
  aw_state_s* h;
  ~Settled() {
    if (h && !h->df_live.empty()) settle(h);
  }
};

// the part of a state buffer a pass touches: the instances [inst0, inst0 + batch) of the view
static void* df_region(const AwPassArgs& a, const void* base) {
  return base ? (char*)base + (size_t)a.inst0 * a.batch_elems * 16 : nullptr;
}
static int df_prepare(aw_state_s* h, AwPassArgs& a, int batch, cudaStream_t st) {
  const long long n = (long long)batch * a.batch_elems;
  void* rin = df_region(a, a.in);
  if (rin && !df_is_live(h, rin)) {
    void* base = a.out ? a.out : (void*)a.in;
    void* dst = df_region(a, base);
    KL(aw_k_convert(rin, 0, dst, 2, n, st));
    a.in = base;
    df_mark(h, dst, n);
  }
  return AW_OK;
}
static void df_outputs(aw_state_s* h, const AwPassArgs& a, int batch) {
  const long long n = (long long)batch * a.batch_elems;
  df_mark(h, df_region(a, a.out), n);
  df_mark(h, df_region(a, a.mid_out), n);
  df_mark(h, df_region(a, a.br_out), n);
}

// The arguments a pass launch of handle h needs beyond its program: twiddle tables, batch stops, row
// lines, the error word, and the double-float conversion of its input (shared by the grouped launch).
static int prep_pass(aw_state_s* h, AwPassArgs& a, const DevBuf& tw, bool row, cudaStream_t st) {
  if (!row && (a.br_out || a.mid_out)) return fail(AW_E_STATE, "column passes have no branch or mid-point store");
  a.tw = tw.p;
  if (!h->df && !h->f32) {
    // the native FP64 passes take the tangent-form table of the same length
    const DevBuf* tt = &tw == &h->tw_r ? h->tt_r
                       : &tw == &h->tw_c ? h->tt_c
                       : &tw == &h->tw_w ? h->tt_w
                       : &tw == &h->tw_l1 ? h->tt_l1
                       : &tw == &h->tw_l2 ? h->tt_l2 : nullptr;
    if (!tt || !tt[0].p) return fail(AW_E_STATE, "no tangent twiddle table for this pass");
    a.twt_mq = tt[0].p;
    a.twt_e = (const unsigned char*)tt[1].p;
  }
  if (h->ni > 1) {
    // every pass of a batch skips the instances that are stopped or inactive, and splits its
    // columns the same way whatever the view
    if (!a.stop) a.stop = dstop(h);
    if (!row && !a.lines_hint) a.lines_hint = h->col_lines;
  }
  if (row && !a.row_lines) a.row_lines = row_lines(h, a.nrows, a.ncols);
  a.err = h->err_dev;
  if (h->df) TRY(df_prepare(h, a, h->vc, st));
  return AW_OK;
}

// `st`: the stream of the launch (the handle's own when null)
static int launch_pass(aw_state_s* h, AwPassArgs& a, const DevBuf& tw, bool row, cudaStream_t st = nullptr) {
  if (!st) st = h->st;
  TRY(prep_pass(h, a, tw, row, st));
  const int batch = h->vc;
  cudaEvent_t pe = prof_mark(h, st);
  int r;
  if (h->df)
    r = row ? aw_launch_row_pass_df(&a, batch, st) : aw_launch_col_pass_df(&a, batch, st);
  else if (h->f32)
    r = row ? aw_launch_row_pass_f32(&a, batch, st) : aw_launch_col_pass_f32(&a, batch, st);
  else
    r = row ? aw_launch_row_pass_f64(&a, batch, st) : aw_launch_col_pass_f64(&a, batch, st);
  const bool reduce_only = !row && !a.out && !a.mid_out && !a.br_out;
  prof_done(h, row ? PROF_ROW : (reduce_only ? PROF_RED : PROF_COL), pass_bytes(h, a) * batch, pe, st);
  ++g_launches;
  if (r == -9) return fail(AW_E_STATE, "%s pass: no kernel of the other shape for %d x %d", row ? "row" : "column",
                          a.nrows, a.ncols);
  if (r)
    return fail(AW_E_CUDA, "%s pass launch failed (%d, %s), grid %d x %d", row ? "row" : "column", r,
                cudaGetErrorString(cudaGetLastError()), a.nrows, a.ncols);
  if (h->df) df_outputs(h, a, batch);
  return AW_OK;
}
static int row_pass(aw_state_s* h, AwPassArgs& a, const DevBuf& tw) { return launch_pass(h, a, tw, true); }
static int col_pass(aw_state_s* h, AwPassArgs& a, const DevBuf& tw, cudaStream_t st = nullptr) {
  return launch_pass(h, a, tw, false, st);
}

static void* tab_col(aw_state_s* h, int slot) { return (char*)h->tabs.p + (size_t)slot * (h->nc + h->nr) * h->esz; }
static void* tab_row(aw_state_s* h, int slot) { return (char*)tab_col(h, slot) + (size_t)h->nc * h->esz; }

// build one table slot: fn 0 = V, 1 = K.  With tlist (device times, count of them), builds count
// tables of times tlist[s] + ta at col/row + s * (nc + nr) elements instead.
// For a batch, the slot's tables of every instance of the view are built, each with its own
// parameters and, given ca_vec / shift_vec (device, one per instance), its own ca and shift.
static int build_tab(aw_state_s* h, int slot, int fn, int mode, double ta, double tb, double ca, double cb,
                     double shift, int maskpow, double tmask, void* col_base = nullptr, const double* tlist = nullptr,
                     int count = 1, const double* ca_vec = nullptr, const double* shift_vec = nullptr) {
  int ncol = h->nc, nrow = h->nr, roll = 0;
  double dcol, drow;
  const aw_config& c = h->cfg;
  if (h->kind == AW_WIGNER_MOYAL || h->kind == AW_WIGNER_BLOCH) {
    dcol = fn == 0 ? c.dXX : c.dPP;
    drow = fn == 0 ? c.dXX_prime : c.dPP_prime;
  } else if (h->kind == AW_SCHRODINGER) {
    nrow = 0;
    dcol = fn == 0 ? c.dX : c.dP;
    roll = fn == 0 ? 0 : ncol / 2;
    drow = 0.0;
  } else {
    dcol = drow = fn == 0 ? c.dX : c.dP;
  }
  long long istride = (long long)TAB_NSLOT * (h->nc + h->nr);
  void* col = col_base ? col_base : at_inst(tab_col(h, slot), istride, h->esz, h->v0);
  void* row = (char*)col + (size_t)h->nc * h->esz;
  int f32 = tab_fmt(h);
  long long tstride = (long long)h->nc + h->nr;
  const double* prm = h->np ? (const double*)h->params.p + (size_t)h->v0 * h->np : nullptr;
  int np = h->np;
  if (ca_vec) ca_vec += h->v0;
  if (shift_vec) shift_vec += h->v0;
  void* args[] = {&col, &row, &f32, &fn, &mode, &ncol, &dcol, &roll, &nrow, &drow,
                  &ta, &tb, &ca, &cb, &shift, &maskpow, &tmask, &tlist, &tstride,
                  &prm, &np, &ca_vec, &shift_vec, &istride};
  const int n = ncol + nrow;
  return hjit(h, h->k_tab, dim3((n + 31) / 32, count, col_base ? 1 : h->vc), dim3(32), args);
}

static int build_mask2d(aw_state_s* h, int which, double t, DevBuf* target = nullptr) {
  DevBuf& m = target ? *target : (which == 0 ? h->maskx : h->maskp);
  void* out = at_inst(m.p, gsz(h), h->f32 ? 4 : 8, h->v0);
  int f32 = tab_fmt(h), nr = h->nr, nc = h->nc;
  double a = h->cfg.dXX, b = h->cfg.dXX_prime, c = h->cfg.dPP, d = h->cfg.dPP_prime;
  const double* prm = h->np ? (const double*)h->params.p + (size_t)h->v0 * h->np : nullptr;
  int np = h->np;
  void* args[] = {&out, &f32, &which, &t, &nr, &nc, &a, &b, &c, &d, &prm, &np};
  return hjit(h, h->k_mask2d, dim3((nc + 127) / 128, nr, h->vc), dim3(128), args);
}

// sum over a buffer (mode as aw_k_partial); result in out[0..1]
static int dsum(aw_state_s* h, const void* p, long long n, int mode, long long stride, double* out) {
  const int nb = 512;
  KL(aw_k_partial(p, h->f32, n, mode, stride, (double2*)h->part.p, nb, h->st));
  std::vector<double> hp(2 * nb);
  CK(cudaMemcpyAsync(hp.data(), h->part.p, hp.size() * 8, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  double sr = 0.0, si = 0.0;
  for (int k = 0; k < nb; ++k) {
    sr += hp[2 * k];
    si += hp[2 * k + 1];
  }
  out[0] = sr;
  out[1] = si;
  return AW_OK;
}


// ============================================================================ creation
// error message setter for the other translation units of the library (C++ linkage, not exported API)
void aw_internal_set_error(const char* msg) { g_err = msg ? msg : ""; }

extern "C" int32_t aw_version(void) { return AW_VERSION; }
extern "C" const char* aw_last_error(void) { return g_err.c_str(); }
extern "C" int64_t aw_launch_count(void) { return g_launches.load(); }

static std::string cstr(const char* s, const char* dflt) { return s ? std::string(s) : std::string(dflt); }

// ============================================================================ tile autotuner
// Columns per block of the propagation column pass (ifft0, phase multiply, fft0), chosen by timing
// every candidate once per (grid, instances, form) in this process.  Wider blocks coalesce the
// strided column loads better, narrower ones put more blocks on the SMs; which wins depends on the
// grid, the batch and the arithmetic form.  The pass has no reductions and every column is
// transformed by the same operations whatever the block width, so the choice never changes a result.
static std::mutex g_tune_mu;
static std::map<std::tuple<int, int, int, int>, int> g_tuned;

static AwFactor fshear_x(aw_state_s* h);
static AwFactor fshear_y(aw_state_s* h);

static int tune_col_lines(aw_state_s* h) {
  if (h->kn.sw) return AW_OK;
  const auto key = std::make_tuple(h->nr, h->nc, h->ni, (h->df ? 2 : (h->f32 ? 1 : 0)) + 4 * h->tuned_col_shape);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tuned.find(key);
    if (it != g_tuned.end()) {
      h->tuned_col_lines = it->second & 0xff;
      h->tuned_col_tma = (it->second >> 8) & 1;
      return AW_OK;
    }
  }
  const int bmax = aw_col_pass_max_lines(h->nr, h->nc, h->f32);
  // candidates: (columns per block) + 256 * (tile staged by TMA), in the column shape chosen for the
  // grid and form (tune_shapes, + 512 when it is the other one); TMA boxes need rows of 16-byte
  // multiples; a width without a kernel of that shape is dropped when it is tried
  std::vector<int> cand;
  const int sh = 512 * h->tuned_col_shape;
  for (int b = 1; b <= bmax; b *= 2) {
    cand.push_back(b + sh);
    if ((b * h->esz) % 16 == 0) cand.push_back(b + 256 + sh);
  }
  int best = cand.empty() ? 1 : cand[0];
  if (cand.size() > 1 || h->tuned_col_shape) {
    CK(cudaMemsetAsync(h->tmp.p, 0, (size_t)h->ni * gsz(h) * h->esz, h->st));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    // three rounds over the candidates, the fastest of each candidate's rounds: single timings
    // early in a process vary with the clocks and picked a slower width every few runs
    std::vector<float> best_of(cand.size(), 0.f);
    for (int round = 0; round < 3; ++round) {
      for (size_t c = 0; c < cand.size(); ++c) {
        AwPassArgs a = pnone(h);
        a.in = a.out = h->tmp.p;
        a.d1 = -1;
        a.f1 = fshear_y(h);  // a table read and two complex multiplies per point, as a phase kick
        a.d2 = +1;
        a.lines_hint = cand[c] & 0xff;
        a.tma = (cand[c] >> 8) & 1;
        a.shape = cand[c] >> 9;
        if (best_of[c] < 0.f) continue;  // no kernel of this shape
        int r = col_pass(h, a, h->tw_c);  // warm-up (first launch of this instantiation)
        if (r == AW_E_STATE) {
          best_of[c] = -1.f;
          continue;
        }
        float ms = 0.f;
        if (!r) {
          cudaEventRecord(e0, h->st);
          for (int k = 0; k < 4 && !r; ++k) r = col_pass(h, a, h->tw_c);
          cudaEventRecord(e1, h->st);
          cudaEventSynchronize(e1);
          cudaEventElapsedTime(&ms, e0, e1);
        }
        if (r) {
          cudaEventDestroy(e0);
          cudaEventDestroy(e1);
          return r;
        }
        if (round == 0 || ms < best_of[c]) best_of[c] = ms;
      }
    }
    size_t bi = cand.size();
    for (size_t c = 0; c < cand.size(); ++c)
      if (best_of[c] >= 0.f && (bi == cand.size() || best_of[c] < best_of[bi])) bi = c;
    if (bi == cand.size()) return fail(AW_E_STATE, "no column-pass kernel for a %d x %d grid", h->nr, h->nc);
    // Native FP64 on a small grid (fewer than two blocks a SM at the fastest width): among the widths
    // within 3 % of the fastest, the one with the most blocks.  Timed alone, one and two columns a
    // block are equal at 256 x 256; inside the step, whose marginal pass and observable reduction
    // overlap the column pass on a second stream, one column a block gave 0.049-0.050 ms a step and
    // two 0.056-0.057 (the double-float form showed no difference).
    int dev = 0, sms = 0;
    if (!h->df && !h->f32 && cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
        (long long)(h->nc / (cand[bi] & 0xff)) * h->ni < 2LL * sms) {
      size_t wi = bi;
      for (size_t c = 0; c < cand.size(); ++c) {
        if (best_of[c] < 0.f || best_of[c] > 1.03f * best_of[bi]) continue;
        const int lc = cand[c] & 0xff, lw = cand[wi] & 0xff;
        if (lc < lw || (lc == lw && best_of[c] < best_of[wi])) wi = c;
      }
      bi = wi;
    }
    best = cand[bi];
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    TRY(settle(h));
  }
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tuned[key] = best;
  h->tuned_col_lines = best & 0xff;
  h->tuned_col_tma = (best >> 8) & 1;
  return AW_OK;
}

// Elements a thread (and so the FFT radix) of the propagation row and column passes, timed once per
// (grid, form) in this process: each pass as ifft, a table kick and fft, in both shapes (where the
// other exists).  A shape changes the FFT's rounding (radix-4 and radix-8 stages round differently),
// so the choice is one per grid and form for the whole process, the same for a single propagator and
// for a batch of any size; columns per block and TMA staging are then tuned per handle.
static std::map<std::tuple<int, int, int>, std::pair<int, int>> g_tuned_shapes;

static int tune_shapes(aw_state_s* h) {
  if (h->kn.sw) return AW_OK;
  const auto key = std::make_tuple(h->nr, h->nc, h->df ? 2 : (h->f32 ? 1 : 0));
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tuned_shapes.find(key);
    if (it != g_tuned_shapes.end()) {
      h->tuned_row_shape = it->second.first;
      h->tuned_col_shape = it->second.second;
      return AW_OK;
    }
  }
  float best_of[2][2] = {{0.f, 0.f}, {0.f, 0.f}};  // [row, column][shape], < 0: no kernel
  CK(cudaMemsetAsync(h->tmp.p, 0, (size_t)gsz(h) * h->esz, h->st));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  int r = AW_OK;
  // launches per timing: at least 4, up to 32 on small grids (a 256^2 pass takes about 10 us, and four
  // of them left the choice to timing noise: the plain 256^2 step measured 0.049 or 0.056 ms by run)
  const long long pts = (long long)h->nr * h->nc;
  const int reps = (int)std::max(4LL, std::min(32LL, (4LL << 20) / std::max(pts, 1LL)));
  for (int round = 0; round < 3 && r == AW_OK; ++round)
    for (int pass = 0; pass < 2 && r == AW_OK; ++pass)
      for (int shape = 0; shape < 2 && r == AW_OK; ++shape) {
        if (best_of[pass][shape] < 0.f) continue;
        const bool row = pass == 0;
        AwPassArgs a = pnone(h);
        a.in = a.out = h->tmp.p;
        a.d1 = -1;
        a.f1 = row ? fshear_x(h) : fshear_y(h);  // a table read and two complex multiplies per point
        a.d2 = +1;
        a.shape = shape;
        if (row) a.row_lines = row_lines(h, h->nr, h->nc);
        r = launch_pass(h, a, row ? h->tw_r : h->tw_c, row);
        if (r == AW_E_STATE) {  // no kernel of this shape for the grid
          best_of[pass][shape] = -1.f;
          r = AW_OK;
          continue;
        }
        float ms = 0.f;
        if (!r) {
          cudaEventRecord(e0, h->st);
          for (int k = 0; k < reps && !r; ++k) r = launch_pass(h, a, row ? h->tw_r : h->tw_c, row);
          cudaEventRecord(e1, h->st);
          cudaEventSynchronize(e1);
          cudaEventElapsedTime(&ms, e0, e1);
        }
        if (round == 0 || ms < best_of[pass][shape]) best_of[pass][shape] = ms;
      }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (r) return r;
  TRY(settle(h));
  // the other shape only when it is clearly faster (3 %): near-equal timings keep the size rule's
  const int row_best = (best_of[0][1] >= 0.f && best_of[0][1] < 0.97f * best_of[0][0]) ? 1 : 0;
  const int col_best = (best_of[1][1] >= 0.f && best_of[1][1] < 0.97f * best_of[1][0]) ? 1 : 0;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tuned_shapes.find(key);  // another handle may have tuned first: its choice stands
  if (it == g_tuned_shapes.end()) it = g_tuned_shapes.emplace(key, std::make_pair(row_best, col_best)).first;
  h->tuned_row_shape = it->second.first;
  h->tuned_col_shape = it->second.second;
  return AW_OK;
}

// Bloch minima of instance i: min over (V(x) + V(x')) = min V(x) + min V(x') since rounding is
// monotone (the reference's V_min / K_min, wigner_bloch_cuda_1d.py:55-92)
// forget the captured step-loop graphs (recaptured on next use)
static void drop_graphs(aw_state_s* h) {
  for (auto& g : h->graph_exec)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}

// The propagation passes' forms (no counterpart in the reference), as chosen by the autotuner:
// form[0] columns per column-pass block, form[1] TMA staging of the column tile, form[2] elements a
// thread of the column pass (0 by the size rule, 1 the other), form[3] the same for the row pass.  Entries
// of `set` below zero keep the current choice; `get` receives the forms in force.
extern "C" int aw_pass_form(aw_handle h, const int32_t* set, int32_t* get) {
  if (!h) return fail(AW_E_ARG, "null handle");
  if (set) {
    const int lines = set[0] > 0 ? set[0] : h->tuned_col_lines;
    const int tma = set[1] >= 0 ? set[1] : h->tuned_col_tma;
    const int bmax = aw_col_pass_max_lines(h->nr, h->nc, h->f32);
    if ((lines & (lines - 1)) || lines > bmax || h->nc % lines)
      return fail(AW_E_ARG, "aw_pass_form: columns per block must be a power of two dividing %d, at most %d", h->nc,
                  bmax);
    if (tma && (lines * h->esz) % 16)
      return fail(AW_E_ARG, "aw_pass_form: TMA boxes need rows of a multiple of 16 bytes (%d columns of %d bytes)",
                  lines, h->esz);
    if (set[2] > 1 || set[3] > 1) return fail(AW_E_ARG, "aw_pass_form: shapes are 0 or 1");
    h->tuned_col_lines = lines;
    h->tuned_col_tma = tma != 0;
    if (set[2] >= 0) h->tuned_col_shape = set[2];
    if (set[3] >= 0) h->tuned_row_shape = set[3];
    drop_graphs(h);  // captured launches carry the old forms
  }
  if (get) {
    get[0] = h->tuned_col_lines;
    get[1] = h->tuned_col_tma;
    get[2] = h->tuned_col_shape;
    get[3] = h->tuned_row_shape;
  }
  return AW_OK;
}

extern "C" int aw_graph(aw_handle h, int32_t enable) {
  if (!h) return fail(AW_E_ARG, "null handle");
  CK(cudaStreamSynchronize(h->st));
  drop_graphs(h);
  h->graph_on = enable != 0;
  return AW_OK;
}

static int bloch_minima(aw_state_s* h, int i) {
  const aw_config* cfg = &h->cfg;
  const int nmax = std::max(h->nr, h->nc);
  TRY(dalloc(h->stage, (size_t)4 * nmax * 8));
  double* d = (double*)h->stage.p;
  const double* prm = h->np ? (const double*)h->params.p + (size_t)i * h->np : nullptr;
  auto eval = [&](int fn, int n, double dx, double* out) -> int {
    void* o = out;
    double tt = cfg->t_initial;
    int np = h->np;
    long long ostride = 0;
    void* args[] = {&o, &fn, &n, &dx, &tt, &prm, &np, &ostride};
    return hjit(h, h->k_values, dim3((n + 255) / 256), dim3(256), args);
  };
  if (h->kind == AW_WIGNER_BLOCH) {
    TRY(eval(0, h->nc, cfg->dXX, d));
    TRY(eval(0, h->nr, cfg->dXX_prime, d + nmax));
    TRY(eval(1, h->nc, cfg->dPP, d + 2 * nmax));
    TRY(eval(1, h->nr, cfg->dPP_prime, d + 3 * nmax));
  } else {
    TRY(eval(0, h->nc, cfg->dX, d));
    TRY(eval(0, h->nr, cfg->dX, d + nmax));
    TRY(eval(1, h->nc, cfg->dP, d + 2 * nmax));
    TRY(eval(1, h->nr, cfg->dP, d + 3 * nmax));
  }
  std::vector<double> hv(4 * (size_t)nmax);
  CK(cudaMemcpyAsync(hv.data(), d, hv.size() * 8, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  double v1 = INFINITY, v2 = INFINITY, k1 = INFINITY, k2 = INFINITY;
  bool knan = false;
  for (int j = 0; j < h->nc; ++j) v1 = std::min(v1, hv[j]);
  for (int r = 0; r < h->nr; ++r) v2 = std::min(v2, hv[nmax + r]);
  for (int j = 0; j < h->nc; ++j) { k1 = std::min(k1, hv[2 * nmax + j]); knan |= !std::isfinite(hv[2 * nmax + j]); }
  for (int r = 0; r < h->nr; ++r) { k2 = std::min(k2, hv[3 * nmax + r]); knan |= !std::isfinite(hv[3 * nmax + r]); }
  double km = k1 + k2;
  if (h->kind == AW_RHO_BLOCH) km = knan ? NAN : 0.0;  // fill_K multiplies a zeroed array (rho_bloch_cuda_1d.py:370)
  h->vmin_i[i] = define_round(v1 + v2);
  h->kmin_i[i] = define_round(km);
  h->minima_ok[i] = 1;
  return AW_OK;
}

// Bloch coefficients of the view's instances for steps of dbeta[k] (k = 0 .. vc-1)
static int upload_bloch(aw_state_s* h, const double* dbeta) {
  std::vector<double> v(4 * (size_t)h->ni);
  CK(cudaMemcpyAsync(v.data(), h->bvec.p, v.size() * 8, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  for (int k = 0; k < h->vc; ++k) {
    const int i = h->v0 + k;
    if (!h->minima_ok[i]) TRY(bloch_minima(h, i));
    v[i] = -0.25 * dbeta[k];
    v[h->ni + i] = 0.5 * h->vmin_i[i];
    v[2 * h->ni + i] = -0.5 * dbeta[k];
    v[3 * h->ni + i] = 0.5 * h->kmin_i[i];
  }
  CK(cudaMemcpyAsync(h->bvec.p, v.data(), v.size() * 8, cudaMemcpyHostToDevice, h->st));
  CK(cudaStreamSynchronize(h->st));
  return AW_OK;
}

// check_only: validate the configuration and stop before the first CUDA call
static int create_impl(const aw_config* cfg, aw_state_s* h, bool check_only = false) {
  h->cfg = *cfg;
  h->kind = cfg->kind;
  if (cfg->precision < AW_C128 || cfg->precision > AW_C128_FP64) return fail(AW_E_ARG, "unknown precision %d", cfg->precision);
  h->f32 = cfg->precision == AW_C64;
  // complex128 runs its passes in double-float arithmetic unless native FP64 is asked for; the
  // one-dimensional Schrodinger propagator keeps FP64 (its passes are launch-bound, not FP64-bound)
  h->df = cfg->precision == AW_C128 && cfg->kind != AW_SCHRODINGER;
  h->esz = h->f32 ? 8 : 16;
  h->consts = cstr(cfg->cuda_consts, "");
  h->V = cstr(cfg->V, "0.");
  h->K = cstr(cfg->K, "0.");
  h->absx = cstr(cfg->abs_boundary_x, "1.");
  h->absp = cstr(cfg->abs_boundary_p, "1.");
  for (int k = 0; k < cfg->n_obs_x; ++k) h->obs_x.push_back(cfg->obs_x[k]);
  for (int k = 0; k < cfg->n_obs_p; ++k) h->obs_p.push_back(cfg->obs_p[k]);
  for (int k = 0; k < cfg->n_terms; ++k) {
    h->tslot.push_back(cfg->term_slot[k]);
    h->tkind.push_back(cfg->term_kind[k]);
    h->tidx.push_back(cfg->term_index[k]);
    h->tcoef.push_back(cfg->term_coef[k]);
  }
  if (cfg->n_terms > 64) return fail(AW_E_ARG, "at most 64 observable terms");
  // every term adds into a slot of its history row, from an expression that exists
  for (int k = 0; k < cfg->n_terms; ++k) {
    const int kind = cfg->term_kind[k], idx = cfg->term_index[k];
    if (cfg->term_slot[k] < 0 || cfg->term_slot[k] >= cfg->n_slots)
      return fail(AW_E_ARG, "observable term %d: slot %d outside 0..%d", k, cfg->term_slot[k], cfg->n_slots - 1);
    if ((kind != AW_TERM_X && kind != AW_TERM_P) || idx < 0 ||
        idx >= (kind == AW_TERM_X ? cfg->n_obs_x : cfg->n_obs_p))
      return fail(AW_E_ARG, "observable term %d: kind %d, index %d has no expression", k, kind, idx);
  }
  h->kn.rotated = h->kind == AW_WIGNER_MOYAL || h->kind == AW_WIGNER_BLOCH;
  h->kn.vn = h->kind == AW_RHO_VNEUMANN || h->kind == AW_RHO_BLOCH;
  h->kn.sw = h->kind == AW_SCHRODINGER;
  if (h->kind < 0 || h->kind > 4) return fail(AW_E_ARG, "unknown propagator kind %d", h->kind);
  const int N = cfg->x_grid_dim;
  if (!is_pow2(N)) return fail(AW_E_ARG, "Coordinate grid size (X_gridDIM) must be a power of two");
  if (h->kn.rotated) {
    if (!is_pow2(cfg->p_grid_dim)) return fail(AW_E_ARG, "Momentum grid size (P_gridDIM) must be a power of two");
    h->nr = cfg->p_grid_dim;
    h->nc = N;
    h->wn = 0;
  } else if (h->kn.vn) {
    h->nr = h->nc = N;
    h->wn = 2 * N;
  } else {
    h->nr = 1;
    h->nc = N;
    h->wn = N;
    if (N > 8192) {
      // longer than one pass tile: an N1 x N2 matrix, N1 <= N2 <= 8192 (no N x N Wigner grid)
      int n1 = 1;
      while ((long long)n1 * n1 * 4 <= N) n1 *= 2;
      h->sw_n1 = n1;
      h->sw_n2 = N / n1;
      h->wn = 0;
      if (h->sw_n2 > 8192) return fail(AW_E_ARG, "wave functions up to 2^25 points");
    } else {
      h->sw_rows = aw_row_pass_lines(N, h->f32);
      if (h->sw_rows <= 0) return fail(AW_E_ARG, "unsupported wave-function length %d", N);
    }
  }
  const int maxn = h->kn.sw ? (1 << 25) : 8192;
  if (h->nc < 32 || h->nc > maxn || (!h->kn.sw && (h->nr < 32 || h->nr > maxn)) || (h->wn && h->wn > 8192))
    return fail(AW_E_ARG, "grid sides must be powers of two in [32, %d] (Wigner grid up to 8192)", maxn);

  // batch
  h->ni = std::max(1, (int)cfg->n_inst);
  h->np = std::max(0, (int)cfg->n_params);
  h->v0 = 0;
  h->vc = h->ni;
  for (int k = 0; k < h->np; ++k) {
    const char* nm = cfg->param_names ? cfg->param_names[k] : nullptr;
    if (!nm || !*nm) return fail(AW_E_ARG, "parameter %d has no name", k);
    static const char* reserved[] = {"X", "P", "XX", "XX_prime", "PP", "PP_prime", "X_prime", "P_prime", "t", "i",
                                     "j", "dX", "dP", "M_PI"};
    for (const char* r : reserved)
      if (!strcmp(nm, r)) return fail(AW_E_ARG, "parameter name %s is taken by the kernels", nm);
    for (const char* c = nm; *c; ++c)
      if (!(isalnum((unsigned char)*c) || *c == '_') || (c == nm && isdigit((unsigned char)*c)))
        return fail(AW_E_ARG, "parameter name %s is not an identifier", nm);
    h->pnames.push_back(nm);
  }
  h->init_expr = cstr(cfg->init_expr, "");
  if (h->ni > 1) {
    if (h->kn.sw) return fail(AW_E_ARG, "batches exist for the Wigner-Moyal, Wigner-Bloch, von Neumann and rho-Bloch propagators");
    if (cfg->v_time_dependent || cfg->k_time_dependent || cfg->absx_mode == 2 || cfg->absp_mode == 2)
      return fail(AW_E_ARG, "a batch needs V, K and absorbing boundaries that do not depend on t");
    if (h->kn.vn && cfg->ehrenfest)
      return fail(AW_E_ARG, "von Neumann batches record trace and purity only (no per-step Ehrenfest observables)");
  }
  if (check_only) return AW_OK;
  h->active.assign(h->ni, 1);
  h->vmin_i.assign(h->ni, 0.0);
  h->kmin_i.assign(h->ni, 0.0);
  h->minima_ok.assign(h->ni, 0);

  CK(cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking));
  // graph windows by default where launch latency is a large part of a step (measured on GB300 with
  // Ehrenfest observables: 256^2 complex64 -26 %, native FP64 -19 %, double-float +-1 %; at 1024^2
  // within 1 % for complex128 and 5 % slower for complex64)
  h->graph_on = (long long)h->nr * h->nc <= 512LL * 512;
  CK(cudaHostAlloc((void**)&h->err_host, sizeof(int), cudaHostAllocMapped));
  *h->err_host = 0;
  CK(cudaHostGetDevicePointer((void**)&h->err_dev, h->err_host, 0));
  if (h->kn.rotated) {
    CK(cudaStreamCreateWithFlags(&h->st2, cudaStreamNonBlocking));
    for (int k = 0; k < 2; ++k) {
      CK(cudaEventCreateWithFlags(&h->ev_z[k], cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&h->ev_f[k], cudaEventDisableTiming));
    }
  }

  // user module
  std::string src = awjit::module_source(h->kn, h->consts, h->V, h->K, h->absx, h->absp, h->obs_x, h->obs_p,
                                         h->pnames, h->init_expr);
  TRY(jit_compile(src, &h->lib));
  TRY(jit_kernel(h->lib, "aw_tab", &h->k_tab));
  if (!h->init_expr.empty()) TRY(jit_kernel(h->lib, "aw_binit", &h->k_binit));
  TRY(jit_kernel(h->lib, "aw_values", &h->k_values));
  TRY(jit_kernel(h->lib, "aw_finalize", &h->k_final));
  if (h->kn.rotated) {
    TRY(jit_kernel(h->lib, "aw_mask2d", &h->k_mask2d));
    TRY(jit_kernel(h->lib, "aw_finalize_rot", &h->k_final_rot));
  }

  // buffers
  const size_t ni = h->ni;
  const size_t grid = (size_t)(h->kn.sw ? h->sw_rows : h->nr) * h->nc;
  // Wigner grid; for a long wave function (no Wigner grid) a psi-sized scratch
  const size_t wgrid = h->kn.rotated ? grid : std::max((size_t)h->wn * h->wn, h->kn.sw ? grid : (size_t)0);
  TRY(dalloc(h->rho, ni * grid * h->esz));
  TRY(dalloc(h->W, ni * wgrid * h->esz));
  TRY(dalloc(h->tmp, std::max(ni * grid, wgrid) * 16));
  CK(cudaMemsetAsync(h->rho.p, 0, ni * grid * h->esz, h->st));
  CK(cudaMemsetAsync(h->W.p, 0, ni * wgrid * h->esz, h->st));
  TRY(dalloc(h->tabs, ni * TAB_NSLOT * (h->nc + h->nr) * h->esz));
  const size_t nscal = 2 * ni + 16 + ni * FIN_TV;
  TRY(dalloc(h->scal, nscal * sizeof(double)));
  TRY(dalloc(h->stop, 2 * ni * sizeof(int)));
  TRY(dalloc(h->part, 1024 * sizeof(double2)));
  CK(cudaMemsetAsync(h->scal.p, 0, nscal * sizeof(double), h->st));
  CK(cudaMemsetAsync(h->stop.p, 0, 2 * ni * sizeof(int), h->st));
  TRY(dalloc(h->bvec, 4 * ni * sizeof(double)));
  CK(cudaMemsetAsync(h->bvec.p, 0, 4 * ni * sizeof(double), h->st));
  if (h->np) {
    TRY(dalloc(h->params, ni * h->np * sizeof(double)));
    CK(cudaMemsetAsync(h->params.p, 0, ni * h->np * sizeof(double), h->st));
  }
  {
    // term tables: int slot[64], kind[64], idx[64], double coef[64]
    TRY(dalloc(h->terms, 64 * 3 * sizeof(int) + 64 * sizeof(double)));
    std::vector<int> ti(64 * 3, 0);
    std::vector<double> tc(64, 0.0);
    for (int k = 0; k < cfg->n_terms; ++k) {
      ti[k] = h->tslot[k];
      ti[64 + k] = h->tkind[k];
      ti[128 + k] = h->tidx[k];
      tc[k] = h->tcoef[k];
    }
    TRY(h2d(h->terms.p, ti.data(), ti.size() * sizeof(int)));
    TRY(h2d((char*)h->terms.p + 64 * 3 * sizeof(int), tc.data(), tc.size() * 8));
  }

  // twiddles
  if (h->sw_n1) {
    TRY(make_twiddles(h->tw_l1, h->sw_n1, tab_fmt(h)));
    TRY(make_twiddles(h->tw_l2, h->sw_n2, tab_fmt(h)));
    if (tab_fmt(h) == 0) {
      TRY(make_tan_twiddles(h->tt_l1, h->sw_n1));
      TRY(make_tan_twiddles(h->tt_l2, h->sw_n2));
    }
    TRY(make_twist4(h->swf_hi, h->swf_lo, &h->swt_lo_n, h->sw_n2, h->sw_n1, N, -1, tab_fmt(h)));
    TRY(make_twist4(h->swi_hi, h->swi_lo, &h->swt_lo_n, h->sw_n2, h->sw_n1, N, +1, tab_fmt(h)));
  } else {
    TRY(make_twiddles(h->tw_r, h->nc, tab_fmt(h)));
    if (tab_fmt(h) == 0) TRY(make_tan_twiddles(h->tt_r, h->nc));
  }
  if (!h->kn.sw) TRY(make_twiddles(h->tw_c, h->nr, tab_fmt(h)));
  if (h->wn) TRY(make_twiddles(h->tw_w, h->wn, tab_fmt(h)));
  if (tab_fmt(h) == 0) {
    if (!h->kn.sw) TRY(make_tan_twiddles(h->tt_c, h->nr));
    if (h->wn) TRY(make_tan_twiddles(h->tt_w, h->wn));
  }

  // shear tables of the Wigner transform
  const double a_shx = tan(M_PI / 8.0);   // phase_shearX: a = tan(theta / 2)
  const double b_shy = -sin(M_PI / 4.0);  // phase_shearY: b = -sin(theta)
  if (h->kn.rotated) {
    // wigner_moyal_cuda_1d.py:639-670: X shear phase -a PP_j XX'_i / Nx (row i, position j),
    // Y shear phase -b PP'_i XX_j / Np (column j, position i)
    std::vector<double> ax(h->nr), ay(h->nc);
    for (int i = 0; i < h->nr; ++i) ax[i] = -a_shx * cfg->dPP * (cfg->dXX_prime * ((double)i - 0.5 * h->nr));
    for (int j = 0; j < h->nc; ++j) ay[j] = -b_shy * cfg->dPP_prime * (cfg->dXX * ((double)j - 0.5 * h->nc));
    TRY(make_shear(h->shx_hi, h->shx_lo, &h->shx_lo_n, ax, h->nc, 1.0 / h->nc, tab_fmt(h)));
    TRY(make_shear(h->shy_hi, h->shy_lo, &h->shy_lo_n, ay, h->nr, 1.0 / h->nr, tab_fmt(h)));
    if (tab_fmt(h) == 0 && (long long)h->nr * h->nc <= 1024LL * 1024) {
      // X shear: nr lines (rows) of nc positions; Y shear: nc lines (columns) of nr positions
      TRY(dalloc(h->shx_full, (size_t)h->nr * h->nc * 16));
      TRY(dalloc(h->shy_full, (size_t)h->nr * h->nc * 16));
      KL(aw_k_shear_full(h->shx_hi.p, h->shx_lo.p, h->shx_lo_n, h->nr, h->nc, h->shx_full.p, h->st));
      KL(aw_k_shear_full(h->shy_hi.p, h->shy_lo.p, h->shy_lo_n, h->nc, h->nr, h->shy_full.p, h->st));
    }
  } else if (h->kn.vn) {
    // rho_vneumann_cuda_1d.py:608-639 on the padded (2N)^2 grid, dXX = dX
    const int M = h->wn;
    std::vector<double> ax(M), ay(M);
    for (int i = 0; i < M; ++i) ax[i] = -a_shx * cfg->dPP * (cfg->dX * ((double)i - 0.5 * M));
    for (int j = 0; j < M; ++j) ay[j] = -b_shy * cfg->dPP * (cfg->dX * ((double)j - 0.5 * M));
    TRY(make_shear(h->shx_hi, h->shx_lo, &h->shx_lo_n, ax, M, 1.0 / M, tab_fmt(h)));
    TRY(make_shear(h->shy_hi, h->shy_lo, &h->shy_lo_n, ay, M, 1.0 / M, tab_fmt(h)));
  } else if (h->wn) {
    // schrodinger_wigner_cuda_1d.py:695-726: P is fft-shifted along the sheared axis
    const int M = h->wn;
    std::vector<double> ax(M), ay(M);
    for (int i = 0; i < M; ++i) ax[i] = -a_shx * cfg->dP * (cfg->dX * ((double)i - 0.5 * M));
    for (int j = 0; j < M; ++j) ay[j] = -b_shy * cfg->dP * (cfg->dX * ((double)j - 0.5 * M));
    TRY(make_shear(h->shx_hi, h->shx_lo, &h->shx_lo_n, ax, M, 1.0 / M, tab_fmt(h)));
    TRY(make_shear(h->shy_hi, h->shy_lo, &h->shy_lo_n, ay, M, 1.0 / M, tab_fmt(h)));
  }

  if (h->kn.vn) TRY(dalloc(h->gdiag, 2 * (size_t)h->nc * 16));

  // reduction scratch of the Wigner column pass
  const int wr = h->kn.rotated ? h->nr : (h->wn ? h->wn : 32), wc = h->kn.rotated ? h->nc : (h->wn ? h->wn : 32);
  h->red_blocks = aw_col_pass_blocks(wr, wc, h->f32);
  if (h->ni > 1) {
    // a batch splits its columns the same way in every launch, chosen for the full batch
    h->col_lines = aw_col_pass_lines(h->nr, h->nc, h->ni, h->f32);
    if (h->col_lines <= 0) return fail(AW_E_ARG, "unsupported batch grid %d x %d", h->nr, h->nc);
    if (h->kn.rotated) h->red_blocks = h->nc / h->col_lines;
  }
  if (h->red_blocks <= 0) return fail(AW_E_ARG, "unsupported Wigner grid %d x %d", wr, wc);
  // per-instance reduction scratch (the pass kernels index it by instance)
  // (a wave function's marginals |psi|^2 and |fft psi|^2 also use red_line / red_cross)
  TRY(dalloc(h->red_line, std::max(ni * (size_t)wc, h->kn.sw ? (size_t)N : 0) * 8));
  TRY(dalloc(h->red_cross, std::max(ni * (size_t)h->red_blocks * wr, h->kn.sw ? (size_t)N : 0) * 8));
  TRY(dalloc(h->red_sq, ni * (size_t)h->red_blocks * 8));
  TRY(dalloc(h->rowsum, std::max((size_t)std::max(wr, wc), h->kn.sw ? (size_t)N : 0) * 8));  // finalize: one per row
  TRY(dalloc(h->diag, ni * (size_t)std::max(h->nr, h->nc) * 16));
  // per-block norm partials: two parities (rot_run); a long wave function's column passes use up to N2
  TRY(dalloc(h->abs2, 2 * ni * (size_t)std::max(std::max(h->nr, 1), h->sw_n2) * 8));
  if (h->kn.rotated) {
    // the marginal column pass: narrow slabs spread over every SM, row partials summed across
    // clusters of 4 blocks in distributed shared memory, so that z_blocks stays small
    h->z_lines = std::min(2, aw_col_pass_max_lines(h->nr, h->nc, h->f32));
    const size_t z_smem = (size_t)h->nr * h->z_lines * h->esz + (size_t)h->nr * 16;
    h->z_cluster = (h->nc / h->z_lines) % 4 == 0 && h->nr % 4 == 0 && z_smem <= 160 * 1024 ? 4 : 1;
    h->z_blocks = h->nc / h->z_lines / h->z_cluster;
    // two parities, so that step n's reduction can run while step n + 1 writes the other
    TRY(dalloc(h->zbuf, 2 * ni * (size_t)(h->nc + h->nr) * 16));
    TRY(dalloc(h->altbuf, 2 * ni * (size_t)h->z_blocks * h->nr * 16));
  }

  // 2-D absorbing masks of the rotated frame (one per instance)
  if (h->kn.rotated) {
    if (cfg->absx_mode) TRY(dalloc(h->maskx, ni * grid * (h->f32 ? 4 : 8)));
    if (cfg->absx_mode == 2) TRY(dalloc(h->maskx2, ni * grid * (h->f32 ? 4 : 8)));
    if (cfg->absp_mode) TRY(dalloc(h->maskp, ni * grid * (h->f32 ? 4 : 8)));
  }

  TRY(tune_shapes(h));
  TRY(tune_col_lines(h));

  if (h->kind == AW_WIGNER_BLOCH || h->kind == AW_RHO_BLOCH) {
    // minima of every instance (a batch recomputes an instance's after aw_set_params)
    for (int i = 0; i < h->ni; ++i) TRY(bloch_minima(h, i));
    h->V_min = h->vmin_i[0];
    h->K_min = h->kmin_i[0];
  }
  CK(cudaStreamSynchronize(h->st));
  return AW_OK;
}

extern "C" int aw_create(const aw_config* cfg, aw_handle* out) {
  if (!cfg || !out) return fail(AW_E_ARG, "null argument");
  aw_state_s* h = new aw_state_s();
  int r = create_impl(cfg, h);
  if (r) {
    std::string keep = g_err;
    aw_destroy(h);
    g_err = keep;
    return r;
  }
  *out = h;
  return AW_OK;
}

extern "C" int aw_check_config(const aw_config* cfg, const char* arch) {
  if (!cfg) return fail(AW_E_ARG, "null argument");
  std::unique_ptr<aw_state_s> h(new aw_state_s());
  TRY(create_impl(cfg, h.get(), true));
  const std::string opt = std::string("--gpu-architecture=") + (arch && *arch ? arch : "sm_103a");
  std::vector<char> cubin;
  TRY(nvrtc_cubin(awjit::module_source(h->kn, h->consts, h->V, h->K, h->absx, h->absp, h->obs_x, h->obs_p,
                                       h->pnames, h->init_expr),
                  opt.c_str(), &cubin));
  TRY(nvrtc_cubin(awjit::init_source(h->kn, h->consts, "1."), opt.c_str(), &cubin));
  TRY(nvrtc_cubin(awjit::observable_source(h->kn, h->consts, "X"), opt.c_str(), &cubin));
  return AW_OK;
}

extern "C" int aw_destroy(aw_handle h) {
  if (!h) return AW_OK;
  if (h->st) cudaStreamSynchronize(h->st);
  DevBuf* bufs[] = {&h->tw_l1, &h->tw_l2, &h->swf_hi, &h->swf_lo, &h->swi_hi, &h->swi_lo,
                    &h->vseq, &h->vtimes, &h->zbuf, &h->altbuf, &h->gdiag, &h->rho, &h->W, &h->snap, &h->tmp, &h->stage, &h->tw_r, &h->tw_c, &h->tw_w, &h->shx_hi,
                    &h->shx_lo, &h->shy_hi, &h->shy_lo, &h->tabs, &h->maskx, &h->maskp, &h->red_line,
                    &h->red_cross, &h->red_sq, &h->rowsum, &h->diag, &h->abs2, &h->scal, &h->stop, &h->hist,
                    &h->terms, &h->part, &h->blk_tabs, &h->params, &h->bvec, &h->maskx2, &h->masksep,
                    &h->hwin, &h->ctimes, &h->tt_r[0], &h->tt_r[1], &h->tt_c[0], &h->tt_c[1], &h->tt_w[0],
                    &h->tt_w[1], &h->tt_l1[0], &h->tt_l1[1], &h->tt_l2[0], &h->tt_l2[1], &h->shx_full,
                    &h->shy_full, &h->kfull, &h->vfull};
  for (DevBuf* b : bufs) dfree(*b);
  for (DevBuf& b : h->sw_states) dfree(b);
  for (auto& g : h->graph_exec)
    if (g) cudaGraphExecDestroy(g);
  if (h->st) cudaStreamDestroy(h->st);
  if (h->err_host) cudaFreeHost(h->err_host);
  if (h->st2) {
    cudaStreamSynchronize(h->st2);
    cudaStreamDestroy(h->st2);
  }
  for (int k = 0; k < 2; ++k) {
    if (h->ev_z[k]) cudaEventDestroy(h->ev_z[k]);
    if (h->ev_f[k]) cudaEventDestroy(h->ev_f[k]);
  }
  prof_clear(h);
  delete h;
  return AW_OK;
}

extern "C" int aw_stream(aw_handle h, void** stream) {
  if (!h || !stream) return fail(AW_E_ARG, "null argument");
  *stream = h->st;
  return AW_OK;
}

// A pass kernel whose bounded wait ran out (its TMA copies did not arrive) records a code in the
// handle's error word and skips its tile; the next call that synchronises reports it.
static int check_err(aw_state_s* h) {
  if (!h->err_host) return AW_OK;
  const int code = *(volatile int*)h->err_host;
  if (!code) return AW_OK;
  *(volatile int*)h->err_host = 0;
  return fail(AW_E_CUDA, "a pass kernel's bounded wait for its TMA tile copies ran out (code %d); the results of "
                         "the call that launched it are incomplete", code);
}

extern "C" int aw_sync(aw_handle h) {
  if (!h) return fail(AW_E_ARG, "null handle");
  CK(cudaStreamSynchronize(h->st));
  return check_err(h);
}

extern "C" int aw_bloch_min(aw_handle h, double* v_min, double* k_min) {
  if (!h) return fail(AW_E_ARG, "null handle");
  if (v_min) *v_min = h->V_min;
  if (k_min) *k_min = h->K_min;
  return AW_OK;
}

// ============================================================================ buffers
// A state buffer of the view: pointer to its first instance's data, rows = view instances x rows
// of one instance.  *base (optional) receives the whole buffer.
static void* buf_of(aw_state_s* h, int which, long long* rows, long long* cols, DevBuf** base = nullptr) {
  DevBuf* b = nullptr;
  long long r = 0, c = 0;
  switch (which) {
    case AW_BUF_RHO:
    case AW_BUF_PSI:
      if ((which == AW_BUF_PSI) != h->kn.sw) return nullptr;
      r = h->nr;
      c = h->nc;
      b = &h->rho;
      break;
    case AW_BUF_WIGNER:
      r = h->kn.rotated ? h->nr : h->wn;
      c = h->kn.rotated ? h->nc : h->wn;
      b = &h->W;
      break;
    case AW_BUF_SNAPSHOT:
      r = h->nr;
      c = h->nc;
      b = &h->snap;
      break;
    default:
      return nullptr;
  }
  if (base) *base = b;
  *rows = r * h->vc;
  *cols = c;
  if (!b->p) return nullptr;  // the snapshot before its first write
  return at_inst(b->p, r * c, h->esz, h->v0);
}

static int clear_stops(aw_state_s* h);

// snapshot storage for every instance, allocated on first use
static int ensure_snap(aw_state_s* h) {
  if (h->snap.p) return AW_OK;
  TRY(dalloc(h->snap, (size_t)h->ni * gsz(h) * h->esz));
  CK(cudaMemsetAsync(h->snap.p, 0, (size_t)h->ni * gsz(h) * h->esz, h->st));
  return AW_OK;
}

extern "C" int aw_buffer(aw_handle h, int32_t which, void** dptr, int64_t* rows, int64_t* cols, int32_t* elem_bytes) {
  if (!h) return fail(AW_E_ARG, "null handle");
  long long r, c;
  if (which == AW_BUF_SNAPSHOT) TRY(ensure_snap(h));
  void* p = buf_of(h, which, &r, &c);
  if (!p) return fail(AW_E_ARG, "no buffer %d for this propagator", which);
  if (dptr) *dptr = p;
  if (rows) *rows = r;
  if (cols) *cols = c;
  if (elem_bytes) *elem_bytes = h->esz;
  return AW_OK;
}

extern "C" int aw_set_buffer(aw_handle h, int32_t which, const void* src, int32_t src_on_device) {
  if (!h || !src) return fail(AW_E_ARG, "null argument");
  long long r, c;
  if (which == AW_BUF_SNAPSHOT) TRY(ensure_snap(h));
  void* b = buf_of(h, which, &r, &c);
  if (!b) return fail(AW_E_ARG, "no buffer %d for this propagator", which);
  const size_t n = (size_t)r * c;
  if (!h->f32) {
    CK(cudaMemcpyAsync(b, src, n * 16, src_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, h->st));
  } else {
    for (size_t off = 0; off < n;) {
      // through the complex128 scratch, at most its size at a time
      const size_t m = std::min(n - off, h->tmp.bytes / 16);
      CK(cudaMemcpyAsync(h->tmp.p, (const char*)src + off * 16, m * 16,
                         src_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, h->st));
      KL(aw_k_convert(h->tmp.p, 0, (char*)b + off * 8, 1, (long long)m, h->st));
      off += m;
    }
  }
  CK(cudaStreamSynchronize(h->st));
  return AW_OK;
}

extern "C" int aw_get_buffer(aw_handle h, int32_t which, void* dst, int32_t dst_on_device) {
  if (!h || !dst) return fail(AW_E_ARG, "null argument");
  long long r, c;
  void* b = buf_of(h, which, &r, &c);
  if (!b) return fail(AW_E_ARG, "no buffer %d for this propagator", which);
  const size_t n = (size_t)r * c;
  if (!h->f32) {
    CK(cudaMemcpyAsync(dst, b, n * 16, dst_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, h->st));
  } else {
    for (size_t off = 0; off < n;) {
      const size_t m = std::min(n - off, h->tmp.bytes / 16);
      KL(aw_k_convert((char*)b + off * 8, 1, h->tmp.p, 0, (long long)m, h->st));
      CK(cudaMemcpyAsync((char*)dst + off * 16, h->tmp.p, m * 16,
                         dst_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, h->st));
      off += m;
    }
  }
  CK(cudaStreamSynchronize(h->st));
  return check_err(h);
}

extern "C" int aw_copy_buffer(aw_handle h, int32_t from, int32_t to) {
  if (!h) return fail(AW_E_ARG, "null handle");
  long long r1, c1, r2, c2;
  if (to == AW_BUF_SNAPSHOT) TRY(ensure_snap(h));
  void* a = buf_of(h, from, &r1, &c1);
  void* b = buf_of(h, to, &r2, &c2);
  if (!a || !b || r1 * c1 != r2 * c2) return fail(AW_E_ARG, "incompatible or empty buffers %d -> %d", from, to);
  CK(cudaMemcpyAsync(b, a, (size_t)r1 * c1 * h->esz, cudaMemcpyDeviceToDevice, h->st));
  return AW_OK;
}

extern "C" int aw_fill_const(aw_handle h, int32_t which, double re, double im) {
  if (!h) return fail(AW_E_ARG, "null handle");
  long long r, c;
  if (which == AW_BUF_SNAPSHOT) TRY(ensure_snap(h));
  void* b = buf_of(h, which, &r, &c);
  if (!b) return fail(AW_E_ARG, "no buffer %d", which);
  KL(aw_k_fill(b, h->f32, r * c, re, im, h->st));
  return AW_OK;
}

extern "C" int aw_fill_expr(aw_handle h, int32_t which, const char* expr) {
  if (!h || !expr) return fail(AW_E_ARG, "null argument");
  long long r, c;
  if (which == AW_BUF_SNAPSHOT) TRY(ensure_snap(h));
  void* b = buf_of(h, which, &r, &c);
  if (!b) return fail(AW_E_ARG, "no buffer %d", which);
  cudaLibrary_t lib;
  TRY(jit_compile(awjit::init_source(h->kn, h->consts, expr), &lib));
  cudaKernel_t k;
  TRY(jit_kernel(lib, "aw_init", &k));
  int f32 = h->f32, nr = (int)(r / h->vc), nc = (int)c;
  double dX = h->cfg.dX, dP = h->cfg.dP;
  for (int q = 0; q < h->vc; ++q) {
    void* out = (char*)b + (size_t)q * nr * nc * h->esz;
    void* args[] = {&out, &f32, &nr, &nc, &dX, &dP};
    TRY(hjit(h, k, dim3((nc + 127) / 128, h->kn.sw ? 1 : nr), dim3(128), args));
  }
  return AW_OK;
}

extern "C" int aw_sum(aw_handle h, int32_t which, double* re, double* im) {
  if (!h) return fail(AW_E_ARG, "null handle");
  long long r, c;
  void* b = buf_of(h, which, &r, &c);
  if (!b) return fail(AW_E_ARG, "no buffer %d", which);
  double s[2];
  TRY(dsum(h, b, r * c, 0, 0, s));
  if (re) *re = s[0];
  if (im) *im = s[1];
  return AW_OK;
}

extern "C" int aw_trace(aw_handle h, double* re, double* im) {
  if (!h) return fail(AW_E_ARG, "null handle");
  if (h->nr != h->nc) return fail(AW_E_STATE, "trace of a non-square grid");
  double s[2];
  TRY(dsum(h, at_inst(h->rho.p, gsz(h), h->esz, h->v0), h->nr, 3, h->nc + 1, s));
  if (re) *re = s[0];
  if (im) *im = s[1];
  return AW_OK;
}

extern "C" int aw_scale(aw_handle h, int32_t which, double re, double im) {
  if (!h) return fail(AW_E_ARG, "null handle");
  long long r, c;
  void* b = buf_of(h, which, &r, &c);
  if (!b) return fail(AW_E_ARG, "no buffer %d", which);
  KL(aw_k_scale(b, h->f32, r * c, re, im, nullptr, h->st));
  return AW_OK;
}

// ============================================================================ Wigner transforms
// rotated frame, W -> rho (wigner_moyal_cuda_1d.py:422-469):
//   S, fft0 | ifft1, shX, fft1 | ifft0, shY, fft0 | ifft1, shX, fft1, S
static AwFactor fshear_x(aw_state_s* h) {
  AwFactor f = fnone();
  f.sh_hi = h->shx_hi.p;
  f.sh_lo = h->shx_lo.p;
  f.sh_lo_n = h->shx_lo_n;
  f.sh_full = h->shx_full.p;
  f.active = 1;
  return f;
}
static AwFactor fshear_y(aw_state_s* h) {
  AwFactor f = fnone();
  f.sh_hi = h->shy_hi.p;
  f.sh_lo = h->shy_lo.p;
  f.sh_full = h->shy_full.p;
  f.sh_lo_n = h->shy_lo_n;
  f.active = 1;
  return f;
}

static int wm_wigner2rho(aw_state_s* h) {
  AwPassArgs a = pnone(h);
  a.in = h->W.p;
  a.out = h->rho.p;
  a.f0 = fsign();
  a.d1 = +1;
  TRY(col_pass(h, a, h->tw_c));
  a = pnone(h);
  a.in = a.out = h->rho.p;
  a.d1 = -1;
  a.f1 = fshear_x(h);
  a.d2 = +1;
  TRY(row_pass(h, a, h->tw_r));
  a = pnone(h);
  a.in = a.out = h->rho.p;
  a.d1 = -1;
  a.f1 = fshear_y(h);
  a.d2 = +1;
  TRY(col_pass(h, a, h->tw_c));
  a = pnone(h);
  a.in = a.out = h->rho.p;
  a.d1 = -1;
  a.f1 = fshear_x(h);
  a.d2 = +1;
  a.f3 = fsign();
  TRY(row_pass(h, a, h->tw_r));
  return AW_OK;
}

// Blackman windows (wigner_moyal_cuda_1d.py:678-698) as real column / row tables
static int ensure_blackman(aw_state_s* h, int nr, int nc) {
  if (h->blk_tabs.p) return AW_OK;
  std::vector<double> t(2 * (size_t)(nr + nc), 0.0);
  for (int j = 0; j < nc; ++j) {
    const double Cj = j * 2.0 * M_PI / (nc - 1.0);
    t[2 * j] = 0.42 - 0.5 * cos(Cj) + 0.08 * cos(2.0 * Cj);
  }
  for (int i = 0; i < nr; ++i) {
    const double Ci = i * 2.0 * M_PI / (nr - 1.0);
    t[2 * (nc + i)] = 0.42 - 0.5 * cos(Ci) + 0.08 * cos(2.0 * Ci);
  }
  TRY(upload_reals(h->blk_tabs, t, tab_fmt(h)));
  return AW_OK;
}

// rho -> W on a (rows x cols) grid held in `buf` (in place), the reference's
// rho2wigner_ minus the initial copy and sign flip:
//   [f0] fft1, shX, ifft1 | fft0, shY, ifft0 | fft1, shX, ifft1 | ifft0, S (+ reductions)
// `first_in` / `first_f0` let the first row pass read another buffer or apply
// the initial sign flip; `reduce` fills red_line / red_cross / red_sq.
struct WignerGrid {
  void* buf;
  int nr, nc;
  const DevBuf *twr, *twc;
};

static int wigner_passes(aw_state_s* h, const WignerGrid& g, const void* first_in, AwFactor first_f0, bool blackman,
                         bool reduce, bool store_last, bool row_first_done = false) {
  AwPassArgs a = pnone(h);
  a.nrows = g.nr;
  a.ncols = g.nc;
  a.batch_elems = (long long)g.nr * g.nc;
  a.batch_tab = 0;  // the Blackman tables are shared by all instances
  void* bcol = blackman ? h->blk_tabs.p : nullptr;
  void* brow = blackman ? (char*)h->blk_tabs.p + (size_t)g.nc * h->esz : nullptr;
  if (!row_first_done) {
    a.in = first_in;
    a.out = g.buf;
    a.f0 = first_f0;
    if (blackman) {
      a.f0.col_tab = bcol;
      a.f0.active = 1;
    }
    a.d1 = +1;
    a.f1 = fshear_x(h);
    a.d2 = -1;
    TRY(row_pass(h, a, *g.twr));
  }
  a = pnone(h);
  a.nrows = g.nr;
  a.ncols = g.nc;
  a.batch_elems = (long long)g.nr * g.nc;
  a.batch_tab = 0;  // the Blackman tables are shared by all instances
  a.in = a.out = g.buf;
  if (blackman) {
    a.f0.row_tab = brow;
    a.f0.active = 1;
  }
  a.d1 = +1;
  a.f1 = fshear_y(h);
  a.d2 = -1;
  TRY(col_pass(h, a, *g.twc));
  a = pnone(h);
  a.nrows = g.nr;
  a.ncols = g.nc;
  a.batch_elems = (long long)g.nr * g.nc;
  a.batch_tab = 0;  // the Blackman tables are shared by all instances
  a.in = a.out = g.buf;
  if (blackman) {
    a.f0.col_tab = bcol;
    a.f0.active = 1;
  }
  a.d1 = +1;
  a.f1 = fshear_x(h);
  a.d2 = -1;
  TRY(row_pass(h, a, *g.twr));
  a = pnone(h);
  a.nrows = g.nr;
  a.ncols = g.nc;
  a.batch_elems = (long long)g.nr * g.nc;
  a.batch_tab = 0;  // the Blackman tables are shared by all instances
  a.in = g.buf;
  a.out = store_last ? g.buf : nullptr;
  if (blackman) {
    a.f0.row_tab = brow;
    a.f0.active = 1;
  }
  a.d1 = -1;
  a.f3 = fsign();
  if (reduce) {
    a.red_line = (double*)h->red_line.p;
    a.red_cross = (double*)h->red_cross.p;
    a.red_sq = (double*)h->red_sq.p;
  }
  TRY(col_pass(h, a, *g.twc));
  return AW_OK;
}

struct FinalArgs {
  const double* colsum;
  int cstride;
  int ncol;
  const double* rowpart;
  int nparts;
  int nrow;
  int proll;
  const double* sqpart;
  double dXdP;
  double* inv;  // may be null
  int pnorm_own;
  int sqrt_norm;
};

// one instance (the first of the view): the argument pointers already point at its data
static int launch_finalize_args(aw_state_s* h, const FinalArgs& f, double t, double* hist_row, int stop_on_purity) {
  const double* colsum = f.colsum;
  const double* rowpart = f.rowpart;
  int nparts = f.nparts;
  const double* sqpart = f.sqpart;
  double* rowsum = (double*)h->rowsum.p;
  double* inv = f.inv;
  int* stop = dstop(h, h->v0);
  const double* prm = h->np ? (const double*)h->params.p + (size_t)h->v0 * h->np : nullptr;
  int ncol = f.ncol, nrow = f.nrow;
  double dX = h->cfg.dX, dP = h->cfg.dP, dXdP = f.dXdP;
  const int* ts = (const int*)h->terms.p;
  const int* tk = ts + 64;
  const int* ti = ts + 128;
  const double* tc = (const double*)((const char*)h->terms.p + 64 * 3 * sizeof(int));
  int nterms = (int)h->tslot.size(), nslots = h->cfg.n_slots;
  int cstride = f.cstride, proll = f.proll, pown = f.pnorm_own, sq = f.sqrt_norm;
  double* tv = dtv(h, h->v0);
  unsigned int* counter = dcounter(h, h->v0);
  // chunks per term: at least 16 columns or rows each, as the rotated frame's reduction
  int nchunk = std::max(1, std::min(64, std::max(ncol, nrow) / 16));
  while (nchunk > 1 && (nterms + 3) * nchunk > 1024) nchunk >>= 1;
  void* args[] = {&colsum, &rowpart, &nparts, &sqpart, &rowsum, &hist_row, &inv, &stop, &stop_on_purity, &t,
                  &ncol, &nrow, &dX, &dP, &dXdP, &ts, &tk, &ti, &tc, &nterms, &nslots, &cstride, &proll, &pown, &sq,
                  &prm, &tv, &counter, &nchunk};
  return hjit(h, h->k_final, dim3((nterms + 3) * nchunk), dim3(128), args);
}

// rotated frame: marginals of W from the reducing column pass
static int launch_finalize(aw_state_s* h, double t, double* hist_row, int stop_on_purity) {
  const int i = h->v0;
  FinalArgs f{(const double*)h->red_line.p + (size_t)i * h->nc, 1, h->nc,
              (const double*)h->red_cross.p + (size_t)i * h->red_blocks * h->nr, h->red_blocks, h->nr, 0,
              (const double*)h->red_sq.p + (size_t)i * h->red_blocks, h->cfg.dXdP, dinv(h, i), 0, 0};
  return launch_finalize_args(h, f, t, hist_row, stop_on_purity);
}

// marginal buffers of parity par (zbuf, altbuf, abs2 hold two sets, each for every instance)
static double2* zbuf_of(aw_state_s* h, int par) { return (double2*)h->zbuf.p + (size_t)par * h->ni * (h->nc + h->nr); }
static double2* altbuf_of(aw_state_s* h, int par) {
  return (double2*)h->altbuf.p + (size_t)par * h->ni * h->z_blocks * h->nr;
}
static double* abs2_of(aw_state_s* h, int par) { return (double*)h->abs2.p + (size_t)par * h->ni * std::max(h->nr, 1); }
// observable rows of instance i
static double* hist_of(aw_state_s* h, int i) { return (double*)h->hist.p + (size_t)i * h->hist_cap * h->hist_cols; }

static int launch_finalize_rot(aw_state_s* h, double t, double* hist_row, int stop_on_purity, int par = 0,
                               cudaStream_t st = nullptr, const double* tptr = nullptr) {
  // every instance of the view: blockIdx.y = instance - v0
  const int i0 = h->v0;
  int nparts = h->z_blocks;
  int nb2 = row_blocks(h, h->nr, h->nc);
  const double2* z = zbuf_of(h, par) + (size_t)i0 * h->nc;
  const double2* wpart = altbuf_of(h, par) + (size_t)i0 * nparts * h->nr;
  const double* abs2 = abs2_of(h, par) + (size_t)i0 * nb2;
  double* tv = dtv(h, i0);
  unsigned int* counter = dcounter(h, i0);
  double* inv = dinv(h, i0);
  int* stop = dstop(h, i0);
  const double* prm = h->np ? (const double*)h->params.p + (size_t)i0 * h->np : nullptr;
  int np = h->np;
  long long hstride = h->hist_cap * h->hist_cols;
  int ncol = h->nc, nrow = h->nr;
  double dX = h->cfg.dX, dP = h->cfg.dP, dXdP = h->cfg.dXdP;
  const int* ts = (const int*)h->terms.p;
  const int* tk = ts + 64;
  const int* ti = ts + 128;
  const double* tc = (const double*)((const char*)h->terms.p + 64 * 3 * sizeof(int));
  int nterms = (int)h->tslot.size(), nslots = h->cfg.n_slots;
  // chunks per term: enough blocks to spread the FP64 expression work and the loads of the row
  // partials over the SMs, at least 16 columns or rows each (smaller chunks slow small grids, whose
  // steps wait for this reduction)
  int nchunk = std::max(1, std::min(64, std::min(ncol, nrow) / 16));
  while (nchunk > 1 && ((std::min(ncol, nrow) % nchunk) || (nterms + 2) * nchunk > 1024)) nchunk >>= 1;
  void* args[] = {&z, &wpart, &nparts, &abs2, &nb2, &tv, &counter, &hist_row, &inv, &stop, &stop_on_purity, &t,
                  &ncol, &nrow, &dX, &dP, &dXdP, &ts, &tk, &ti, &tc, &nterms, &nslots, &nchunk, &prm, &np, &hstride,
                  &tptr};
  return hjit_on(h, h->k_final_rot, dim3((nterms + 2) * nchunk, h->vc), dim3(128), args, st ? st : h->st);
}

// room for `rows` observable rows of `cols` values per instance (cols 0: n_slots + 2)
static int ensure_hist(aw_state_s* h, long long rows, int cols = 0) {
  h->hist_cols = cols ? cols : h->cfg.n_slots + 2;
  h->hist_cap = std::max(rows, 1LL);
  const size_t need = (size_t)h->ni * h->hist_cap * h->hist_cols * 8;
  if (h->hist.bytes < need) TRY(dalloc(h->hist, need));
  h->hist_rows = 0;
  return AW_OK;
}

// stop flags of the view at the start of a run: inactive instances stay stopped
static int reset_stops(aw_state_s* h) {
  std::vector<int> f(h->vc);
  for (int k = 0; k < h->vc; ++k) f[k] = h->active.empty() || h->active[h->v0 + k] ? 0 : 1;
  CK(cudaMemcpyAsync(dstop(h, h->v0), f.data(), f.size() * sizeof(int), cudaMemcpyHostToDevice, h->st));
  return AW_OK;
}

// normalize_rho_wigner (wigner_moyal_cuda_1d.py:608-622): W = rho2wigner(rho); norm; W, rho /= norm
// (one instance at a time: the reducing Wigner transform feeds the single-instance finalize)
static int wm_normalize(aw_state_s* h, long long hist_row) {
  const int v0 = h->v0, vc = h->vc;
  for (int i = v0; i < v0 + vc; ++i) {
    h->v0 = i;
    h->vc = 1;
    WignerGrid g{h->W.p, h->nr, h->nc, &h->tw_r, &h->tw_c};
    int r = wigner_passes(h, g, h->rho.p, fsign(), false, true, true);
    if (!r) r = launch_finalize(h, 0.0, hist_of(h, i) + (size_t)hist_row * h->hist_cols, 0);
    if (!r) r = settle(h);
    if (!r) r = vscale(h, h->W.p, gsz(h));
    if (!r) r = vscale(h, h->rho.p, gsz(h));
    h->v0 = v0;
    h->vc = vc;
    TRY(r);
  }
  return AW_OK;
}

extern "C" int aw_wigner2rho(aw_handle h) {
  if (!h) return fail(AW_E_ARG, "null handle");
  Settled guard{h};
  TRY(clear_stops(h));
  if (!h->kn.rotated) return fail(AW_E_STATE, "wigner2rho exists for the Wigner-Moyal / Wigner-Bloch propagators");
  return wm_wigner2rho(h);
}

extern "C" int aw_normalize_rho_wigner(aw_handle h) {
  if (!h) return fail(AW_E_ARG, "null handle");
  Settled guard{h};
  TRY(clear_stops(h));
  if (!h->kn.rotated) return fail(AW_E_STATE, "normalize_rho_wigner exists for the Wigner-Moyal propagators");
  TRY(ensure_hist(h, 1));
  return wm_normalize(h, 0);
}

static int vn_get_wigner(aw_state_s* h, int blackman);
static int sw_get_wigner(aw_state_s* h, int blackman);

extern "C" int aw_rho2wigner(aw_handle h, int32_t blackman) {
  if (!h) return fail(AW_E_ARG, "null handle");
  Settled guard{h};
  TRY(clear_stops(h));
  if (h->kn.rotated) {
    if (blackman) TRY(ensure_blackman(h, h->nr, h->nc));
    WignerGrid g{h->W.p, h->nr, h->nc, &h->tw_r, &h->tw_c};
    return wigner_passes(h, g, h->rho.p, fsign(), blackman != 0, false, true);
  }
  if (h->kn.vn) return vn_get_wigner(h, blackman);
  return sw_get_wigner(h, blackman);
}

// ============================================================================ rotated-frame stepping
// Phase factors of one step of the reference's single_step_propagation
// (wigner_moyal_cuda_1d.py:543-561) for the rotated frame:
//   expV(t) = S * exp(-i dt/2 [V(XX,t+dt/2) - V(XX',t+dt/2)]) * absx
//   expK(t) = exp(-i dt [K(PP,t+dt/2) - K(PP',t+dt/2)]) * absp
// The step is executed as three passes
//   row:    [previous ifft1, V-kick]  S V(t_n) ... fft1
//   column: ifft0, K-kick, fft0
//   row:    ifft1, /N^2, V-kick(t_n)  [fused with the next step's first kick]
// and the sign flips of consecutive kicks cancel.
struct StepPlan {
  bool bloch;         // Bloch (imaginary-time) factors instead of unitary ones
  double dbeta;
  bool ehrenfest;     // per-step Wigner transform, normalisation and observables
  bool keep_rho;      // write rho_n (position representation) every step
  int stop_on_purity; // Gibbs loop: stop after the first step with purity >= 1
  bool per_inst = false;  // Bloch coefficients per instance (h->bvec) instead of dbeta, V_min, K_min
};

// Bloch coefficient vectors of a batch (ca = -dbeta/4 for V, -dbeta/2 for K; shift = minimum / 2)
static double* bvec_of(aw_state_s* h, int which) { return (double*)h->bvec.p + (size_t)which * h->ni; }

static AwFactor ftab(aw_state_s* h, int slot) {
  AwFactor f = fnone();
  f.col_tab = tab_col(h, slot);
  f.row_tab = tab_row(h, slot);
  f.active = 1;
  return f;
}

static int prepare_maskx(aw_state_s* h);
static int fold_maskx(aw_state_s* h, void* col, int count);

static int rot_tables_V(aw_state_s* h, const StepPlan& p, double tn, double tn1, bool pair) {
  const aw_config& c = h->cfg;
  if (p.bloch) {
    // bloch_expV: exp(-dbeta/4 (V(XX) + V(XX') - V_min)), split evenly over the two factors
    if (p.per_inst)
      return build_tab(h, TAB_BV, 0, 1, c.t_initial, 0.0, 0.0, 0.0, 0.0, 0, 0.0, nullptr, nullptr, 1, bvec_of(h, 0),
                       bvec_of(h, 1));
    return build_tab(h, TAB_BV, 0, 1, c.t_initial, 0.0, -0.25 * p.dbeta, 0.0, 0.5 * h->V_min, 0, 0.0);
  }
  const double half = 0.5 * c.dt;
  if (c.absx_mode == 1) TRY(prepare_maskx(h));
  TRY(build_tab(h, TAB_V1, 0, 0, tn + half, 0.0, -half, 0.0, 0.0, 0, 0.0));
  TRY(fold_maskx(h, tab_col(h, TAB_V1), 1));
  if (pair) {
    TRY(build_tab(h, TAB_V1B, 0, 0, tn1 + half, 0.0, -half, 0.0, 0.0, 0, 0.0));
    TRY(fold_maskx(h, tab_col(h, TAB_V1B), 1));
  }
  return AW_OK;
}

static int rot_tables_K(aw_state_s* h, const StepPlan& p, double tn) {
  const aw_config& c = h->cfg;
  if (p.bloch && p.per_inst)
    return build_tab(h, TAB_BK, 1, 1, c.t_initial, 0.0, 0.0, 0.0, 0.0, 0, 0.0, nullptr, nullptr, 1, bvec_of(h, 2),
                     bvec_of(h, 3));
  if (p.bloch)
    return build_tab(h, TAB_BK, 1, 1, c.t_initial, 0.0, -0.5 * p.dbeta, 0.0, 0.5 * h->K_min, 0, 0.0);
  return build_tab(h, TAB_K, 1, 0, tn + 0.5 * c.dt, 0.0, -c.dt, 0.0, 0.0, 0, 0.0);
}

// The time-independent x mask of a single propagator, built once.  The reference evaluates
// abs_boundary_x(XX, XX') per point inside every kick; when the mask is a product f(XX) g(XX') (the
// usual absorber, e.g. cos(...XX...) * cos(...XX_prime...)) its factors are folded into the column
// and row tables of the V kick instead, so that the passes read no mask.  The test is numerical:
// every point within a few rounding errors of m[i, j0] m[i0, j] / m[i0, j0].
static int prepare_maskx(aw_state_s* h) {
  if (h->maskx_ready) return AW_OK;
  TRY(build_mask2d(h, 0, 0.0));
  h->maskx_ready = true;
  h->maskx_sep = false;
  if (h->ni != 1) return AW_OK;
  const int nr = h->nr, nc = h->nc;
  const size_t n = (size_t)nr * nc;
  // read back on the handle's stream (non-blocking: a plain cudaMemcpy would not wait for the build)
  std::vector<double> m(n);
  if (h->f32) {
    std::vector<float> f(n);
    CK(cudaMemcpyAsync(f.data(), h->maskx.p, n * 4, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    for (size_t k = 0; k < n; ++k) m[k] = f[k];
  } else if (h->df) {
    std::vector<float> f(2 * n);
    CK(cudaMemcpyAsync(f.data(), h->maskx.p, n * 8, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    for (size_t k = 0; k < n; ++k) m[k] = (double)f[2 * k] + (double)f[2 * k + 1];
  } else {
    CK(cudaMemcpyAsync(m.data(), h->maskx.p, n * 8, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
  }
  size_t piv = 0;
  for (size_t k = 1; k < n; ++k)
    if (std::fabs(m[k]) > std::fabs(m[piv])) piv = k;
  const double mx = std::fabs(m[piv]);
  if (!(mx > 0.0) || !std::isfinite(mx)) return AW_OK;
  const int i0 = (int)(piv / nc), j0 = (int)(piv % nc);
  const double tol = (h->f32 ? 1e-6 : 3e-14) * mx;
  for (int i = 0; i < nr; ++i) {
    const double u = m[(size_t)i * nc + j0] / m[piv];
    for (int j = 0; j < nc; ++j)
      if (!(std::fabs(u * m[(size_t)i0 * nc + j] - m[(size_t)i * nc + j]) <= tol)) return AW_OK;
  }
  std::vector<double> sv(nc + nr);
  for (int j = 0; j < nc; ++j) sv[j] = m[(size_t)i0 * nc + j];
  for (int i = 0; i < nr; ++i) sv[nc + i] = m[(size_t)i * nc + j0] / m[piv];
  TRY(dalloc(h->masksep, sv.size() * sizeof(double)));
  CK(cudaMemcpyAsync(h->masksep.p, sv.data(), sv.size() * sizeof(double), cudaMemcpyHostToDevice, h->st));
  CK(cudaStreamSynchronize(h->st));
  h->maskx_sep = true;
  return AW_OK;
}

// folds a separable x mask into `count` V-kick tables at `col` (nc + nr entries each, consecutive)
static int fold_maskx(aw_state_s* h, void* col, int count) {
  if (!h->maskx_sep) return AW_OK;
  KL(aw_k_scale_lines(col, tab_fmt(h), (const double*)h->masksep.p, h->nc + h->nr, count,
                      (long long)h->nc + h->nr, h->st));
  return AW_OK;
}

// V-kick factor of time point n (time t_mask = t_n for the absorber, as expV of
// wigner_moyal_cuda_1d.py:742-760 evaluates abs_boundary_x at the kernel's t).  A time-dependent
// absorber alternates between two mask buffers by the parity of n, since the row pass applies the
// kicks of t_n and t_n+1 together; a buffer is rebuilt only when it holds another time.
static int vkick(aw_state_s* h, const StepPlan& p, int slot, bool sign, double t_mask, AwFactor* f, long long n) {
  *f = ftab(h, p.bloch ? TAB_BV : slot);
  f->sign = sign;
  if (!p.bloch && h->cfg.absx_mode == 2) {
    const int b = (int)(n & 1);
    DevBuf& m = b ? h->maskx2 : h->maskx;
    if (!(h->maskx_t[b] == t_mask)) {
      TRY(build_mask2d(h, 0, t_mask, &m));
      h->maskx_t[b] = t_mask;
    }
    f->mask = m.p;
    f->mask_pow = 1;
  } else if (!p.bloch && h->cfg.absx_mode) {
    TRY(prepare_maskx(h));
    if (!h->maskx_sep) {
      f->mask = h->maskx.p;
      f->mask_pow = 1;
    }
  }
  return AW_OK;
}

// Run `steps` steps of the rotated-frame propagator on rho.
//   times[n] (n = 1..steps) are the reference's self.t values after the increment.
//   rows of observables go to hist (one per step) when p.ehrenfest.
static int rot_run(aw_state_s* h, const StepPlan& p, long long steps, const std::vector<double>& times, double* hist) {
  const aw_config& c = h->cfg;
  const bool vdep = !p.bloch && (c.v_time_dependent || c.absx_mode == 2);
  const bool kdep = !p.bloch && (c.k_time_dependent || c.absp_mode == 2);
  const long long grid = (long long)h->nr * h->nc;
  const double inv_n2 = p.bloch ? 1.0 : 1.0 / (double)grid;  // WM divides by N^2 (wm:557); Bloch does not
  // Real-time propagation is linear and every recorded observable is a ratio to the norm of the
  // same step (sum f W / sum W, purity sum W^2 / (sum W)^2), so the per-step normalisation of
  // normalize_rho_wigner (wm:608-622) is deferred to the end of the call: the step loop does not
  // wait for the reduction, which runs on a side stream.  Bloch steps normalise every step.
  const bool defer = !p.bloch && p.ehrenfest && h->st2;
  cudaStream_t side = h->side();
  // With the deferred reduction the marginal pass of step n runs on the side stream as well, where
  // it overlaps the column and row passes of step n + 1 (and fills their last partial waves of
  // blocks).  The branch outputs then alternate between W and tmp, the last step's in W, so that a
  // row pass never overwrites a branch output that a marginal pass may still read.
  auto wbuf = [&](long long n) -> void* { return (!defer || ((steps - n) & 1) == 0) ? h->W.p : h->tmp.p; };
  // scale applied in the column pass: 1/N^2 and, for Bloch steps, 1/norm of the previous step
  TRY(vinv_reset(h));
  TRY(reset_stops(h));  // a stop raised by an earlier call must not persist
  const int* stop = p.stop_on_purity || h->ni > 1 ? (const int*)dstop(h) : nullptr;

  if (!vdep) TRY(rot_tables_V(h, p, times[1], times[1], false));
  if (!kdep) TRY(rot_tables_K(h, p, times[1]));
  // Native FP64 real time with a K kick that does not change during the call: the kick and the 1/N^2 the
  // column pass folds into it (when no per-call scale is read) as one full table where the full shear
  // tables exist, so that the FP64-bound column pass makes one complex product a point instead of two
  // (the line constant and the table along the line)
  const bool kfull = h->shy_full.p && !p.bloch && !kdep && h->ni == 1 && !c.absp_mode && !(p.ehrenfest && !defer);
  if (kfull) {
    if (!h->kfull.p) TRY(dalloc(h->kfull, (size_t)grid * 16));
    KL(aw_k_sep_full(tab_col(h, TAB_K), tab_row(h, TAB_K), inv_n2, h->nr, h->nc, 0, h->kfull.p, h->st));
  }
  // the same for a V kick that does not change during the call (no 2-D x mask left after folding):
  // the row pass applies it twice a step, each one complex product a point instead of two
  const bool vfull = h->shx_full.p && !p.bloch && !vdep && h->ni == 1 && !(c.absx_mode && !h->maskx_sep);
  if (vfull) {
    if (!h->vfull.p) TRY(dalloc(h->vfull, (size_t)grid * 16));
    KL(aw_k_sep_full(tab_col(h, TAB_V1), tab_row(h, TAB_V1), 1.0, h->nr, h->nc, 1, h->vfull.p, h->st));
  }
  // With a time-dependent V the kick tables of up to VSEQ consecutive time points are built by one
  // launch: table s of the run holds exp(-i dt/2 V(., t_{n0+s} + dt/2)).
  const long long VSEQ = 256;
  long long vs_n0 = 0, vs_cnt = 0;
  if (vdep) {
    TRY(dalloc(h->vseq, (size_t)VSEQ * (h->nc + h->nr) * h->esz));
    TRY(dalloc(h->vtimes, (size_t)VSEQ * sizeof(double)));
  }
  // kick factor of time point n (table slot TAB_V1 when V does not depend on time)
  auto vfactor = [&](long long n, bool sign, AwFactor* f) -> int {
    TRY(vkick(h, p, TAB_V1, sign, times[n], f, n));
    if (vfull) {
      *f = fnone();
      f->sign = sign;
      f->sh_full = h->vfull.p;
      f->active = 1;
      return AW_OK;
    }
    if (!vdep) return AW_OK;
    const long long need_hi = std::min(n + 1, steps + 1);
    if (n < vs_n0 || need_hi >= vs_n0 + vs_cnt) {
      vs_n0 = n;
      vs_cnt = std::min(VSEQ, steps + 2 - n);
      std::vector<double> tl(times.begin() + n, times.begin() + n + vs_cnt);
      // from pageable memory: staged before the call returns, ordered on the stream
      CK(cudaMemcpyAsync(h->vtimes.p, tl.data(), tl.size() * sizeof(double), cudaMemcpyHostToDevice, h->st));
      const double half = 0.5 * c.dt;
      TRY(build_tab(h, 0, 0, 0, half, 0.0, -half, 0.0, 0.0, 0, 0.0, h->vseq.p, (const double*)h->vtimes.p,
                    (int)vs_cnt));
      TRY(fold_maskx(h, h->vseq.p, (int)vs_cnt));
    }
    f->col_tab = (char*)h->vseq.p + (size_t)(n - vs_n0) * (h->nc + h->nr) * h->esz;
    f->row_tab = (char*)f->col_tab + (size_t)h->nc * h->esz;
    return AW_OK;
  };

  // first kick: rho (position) -> S V(t_1) -> fft1
  {
    AwPassArgs a = pnone(h);
    a.in = a.out = h->rho.p;
    TRY(vfactor(1, true, &a.f2));
    a.d2 = +1;
    a.stop = stop;
    TRY(row_pass(h, a, h->tw_r));
  }
  // Graph windows (see aw_graph): GW consecutive steps captured once and replayed.  A window holds no
  // per-step argument: its kick tables are rebuilt into slots 0..GW before every replay, its step
  // times read from h->vtimes by the observable reduction, its history rows written to h->hwin and
  // copied into place after the replay.
  const long long GW = std::min<long long>(AW_GRAPH_MAX, (steps - 2) & ~1LL);
  const bool graphable = defer && h->graph_on && !kdep && c.absx_mode != 2 && !p.keep_rho && !p.stop_on_purity &&
                         h->ni == 1 && !h->prof_on && GW >= AW_GRAPH_MIN;
  long long win_n0 = 0;        // first step of the window being captured (0: none)
  if (graphable) {
    TRY(dalloc(h->vtimes, (size_t)VSEQ * sizeof(double)));
    TRY(dalloc(h->hwin, (size_t)AW_GRAPH_MAX * h->hist_cols * sizeof(double)));
    // the call's step times, uploaded once (a copy from pageable memory waits for the stream); each
    // window copies its own on the device
    TRY(dalloc(h->ctimes, (size_t)(steps + 2) * sizeof(double)));
    CK(cudaMemcpyAsync(h->ctimes.p, times.data(), (size_t)(steps + 2) * sizeof(double), cudaMemcpyHostToDevice,
                       h->st));
  }

  auto one_step = [&](long long n) -> int {
    const bool last = n == steps;
    const int par = defer ? (int)(n & 1) : 0;
    // column pass: scale, ifft0, K-kick, fft0
    {
      if (kdep) TRY(rot_tables_K(h, p, times[n]));
      AwPassArgs a = pnone(h);
      a.in = a.out = h->rho.p;
      a.d1 = -1;
      a.f1 = ftab(h, p.bloch ? TAB_BK : TAB_K);
      // the scale (1/N^2, and with per-step observables and no side stream the previous step's 1/norm)
      // applied after ifft0 (linear), folded into the K kick's per-column constant: a complex product a
      // point fewer than scaling before the transform (1/N^2 alone, a power of two, gives the same bits)
      a.f1.scale = inv_n2;
      a.f1.scale_ptr = p.ehrenfest && !defer ? dinv(h) : nullptr;
      if (!p.bloch && c.absp_mode) {
        if (c.absp_mode == 2 || !h->maskp_ready) {
          TRY(build_mask2d(h, 1, times[n]));
          h->maskp_ready = true;
        }
        a.f1.mask = h->maskp.p;
        a.f1.mask_pow = 1;
      }
      if (kfull) {
        a.f1 = fnone();
        a.f1.sh_full = h->kfull.p;
        a.f1.active = 1;
      }
      a.d2 = +1;
      a.stop = stop;
      a.lines_hint = h->tuned_col_lines;
      a.tma = h->tuned_col_tma;
      a.shape = h->tuned_col_shape;
      TRY(col_pass(h, a, h->tw_c));
    }
    // the marginal pass and reduction of step n - 2 read this parity's branch output and sums (in a
    // window being captured, the first two steps' predecessors finished before the window started)
    if (defer && n >= 3 && (!win_n0 || n >= win_n0 + 2)) CK(cudaStreamWaitEvent(h->st, h->ev_f[par], 0));
    // row pass: ifft1, V-kick(t_n) [branch: Wigner transform] [next kick(t_{n+1}), fft1 | S]
    {
      AwPassArgs a = pnone(h);
      a.in = a.out = h->rho.p;
      a.d1 = -1;
      a.shape = h->tuned_row_shape;
      TRY(vfactor(n, false, &a.f1));
      if (p.ehrenfest) {
        a.br_out = wbuf(n);
        a.br_d1 = +1;
        a.fbr = fshear_x(h);
        a.br_d2 = -1;
        a.red_abs2 = abs2_of(h, par);  // Sum |rho_n|^2 for the purity
      }
      if (p.keep_rho) {
        a.mid_out = h->snap.p;
        a.mid_sign = 1;
      }
      if (!last) {
        TRY(vfactor(n + 1, false, &a.f2));
        a.d2 = +1;
      } else {
        a.f2 = fsign();
      }
      a.stop = stop;
      TRY(row_pass(h, a, h->tw_r));
    }
    if (p.ehrenfest) {
      // The per-step observables need only the marginals of W = S ifft0 C ifft0 (shY . fft0 A), where
      // A is the branch output and C the second X shear; both marginals follow from Q_j = shY . fft0 A_j
      // by alternating sums (aw_finalize_rot), so this column pass runs one FFT per column and writes
      // nothing back.  The last step completes W.
      AwPassArgs a = pnone(h);
      a.in = wbuf(n);
      a.d1 = +1;
      a.f1 = fshear_y(h);
      a.col_alt = zbuf_of(h, par);
      a.alt_cross = altbuf_of(h, par);
      a.lines_hint = h->z_lines;
      a.cluster = h->z_cluster;
      a.stop = stop;
      double* hrow = win_n0 ? (double*)h->hwin.p + (size_t)(n - win_n0) * h->hist_cols
                            : hist + (size_t)(n - 1) * h->hist_cols;
      const double* tptr = win_n0 ? (const double*)h->vtimes.p + (n - win_n0) : nullptr;
      if (defer) {
        // after the row pass of step n, on the side stream: marginal pass, then the reduction
        CK(cudaEventRecord(h->ev_z[par], h->st));
        CK(cudaStreamWaitEvent(side, h->ev_z[par], 0));
        TRY(col_pass(h, a, h->tw_c, side));
        TRY(launch_finalize_rot(h, times[n], hrow, 0, par, side, tptr));
        CK(cudaEventRecord(h->ev_f[par], side));
      } else {
        TRY(col_pass(h, a, h->tw_c));
        TRY(launch_finalize_rot(h, times[n], hrow, p.stop_on_purity));
      }
      if (last) {
        // completes W in place: after the marginal pass has read it
        if (defer) CK(cudaStreamWaitEvent(h->st, h->ev_f[par], 0));
        WignerGrid g{h->W.p, h->nr, h->nc, &h->tw_r, &h->tw_c};
        TRY(wigner_passes(h, g, h->W.p, fnone(), false, false, true, true));
      }
    }
    return AW_OK;
  };

  // one window of GW steps from n0 (even, and the window ends before the last step): inputs
  // refreshed on the stream, the graph of the window's branch-output parity captured on first use,
  // then replayed
  auto window = [&](long long n0) -> int {
    // the side stream's reductions of the steps before the window are done before it starts
    for (int k = 0; k < 2; ++k) CK(cudaStreamWaitEvent(h->st, h->ev_f[k], 0));
    // times t_{n0} .. t_{n0 + GW + 1}: the window's steps and the kicks of their successors (so that no
    // table is rebuilt inside the window)
    CK(cudaMemcpyAsync(h->vtimes.p, (const double*)h->ctimes.p + n0, (size_t)(GW + 2) * sizeof(double),
                       cudaMemcpyDeviceToDevice, h->st));
    if (vdep) {
      vs_n0 = n0;
      vs_cnt = GW + 2;
      const double half = 0.5 * c.dt;
      TRY(build_tab(h, 0, 0, 0, half, 0.0, -half, 0.0, 0.0, 0, 0.0, h->vseq.p, (const double*)h->vtimes.p,
                    (int)vs_cnt));
      TRY(fold_maskx(h, h->vseq.p, (int)vs_cnt));
    }
    // the graph of this window length and of this parity of the call's step count (which of W / tmp
    // each step branches into)
    const long long gkey = 2 * GW + (steps & 1);
    int key = -1;
    for (int k = 0; k < AW_GRAPH_CACHE; ++k)
      if (h->graph_exec[k] && h->graph_key[k] == gkey) key = k;
    if (key < 0) {
      key = 0;  // a free slot, else the least recently used
      for (int k = 0; k < AW_GRAPH_CACHE; ++k) {
        if (!h->graph_exec[k]) {
          key = k;
          break;
        }
        if (h->graph_used[k] < h->graph_used[key]) key = k;
      }
      if (h->graph_exec[key]) {
        cudaGraphExecDestroy(h->graph_exec[key]);
        h->graph_exec[key] = nullptr;
      }
      h->graph_key[key] = gkey;
      win_n0 = n0;
      const long long launches0 = g_launches.load();
      CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
      int r = AW_OK;
      for (long long n = n0; n < n0 + GW && r == AW_OK; ++n) r = one_step(n);
      // the side stream's last two reductions join the window
      for (int k = 0; k < 2 && r == AW_OK; ++k)
        if (cudaStreamWaitEvent(h->st, h->ev_f[k], 0) != cudaSuccess) r = fail(AW_E_CUDA, "graph join failed");
      cudaGraph_t g = nullptr;
      const cudaError_t e = cudaStreamEndCapture(h->st, &g);
      win_n0 = 0;
      const long long captured = g_launches.load() - launches0;
      g_launches = launches0;  // nothing ran during the capture: the launches count when the graph runs
      cudaError_t ie = cudaErrorUnknown;
      if (r == AW_OK && e == cudaSuccess) ie = cudaGraphInstantiate(&h->graph_exec[key], g, 0);
      if (g) cudaGraphDestroy(g);
      if (ie != cudaSuccess) {
        // nothing of the window ran: this handle steps on the streams from now on, starting here
        h->graph_exec[key] = nullptr;
        h->graph_on = false;
        cudaGetLastError();
        for (long long n = n0; n < n0 + GW; ++n) TRY(one_step(n));
        return AW_OK;
      }
      h->graph_launches[key] = captured;
    }
    h->graph_used[key] = ++h->graph_clock;
    CK(cudaGraphLaunch(h->graph_exec[key], h->st));
    g_launches += h->graph_launches[key];
    // the window's history rows, and the side-stream events re-recorded on the stream (their records
    // inside the capture belong to the graph)
    CK(cudaMemcpyAsync(hist + (size_t)(n0 - 1) * h->hist_cols, h->hwin.p, (size_t)GW * h->hist_cols * sizeof(double),
                       cudaMemcpyDeviceToDevice, h->st));
    for (int k = 0; k < 2; ++k) CK(cudaEventRecord(h->ev_f[k], h->st));
    return AW_OK;
  };

  for (long long n = 1; n <= steps;) {
    if (graphable && n >= 2 && !(n & 1) && n + GW <= steps) {
      TRY(window(n));
      n += GW;
    } else {
      TRY(one_step(n));
      ++n;
    }
  }
  // join: the last reduction wrote the history and 1/norm that the caller applies
  if (defer && steps > 0) CK(cudaStreamWaitEvent(h->st, h->ev_f[(int)(steps & 1)], 0));
  return AW_OK;
}

extern "C" int aw_propagate(aw_handle h, int64_t steps, double* t) {
  if (!h || !t) return fail(AW_E_ARG, "null argument");
  if (steps < 0) return fail(AW_E_ARG, "negative step count");
  Settled guard{h};
  int vn_propagate(aw_state_s*, long long, double*);
  int sw_propagate(aw_state_s*, long long, double*);
  if (h->kn.vn) return vn_propagate(h, steps, t);
  if (h->kn.sw) return sw_propagate(h, steps, t);
  const aw_config& c = h->cfg;
  std::vector<double> times(steps + 2);
  times[0] = *t;
  for (long long n = 1; n <= steps + 1; ++n) times[n] = times[n - 1] + c.dt;  // self.t += self.dt
  TRY(ensure_hist(h, steps + 1));
  if (steps == 0) {
    if (!c.ehrenfest) TRY(wm_normalize(h, 0));
    return AW_OK;
  }
  StepPlan p{false, 0.0, c.ehrenfest != 0, false, 0};
  TRY(rot_run(h, p, steps, times, hist_of(h, h->v0)));
  if (c.ehrenfest) {
    // the last step's normalisation, applied to both arrays
    TRY(settle(h));
    TRY(vscale(h, h->W.p, gsz(h)));
    TRY(vscale(h, h->rho.p, gsz(h)));
    h->hist_rows = steps;
  } else {
    TRY(wm_normalize(h, steps));
    h->hist_rows = 0;
  }
  *t = times[steps];
  return AW_OK;
}

// One split step at time t, as single_step_propagation does it (wigner_moyal_cuda_1d.py:543-561,
// rho_vneumann_cuda_1d.py:450-468, schrodinger_wigner_cuda_1d.py:356-369): V and K at the kernels'
// times for t, not normalised, no observables, t unchanged.
int vn_single_step(aw_state_s* h, double t);
int sw_single_step(aw_state_s* h, double t);
extern "C" int aw_single_step(aw_handle h, double t) {
  if (!h) return fail(AW_E_ARG, "null handle");
  Settled guard{h};
  TRY(clear_stops(h));
  if (h->kn.vn) return vn_single_step(h, t);
  if (h->kn.sw) return sw_single_step(h, t);
  const std::vector<double> times{t - h->cfg.dt, t, t + h->cfg.dt};
  StepPlan p{false, 0.0, false, false, 0};
  return rot_run(h, p, 1, times, nullptr);
}

extern "C" int aw_history_of(aw_handle h, int32_t inst, double* out, int64_t max_rows, int64_t* rows, int32_t* cols) {
  if (!h) return fail(AW_E_ARG, "null handle");
  if (inst < 0 || inst >= h->ni) return fail(AW_E_ARG, "no instance %d", inst);
  const long long n = std::min<long long>(h->hist_rows, max_rows);
  if (rows) *rows = h->hist_rows;
  if (cols) *cols = h->hist_cols;
  if (out && n > 0 && h->hist.p) {
    CK(cudaMemcpyAsync(out, hist_of(h, inst), (size_t)n * h->hist_cols * 8, cudaMemcpyDeviceToHost, h->st));
  }
  CK(cudaStreamSynchronize(h->st));
  return check_err(h);
}

extern "C" int aw_history(aw_handle h, double* out, int64_t max_rows, int64_t* rows, int32_t* cols) {
  if (!h) return fail(AW_E_ARG, "null handle");
  return aw_history_of(h, h->v0, out, max_rows, rows, cols);
}

// ============================================================================ observables
static int get_obs_kernel(aw_state_s* h, const char* expr, cudaKernel_t* k) {
  auto it = h->obs_kernels.find(expr);
  if (it != h->obs_kernels.end()) {
    *k = it->second;
    return AW_OK;
  }
  cudaLibrary_t lib;
  TRY(jit_compile(awjit::observable_source(h->kn, h->consts, expr), &lib));
  TRY(jit_kernel(lib, "aw_obs", k));
  h->obs_kernels[expr] = *k;
  return AW_OK;
}

extern "C" int aw_average(aw_handle h, const char* expr, double t, double* out) {
  if (!h || !expr || !out) return fail(AW_E_ARG, "null argument");
  if (h->kn.vn) return fail(AW_E_STATE, "use aw_average_ops for density-matrix propagators");
  cudaKernel_t k;
  TRY(get_obs_kernel(h, expr, &k));
  // the first instance of the view
  const void* src = at_inst(h->kn.rotated ? h->W.p : h->rho.p, gsz(h), h->esz, h->v0);
  int f32 = h->f32, nr = h->kn.rotated ? h->nr : 1, nc = h->nc;
  double* part = (double*)h->part.p;
  double dX = h->cfg.dX, dP = h->cfg.dP;
  void* args[] = {&src, &f32, &t, &part, &nr, &nc, &dX, &dP};
  const int nb = 256;
  TRY(hjit(h, k, dim3(nb), dim3(256), args));
  std::vector<double> hp(nb);
  CK(cudaMemcpyAsync(hp.data(), part, nb * 8, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  double s = 0.0;
  for (int b = 0; b < nb; ++b) s += hp[b];
  *out = h->kn.rotated ? s * h->cfg.dXdP : s;
  return AW_OK;
}

extern "C" int aw_purity(aw_handle h, double* out) {
  if (!h || !out) return fail(AW_E_ARG, "null argument");
  double s[2];
  if (h->kn.rotated) {
    TRY(dsum(h, at_inst(h->W.p, gsz(h), h->esz, h->v0), gsz(h), 1, 0, s));
    *out = 2.0 * M_PI * s[0] * h->cfg.dXdP;
  } else if (h->kn.vn) {
    TRY(dsum(h, at_inst(h->rho.p, gsz(h), h->esz, h->v0), gsz(h), 2, 0, s));
    *out = s[0] * h->cfg.dX * h->cfg.dX;
  } else {
    return fail(AW_E_STATE, "purity is defined for density-matrix and Wigner propagators");
  }
  return AW_OK;
}

// ============================================================================ Bloch
extern "C" int aw_bloch_step(aw_handle h, double dbeta, double* out) {
  if (!h) return fail(AW_E_ARG, "null handle");
  Settled guard{h};
  int vn_bloch_step(aw_state_s*, double, double*);
  if (h->kind == AW_RHO_BLOCH) return vn_bloch_step(h, dbeta, out);
  if (h->kind != AW_WIGNER_BLOCH) return fail(AW_E_STATE, "Bloch steps need a Bloch propagator");
  TRY(ensure_hist(h, 1));
  StepPlan p{true, dbeta, true, false, 0};
  if (h->ni > 1) {
    std::vector<double> db(h->vc, dbeta);
    TRY(upload_bloch(h, db.data()));
    p.per_inst = true;
  }
  std::vector<double> times(3, 0.0);
  TRY(rot_run(h, p, 1, times, hist_of(h, h->v0)));
  TRY(settle(h));
  TRY(vscale(h, h->W.p, gsz(h)));
  TRY(vscale(h, h->rho.p, gsz(h)));
  if (out) {
    CK(cudaMemcpyAsync(out, hist_of(h, h->v0), (size_t)h->hist_cols * 8, cudaMemcpyDeviceToHost, h->st));
  }
  CK(cudaStreamSynchronize(h->st));
  return AW_OK;
}

// get_gibbs_state's loop (wigner_bloch_cuda_1d.py:119-155) on every active instance of the view:
// `steps` Bloch steps of dbeta[k], each instance stopping after its first step with purity >= 1;
// done[k] / purity[k] report the steps that ran and the last purity.
static int rot_gibbs(aw_state_s* h, const double* dbeta, long long steps, long long* done, double* purity) {
  for (int k = 0; k < h->vc; ++k) {
    if (done) done[k] = 0;
  }
  if (steps <= 0) return AW_OK;
  TRY(ensure_hist(h, steps + 1));
  CK(cudaMemsetAsync(h->hist.p, 0, (size_t)h->ni * h->hist_cap * h->hist_cols * 8, h->st));
  TRY(dalloc(h->snap, (size_t)h->ni * gsz(h) * h->esz));
  StepPlan p{true, dbeta[0], true, true, 1};
  if (h->ni > 1) {
    TRY(upload_bloch(h, dbeta));
    p.per_inst = true;
  }
  std::vector<double> times(steps + 2, 0.0);
  TRY(rot_run(h, p, steps, times, hist_of(h, h->v0)));
  // how many steps ran: rows are written in order until the stop flag is raised; the finalize
  // of the stopping step still writes (the flag is checked at entry), so count rows whose norm
  // entry was written
  const int cols = h->hist_cols;
  std::vector<double> hh((size_t)h->vc * h->hist_cap * cols);
  CK(cudaMemcpyAsync(hh.data(), hist_of(h, h->v0), hh.size() * 8, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  std::vector<long long> ran(h->vc, 0);
  for (int k = 0; k < h->vc; ++k) {
    const double* hk = hh.data() + (size_t)k * h->hist_cap * cols;
    for (long long n = 0; n < steps; ++n) {
      if (hk[(size_t)n * cols + cols - 1] == 0.0) break;
      ran[k] = n + 1;
    }
    if (done) done[k] = ran[k];
    if (purity && ran[k] > 0) purity[k] = hk[(size_t)(ran[k] - 1) * cols + cols - 2];
  }
  h->hist_rows = steps;  // rows 0 .. done - 1 of each instance hold its per-step observables
  // rho_n of the last executed step (position representation, unnormalised) and its W, for the
  // instances that ran
  TRY(settle(h));
  TRY(reset_stops(h));
  for (int k = 0; k < h->vc; ++k) {
    const int i = h->v0 + k;
    if (ran[k] == 0) continue;
    CK(cudaMemcpyAsync(at_inst(h->rho.p, gsz(h), h->esz, i), at_inst(h->snap.p, gsz(h), h->esz, i),
                       (size_t)gsz(h) * h->esz, cudaMemcpyDeviceToDevice, h->st));
  }
  {
    WignerGrid g{h->W.p, h->nr, h->nc, &h->tw_r, &h->tw_c};
    TRY(wigner_passes(h, g, h->rho.p, fsign(), false, false, true));
  }
  TRY(settle(h));
  TRY(vscale(h, h->W.p, gsz(h)));
  TRY(vscale(h, h->rho.p, gsz(h)));
  CK(cudaStreamSynchronize(h->st));
  return AW_OK;
}

extern "C" int aw_gibbs(aw_handle h, double dbeta, int64_t steps, int64_t* done, double* purity) {
  if (!h) return fail(AW_E_ARG, "null handle");
  std::vector<double> db(h->vc, dbeta);
  std::vector<int64_t> d(h->vc, 0);
  std::vector<double> pu(h->vc, 0.0);
  TRY(aw_gibbs_batch(h, db.data(), steps, d.data(), pu.data()));
  if (done) *done = d[0];
  if (purity && d[0] > 0) *purity = pu[0];
  return AW_OK;
}

extern "C" int aw_gibbs_batch(aw_handle h, const double* dbeta, int64_t steps, int64_t* done, double* purity) {
  if (!h || !dbeta) return fail(AW_E_ARG, "null argument");
  Settled guard{h};
  int vn_gibbs(aw_state_s*, const double*, long long, long long*, double*);
  std::vector<long long> d(h->vc, 0);
  if (h->kind == AW_RHO_BLOCH) {
    TRY(vn_gibbs(h, dbeta, steps, d.data(), purity));
  } else if (h->kind == AW_WIGNER_BLOCH) {
    TRY(rot_gibbs(h, dbeta, steps, d.data(), purity));
  } else {
    return fail(AW_E_STATE, "get_gibbs_state needs a Bloch propagator");
  }
  if (done)
    for (int k = 0; k < h->vc; ++k) done[k] = d[k];
  return AW_OK;
}

// ============================================================================ von Neumann / rho-Bloch
// rho(x, x') on an N x N grid, the reference's RhoVNeumannCUDA1D / RhoBlochCUDA1D.
// One step is the rotated-frame sequence with X / P tables (rho_vneumann_cuda_1d.py:450-468,
// rho_bloch_cuda_1d.py:225-246) and the per-step trace normalisation folded into the next pass.
struct VnPlan {
  bool bloch;
  double dbeta;
  bool observables;    // per-step X / P diagonals and the user's averages
  bool keep_rho;       // store rho_n (position representation) every step
  int stop_on_purity;
  int complex_trace;   // rho-Bloch divides by the complex trace (rho_bloch_cuda_1d.py:244)
  bool per_inst = false;  // Bloch coefficients per instance (h->bvec)
};

static int vn_tables(aw_state_s* h, const VnPlan& p, double tn, bool kfirst) {
  const aw_config& c = h->cfg;
  if (p.bloch && p.per_inst) {
    TRY(build_tab(h, TAB_BV, 0, 1, c.t_initial, 0.0, 0.0, 0.0, 0.0, 0, 0.0, nullptr, nullptr, 1, bvec_of(h, 0),
                  bvec_of(h, 1)));
    return build_tab(h, TAB_BK, 1, 1, c.t_initial, 0.0, 0.0, 0.0, 0.0, 0, 0.0, nullptr, nullptr, 1, bvec_of(h, 2),
                     bvec_of(h, 3));
  }
  if (p.bloch) {
    TRY(build_tab(h, TAB_BV, 0, 1, c.t_initial, 0.0, -0.25 * p.dbeta, 0.0, 0.5 * h->V_min, 0, 0.0));
    return build_tab(h, TAB_BK, 1, 1, c.t_initial, 0.0, -0.5 * p.dbeta, 0.0, 0.5 * h->K_min, 0, 0.0);
  }
  const double half = 0.5 * c.dt;
  // expV: exp(-i dt/2 [V(X,t+dt/2) - V(X',t+dt/2)]) abs_boundary_x(X) abs_boundary_x(X')  (vn:754-770)
  TRY(build_tab(h, TAB_V1, 0, 0, tn + half, 0.0, -half, 0.0, 0.0, c.absx_mode ? 1 : 0, 0.0));
  // expK: exp(-i dt [K(P,t+dt/2) - K(P',t+dt/2)]) abs_boundary_p(P) abs_boundary_p(P')    (vn:733-745)
  if (kfirst) TRY(build_tab(h, TAB_K, 1, 0, tn + half, 0.0, -c.dt, 0.0, 0.0, c.absp_mode ? 1 : 0, 0.0));
  return AW_OK;
}

// momentum-space diagonal of rho_n:  M_k = (1/N) Sum_i [fft1(S rho_n)]_ik exp(+2 pi i k i / N),
// so that Tr[g(p) rho] dX = Sum_k g(P_k) M_k dX (the p branch of get_average, vn:548-561).  With
// d = j - i the double sum is a DFT of the diagonal sums of S rho_n:
//   M_k = (1/N) Sum_d G_d exp(-2 pi i k d / N),   G_d = Sum_i (S rho_n)_{i, (i + d) mod N},
// so the row pass stores its branch point rotated (no transform), a column pass adds the diagonals and
// one N-point DFT a step gives M (aw_k_diag_dft).
//   hist: the first instance's rows (hist_stride values apart), instances inst_stride values apart
static int vn_run(aw_state_s* h, const VnPlan& p, long long steps, const std::vector<double>& times, double* hist,
                  int hist_stride, long long inst_stride = 0) {
  const aw_config& c = h->cfg;
  const bool vdep = !p.bloch && c.v_time_dependent;
  const bool kdep = !p.bloch && c.k_time_dependent;
  const int N = h->nc;
  if (h->ni > 1 && p.observables) return fail(AW_E_STATE, "per-step observables need a single propagator");
  TRY(vinv_reset(h));
  TRY(reset_stops(h));  // a stop raised by an earlier call must not persist
  const int* stop = p.stop_on_purity || h->ni > 1 ? (const int*)dstop(h) : nullptr;
  const int nrb = row_blocks(h, h->nr, h->nc);
  const int vslot = p.bloch ? TAB_BV : TAB_V1;
  const int kslot = p.bloch ? TAB_BK : TAB_K;
  // for time-dependent V the next step's kick needs its own table
  if (!vdep) TRY(vn_tables(h, p, times[1], true));
  {
    if (vdep) TRY(vn_tables(h, p, times[1], !kdep));
    AwPassArgs a = pnone(h);
    a.in = a.out = h->rho.p;
    a.f2 = ftab(h, vslot);
    a.f2.sign = 1;
    a.d2 = +1;
    a.stop = stop;
    TRY(row_pass(h, a, h->tw_r));
  }
  for (long long n = 1; n <= steps; ++n) {
    const bool last = n == steps;
    {
      if (kdep) TRY(build_tab(h, TAB_K, 1, 0, times[n] + 0.5 * c.dt, 0.0, -c.dt, 0.0, 0.0, c.absp_mode ? 1 : 0, 0.0));
      // the previous step's 1/trace is applied by the row pass below, with its V kick's line constant
      // (every pass between is linear): one product a line there instead of one a point here
      AwPassArgs a = pnone(h);
      a.in = a.out = h->rho.p;
      a.d1 = -1;
      a.f1 = ftab(h, kslot);
      a.d2 = +1;
      a.stop = stop;
      a.lines_hint = h->tuned_col_lines;
      a.tma = h->tuned_col_tma;
      a.shape = h->tuned_col_shape;
      TRY(col_pass(h, a, h->tw_c));
    }
    {
      if (vdep) {
        // tables at t_n and at t_{n+1} for the fused kicks
        TRY(build_tab(h, TAB_V1, 0, 0, times[n] + 0.5 * c.dt, 0.0, -0.5 * c.dt, 0.0, 0.0, c.absx_mode ? 1 : 0, 0.0));
        if (!last)
          TRY(build_tab(h, TAB_V1B, 0, 0, times[n + 1] + 0.5 * c.dt, 0.0, -0.5 * c.dt, 0.0, 0.0, c.absx_mode ? 1 : 0, 0.0));
      }
      AwPassArgs a = pnone(h);
      a.in = a.out = h->rho.p;
      a.d1 = -1;
      a.shape = h->tuned_row_shape;
      a.f1 = ftab(h, vslot);
      a.f1.scale_ptr = dinv(h);  // 1/trace of the previous step (see the column pass)
      a.diag_out = (double2*)h->diag.p;
      if (p.stop_on_purity || p.bloch) a.red_abs2 = (double*)h->abs2.p;
      if (p.keep_rho) {
        a.mid_out = h->snap.p;
        a.mid_sign = 1;
      }
      if (p.observables) {
        // the branch point, each row i rotated left by i and signed (-1)^i: its alternating column
        // sums are the diagonal sums G_d (below)
        a.br_out = h->tmp.p;
        a.br_rot = 1;
      }
      if (!last) {
        a.f2 = ftab(h, vdep ? TAB_V1B : vslot);
        a.d2 = +1;
      } else {
        a.f2 = fsign();
      }
      a.stop = stop;
      TRY(row_pass(h, a, h->tw_r));
    }
    double* hrow = hist ? hist + (size_t)(n - 1) * hist_stride : nullptr;
    if (p.observables) {
      // G_d = Sum_i (S rho)_{i, i+d} (alternating column sums of the rotated branch), then
      // Re M_k = Re (1/N) Sum_d G_d exp(-2 pi i k d / N) into red_line
      AwPassArgs a = pnone(h);
      a.in = h->tmp.p;
      a.col_alt = (double2*)h->gdiag.p;
      a.stop = stop;
      TRY(col_pass(h, a, h->tw_c));
      KL(aw_k_diag_dft((const double2*)h->gdiag.p, N, (double2*)h->gdiag.p + N, (double*)h->red_line.p, 1.0 / N,
                       h->st));
    }
    if (p.bloch || !p.observables) {
      KL(aw_k_trace_finalize_n((const double2*)h->diag.p + (size_t)h->v0 * N,
                               N, (const double*)h->abs2.p + (size_t)h->v0 * nrb, nrb, c.dX,
                               p.complex_trace, dinv(h, h->v0), p.observables ? nullptr : hrow, inst_stride,
                               dstop(h, h->v0), p.stop_on_purity, h->vc, h->st));
    }
    if (p.observables) {
      FinalArgs f{(const double*)h->diag.p, 2, N, (const double*)h->red_line.p, 1, N, 0, nullptr, c.dX,
                  p.bloch ? nullptr : dinv(h), 0, 0};
      TRY(launch_finalize_args(h, f, times[n], hrow, 0));
    }
  }
  return AW_OK;
}

int vn_propagate(aw_state_s* h, long long steps, double* t) {
  const aw_config& c = h->cfg;
  std::vector<double> times(steps + 2);
  times[0] = *t;
  for (long long n = 1; n <= steps + 1; ++n) times[n] = times[n - 1] + c.dt;
  TRY(ensure_hist(h, steps + 1));
  if (steps == 0) return AW_OK;
  VnPlan p{false, 0.0, c.ehrenfest != 0, false, 0, 0};
  TRY(vn_run(h, p, steps, times, c.ehrenfest ? hist_of(h, h->v0) : nullptr, h->hist_cols));
  TRY(settle(h));
  TRY(vscale(h, h->rho.p, gsz(h)));
  h->hist_rows = c.ehrenfest ? steps : 0;
  *t = times[steps];
  return AW_OK;
}

// ============================================================================ grouped propagation
// von Neumann propagators of different grid sizes (each a single propagator or a batch) advanced
// together (no counterpart in the reference, which runs one propagator per script).  Short members
// (group_own below): each pass of a step is one persistent launch over the tiles of all of them
// (aw_group.cuh), the trace normalisation one launch over all their instances; the steps are
// rho_vneumann_cuda_1d.py:429-448 as in vn_run, every member computing with 8 elements a thread
// (radix-8 stages) in both passes, the same bits whichever other members share the launch.  Longer
// members fill the GPU with their own launches: they run their own step loop (vn_propagate, the bits
// of aw_propagate) on their own streams, concurrently with the grouped launches.
//   Measured against the same propagators each through its own propagate() on its own stream (which
// the device overlaps), 8 members of one side: complex64 1.9x (64), 1.8x (128), 1.3x (256); double-float
// 1.5x, 1.4x, 0.94x; native FP64 1.2x, 1.3x, 0.78x; members of 512 and more ran at 0.6-0.97x grouped.
static bool group_own(const aw_state_s* h) { return h->nc > (h->f32 ? 256 : 128); }
namespace {
struct StreamSwap {  // the members' work goes to one stream for the duration of the call
  std::vector<std::pair<aw_state_s*, cudaStream_t>> saved;
  ~StreamSwap() {
    for (auto& p : saved) p.first->st = p.second;
  }
};
}  // namespace

static int group_pass(aw_handle* hs, int count, bool row, std::vector<AwPassArgs>& args, cudaStream_t st) {
  AwGroupArgs g;
  memset(&g, 0, sizeof g);
  g.count = count;
  for (int m = 0; m < count; ++m) {
    aw_state_s* h = hs[m];
    const AwPassArgs& q = args[m];
    // the grouped kernel is compiled without these outputs (aw_pass_body's LEAN form)
    if (q.br_out || q.mid_out || q.red_abs2 || q.red_line || q.red_cross || q.red_sq || q.col_alt || q.alt_cross ||
        q.tma || q.cluster > 1)
      return fail(AW_E_STATE, "grouped passes store no branch, mid-point or reduction outputs");
    TRY(prep_pass(h, args[m], row ? h->tw_r : h->tw_c, row, st));
    const int lines = aw_group_tile_lines(row ? h->nc : h->nr);
    g.tiles_x[m] = (row ? h->nr : h->nc) / lines;
    g.start[m + 1] = g.start[m] + g.tiles_x[m] * h->vc;
    g.a[m] = args[m];
  }
  const aw_state_s* h0 = hs[0];
  const int r = h0->df ? aw_launch_group_df(&g, row, st) : (h0->f32 ? aw_launch_group_f32(&g, row, st)
                                                                     : aw_launch_group_f64(&g, row, st));
  ++g_launches;
  if (r) return fail(AW_E_CUDA, "grouped %s pass launch failed (%d, %s)", row ? "row" : "column", r,
                     cudaGetErrorString(cudaGetLastError()));
  for (int m = 0; m < count; ++m)
    if (hs[m]->df) df_outputs(hs[m], args[m], hs[m]->vc);
  return AW_OK;
}

static int group_run(aw_handle* hs, int count, int64_t steps, double** tp);

extern "C" int aw_group_propagate(aw_handle* hs, int32_t count, int64_t steps, double* t) {
  if (!hs || !t) return fail(AW_E_ARG, "aw_group_propagate: null argument");
  if (count < 1 || count > AW_GROUP_MAX) return fail(AW_E_ARG, "aw_group_propagate: 1 to %d propagators", AW_GROUP_MAX);
  if (steps < 0) return fail(AW_E_ARG, "aw_group_propagate: negative step count");
  for (int m = 0; m < count; ++m) {
    aw_state_s* h = hs[m];
    if (!h) return fail(AW_E_ARG, "aw_group_propagate: null handle %d", m);
    for (int k = 0; k < m; ++k)
      if (hs[k] == h) return fail(AW_E_ARG, "aw_group_propagate: handle %d appears twice", m);
    const aw_config& c = h->cfg;
    if (h->kind != AW_RHO_VNEUMANN)
      return fail(AW_E_STATE, "aw_group_propagate: von Neumann propagators only (member %d)", m);
    if (c.ehrenfest || c.v_time_dependent || c.k_time_dependent || c.absx_mode == 2 || c.absp_mode == 2)
      return fail(AW_E_STATE, "aw_group_propagate: member %d records observables or has a time-dependent V, K or "
                              "absorber", m);
    if (h->nc < 64 || h->nc > 2048 || (h->nc & (h->nc - 1)) || h->nr != h->nc)
      return fail(AW_E_ARG, "aw_group_propagate: grid sides 64 to 2048 (member %d: %d)", m, h->nc);
    if (h->df != hs[0]->df || h->f32 != hs[0]->f32)
      return fail(AW_E_ARG, "aw_group_propagate: all members in one arithmetic form");
  }
  // the large members: their own step loops, enqueued first on their own streams
  std::vector<aw_state_s*> grouped;
  std::vector<double*> gt;
  for (int m = 0; m < count; ++m) {
    if (group_own(hs[m])) {
      Settled guard{hs[m]};
      TRY(vn_propagate(hs[m], steps, &t[m]));
    } else {
      grouped.push_back(hs[m]);
      gt.push_back(&t[m]);
    }
  }
  return grouped.empty() ? AW_OK : group_run(grouped.data(), (int)grouped.size(), steps, gt.data());
}

// the grouped launches of the short members (validated by aw_group_propagate)
static int group_run(aw_handle* hs, int count, int64_t steps, double** tp) {
  for (int m = 0; m < count; ++m) CK(cudaStreamSynchronize(hs[m]->st));
  StreamSwap swap;
  cudaStream_t st = hs[0]->st;
  for (int m = 1; m < count; ++m) {
    swap.saved.push_back({hs[m], hs[m]->st});
    hs[m]->st = st;
  }
  // the states go back to complex128 however the call ends (before the streams are restored)
  std::vector<Settled> guards;
  guards.reserve(count);
  for (int m = 0; m < count; ++m) guards.push_back(Settled{hs[m]});
  std::vector<std::vector<double>> times(count);
  VnPlan p{false, 0.0, false, false, 0, 0};
  for (int m = 0; m < count; ++m) {
    aw_state_s* h = hs[m];
    times[m].resize(steps + 2);
    times[m][0] = *tp[m];
    for (long long n = 1; n <= steps + 1; ++n) times[m][n] = times[m][n - 1] + h->cfg.dt;
    TRY(ensure_hist(h, steps + 1));
    h->hist_rows = 0;
    if (steps == 0) continue;
    TRY(vinv_reset(h));
    TRY(reset_stops(h));
    TRY(vn_tables(h, p, times[m][1], true));
  }
  if (steps == 0) return AW_OK;
  std::vector<AwPassArgs> args(count);
  auto stop_of = [&](aw_state_s* h) -> const int* { return h->ni > 1 ? (const int*)dstop(h) : nullptr; };
  // first kick: rho (position) -> S V(t_1) -> fft1
  for (int m = 0; m < count; ++m) {
    aw_state_s* h = hs[m];
    AwPassArgs a = pnone(h);
    a.in = a.out = h->rho.p;
    a.f2 = ftab(h, TAB_V1);
    a.f2.sign = 1;
    a.d2 = +1;
    a.stop = stop_of(h);
    args[m] = a;
  }
  TRY(group_pass(hs, count, true, args, st));
  AwTraceGroup tg;
  memset(&tg, 0, sizeof tg);
  tg.count = count;
  for (int m = 0; m < count; ++m) {
    aw_state_s* h = hs[m];
    tg.diag[m] = (const double2*)h->diag.p + (size_t)h->v0 * h->nc;
    tg.n[m] = h->nc;
    tg.ninst[m] = h->vc;
    tg.dX[m] = h->cfg.dX;
    tg.inv[m] = dinv(h, h->v0);
    tg.stop[m] = dstop(h, h->v0);
  }
  for (long long n = 1; n <= steps; ++n) {
    const bool last = n == steps;
    for (int m = 0; m < count; ++m) {  // column pass: 1/trace, ifft0, K kick, fft0 (grouped members)
      aw_state_s* h = hs[m];
      AwPassArgs a = pnone(h);
      a.in = a.out = h->rho.p;
      a.f0 = fnone();
      a.f0.scale_ptr = dinv(h);
      a.f0.active = 1;
      a.d1 = -1;
      a.f1 = ftab(h, TAB_K);
      a.d2 = +1;
      a.stop = stop_of(h);
      args[m] = a;
    }
    TRY(group_pass(hs, count, false, args, st));
    for (int m = 0; m < count; ++m) {  // row pass: ifft1, V kick, diagonal, next kick, fft1
      aw_state_s* h = hs[m];
      AwPassArgs a = pnone(h);
      a.in = a.out = h->rho.p;
      a.d1 = -1;
      a.f1 = ftab(h, TAB_V1);
      a.diag_out = (double2*)h->diag.p;
      if (!last) {
        a.f2 = ftab(h, TAB_V1);
        a.d2 = +1;
      } else {
        a.f2 = fsign();
      }
      a.stop = stop_of(h);
      args[m] = a;
    }
    TRY(group_pass(hs, count, true, args, st));
    {
      const int r = aw_k_trace_finalize_group(&tg, st);
      ++g_launches;
      if (r) return fail(AW_E_CUDA, "grouped trace launch failed (%d)", r);
    }
  }
  for (int m = 0; m < count; ++m) {
    aw_state_s* h = hs[m];
    TRY(settle(h));
    TRY(vscale(h, h->rho.p, gsz(h)));
    *tp[m] = times[m][steps];
  }
  // each member's own stream continues after the group's work
  cudaEvent_t done;
  CK(cudaEventCreateWithFlags(&done, cudaEventDisableTiming));
  CK(cudaEventRecord(done, st));
  for (auto& sv : swap.saved) CK(cudaStreamWaitEvent(sv.second, done, 0));
  cudaEventDestroy(done);
  return AW_OK;
}

int vn_single_step(aw_state_s* h, double t) {
  const std::vector<double> times{t - h->cfg.dt, t, t + h->cfg.dt};
  VnPlan p{false, 0.0, false, false, 0, 0};
  return vn_run(h, p, 1, times, nullptr, h->hist_cols);
}

int vn_bloch_step(aw_state_s* h, double dbeta, double* out) {
  if (h->ni > 1) return fail(AW_E_STATE, "single rho-Bloch steps need a single propagator (use aw_gibbs_batch)");
  TRY(ensure_hist(h, 2));
  CK(cudaMemsetAsync(h->hist.p, 0, 2 * (size_t)h->hist_cols * 8, h->st));
  const bool obs = h->cfg.n_slots > 0;
  VnPlan p{true, dbeta, obs, false, 0, 1};
  std::vector<double> times(3, 0.0);
  // observables go to row 0, the trace finalize (purity, trace) to row 1
  TRY(vn_run(h, p, 1, times, (double*)h->hist.p, h->hist_cols));
  if (obs)
    KL(aw_k_trace_finalize((const double2*)h->diag.p, h->nc, (const double*)h->abs2.p,
                           row_blocks(h, h->nr, h->nc), h->cfg.dX, 1, dmisc(h, 0),
                           (double*)h->hist.p + h->hist_cols, nullptr, 0, h->st));
  TRY(settle(h));
  TRY(vscale(h, h->rho.p, gsz(h)));
  if (out) {
    std::vector<double> hh(2 * (size_t)h->hist_cols);
    CK(cudaMemcpyAsync(hh.data(), h->hist.p, hh.size() * 8, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    const int ns = h->cfg.n_slots;
    for (int k = 0; k < ns; ++k) out[k] = hh[k];
    out[ns] = obs ? hh[h->hist_cols] : hh[0];  // purity
    out[ns + 1] = obs ? hh[h->hist_cols + 1] : hh[1];
  }
  CK(cudaStreamSynchronize(h->st));
  return AW_OK;
}

int vn_gibbs(aw_state_s* h, const double* dbeta, long long steps, long long* done, double* purity) {
  for (int k = 0; k < h->vc; ++k) done[k] = 0;
  if (steps <= 0) return AW_OK;
  const int hc = 3;  // purity, Re trace, Im trace
  TRY(ensure_hist(h, steps + 1, hc));
  CK(cudaMemsetAsync(h->hist.p, 0, (size_t)h->ni * h->hist_cap * hc * 8, h->st));
  TRY(dalloc(h->snap, (size_t)h->ni * gsz(h) * h->esz));
  VnPlan p{true, dbeta[0], false, true, 1, 1};
  if (h->ni > 1) {
    TRY(upload_bloch(h, dbeta));
    p.per_inst = true;
  }
  std::vector<double> times(steps + 2, 0.0);
  TRY(vn_run(h, p, steps, times, hist_of(h, h->v0), hc, h->hist_cap * hc));
  std::vector<double> hh((size_t)h->vc * h->hist_cap * hc);
  CK(cudaMemcpyAsync(hh.data(), hist_of(h, h->v0), hh.size() * 8, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  std::vector<long long> ran(h->vc, 0);
  for (int k = 0; k < h->vc; ++k) {
    const double* hk = hh.data() + (size_t)k * h->hist_cap * hc;
    for (long long n = 0; n < steps; ++n) {
      if (hk[(size_t)n * hc + 1] == 0.0) break;
      ran[k] = n + 1;
    }
    done[k] = ran[k];
    if (purity && ran[k] > 0) purity[k] = hk[(size_t)(ran[k] - 1) * hc];
  }
  TRY(settle(h));
  for (int k = 0; k < h->vc; ++k) {
    const int i = h->v0 + k;
    if (ran[k] == 0) continue;
    CK(cudaMemcpyAsync(at_inst(h->rho.p, gsz(h), h->esz, i), at_inst(h->snap.p, gsz(h), h->esz, i),
                       (size_t)gsz(h) * h->esz, cudaMemcpyDeviceToDevice, h->st));
  }
  TRY(vscale(h, h->rho.p, gsz(h)));
  CK(cudaStreamSynchronize(h->st));
  h->hist_rows = 0;
  return AW_OK;
}

// get_wignerfunction (rho_vneumann_cuda_1d.py:387-427): embed rho in the centre of a zeroed
// (2N)^2 grid, sign flip, three shears, ifft0, sign flip, normalise by Re Sum W dXdP_wigner
static int vn_get_wigner(aw_state_s* h, int blackman) {
  const int N = h->nc, M = h->wn, pad = N / 2;
  if (blackman) TRY(ensure_blackman(h, M, M));
  const int v0 = h->v0, vc = h->vc;
  for (int i = v0; i < v0 + vc; ++i) {
    h->v0 = i;
    h->vc = 1;
    void* Wi = at_inst(h->W.p, (long long)M * M, h->esz, i);
    int r = 0;
    {
      cudaEvent_t pe_ = prof_mark(h);
      r = aw_k_embed(at_inst(h->rho.p, gsz(h), h->esz, i), h->f32, N, Wi, M, pad, h->st);
      prof_done(h, PROF_UTIL, 0.0, pe_);
      ++g_launches;
      if (r) r = fail(AW_E_CUDA, "embedding launch failed");
    }
    WignerGrid g{h->W.p, M, M, &h->tw_w, &h->tw_w};
    if (!r) r = wigner_passes(h, g, h->W.p, fsign(), blackman != 0, false, true);
    if (!r) r = settle(h);
    double sm[2] = {0.0, 0.0};
    if (!r) r = dsum(h, Wi, (long long)M * M, 0, 0, sm);
    if (!r) {
      cudaEvent_t pe_ = prof_mark(h);
      r = aw_k_scale(Wi, h->f32, (long long)M * M, 1.0 / (sm[0] * h->cfg.dXdP), 0.0, nullptr, h->st);
      prof_done(h, PROF_UTIL, 0.0, pe_);
      ++g_launches;
      if (r) r = fail(AW_E_CUDA, "scale launch failed");
    }
    h->v0 = v0;
    h->vc = vc;
    TRY(r);
  }
  return AW_OK;
}

extern "C" int aw_average_ops(aw_handle h, const char* const* ops, int32_t n_ops, double t, double* out) {
  if (!h || !out) return fail(AW_E_ARG, "null argument");
  if (!h->kn.vn) return fail(AW_E_STATE, "ordered operator averages are defined for density matrices");
  Settled guard{h};
  const long long n = (long long)h->nr * h->nc;
  const int keep_v0 = h->v0, keep_vc = h->vc;
  // the first instance of the view, copied to the scratch buffer (which the passes treat as instance 0)
  CK(cudaMemcpyAsync(h->tmp.p, at_inst(h->rho.p, n, h->esz, h->v0), n * h->esz, cudaMemcpyDeviceToDevice, h->st));
  h->v0 = 0;
  h->vc = 1;
  struct ViewBack {
    aw_state_s* h;
    int v0, vc;
    ~ViewBack() {
      h->v0 = v0;
      h->vc = vc;
    }
  } view_back{h, keep_v0, keep_vc};
  TRY(clear_stops(h));
  bool is_x = false;
  for (int k = 0; k < n_ops; ++k) {
    is_x = !is_x;
    if (!ops[k] || !ops[k][0]) continue;
    cudaKernel_t kern;
    TRY(get_obs_kernel(h, ops[k], &kern));
    void* buf = h->tmp.p;
    int f32 = h->f32, nr = h->nr, nc = h->nc;
    double* unused = nullptr;
    double dX = h->cfg.dX, dP = h->cfg.dP;
    void* args[] = {&buf, &f32, &t, &unused, &nr, &nc, &dX, &dP};
    if (is_x) {
      TRY(settle(h));
      TRY(hjit(h, kern, dim3((nc + 127) / 128, nr), dim3(128), args));
    } else {
      // sign flip, fft1, / N, observable, ifft1, sign flip (rho_vneumann_cuda_1d.py:549-561)
      AwPassArgs a = pnone(h);
      a.in = a.out = h->tmp.p;
      a.f0 = fsign();
      a.d1 = +1;
      a.f1 = fnone();
      a.f1.scale = 1.0 / nc;
      a.f1.active = 1;
      TRY(row_pass(h, a, h->tw_r));
      TRY(settle(h));
      TRY(hjit(h, kern, dim3((nc + 127) / 128, nr), dim3(128), args));
      a = pnone(h);
      a.in = a.out = h->tmp.p;
      a.d1 = -1;
      a.f3 = fsign();
      TRY(row_pass(h, a, h->tw_r));
    }
  }
  TRY(settle(h));
  double s[2];
  TRY(dsum(h, h->tmp.p, h->nr, 3, h->nc + 1, s));
  *out = s[0] * h->cfg.dX;
  return AW_OK;
}

// ============================================================================ Schrodinger
// psi on N points, stored as row 0 of a small zero-padded tile so that the row pass
// kernels apply unchanged.  One step (schrodinger_wigner_cuda_1d.py:356-390):
//   expV(t) -> fft -> expK(t) -> ifft -> expV(t) -> [Ehrenfest] -> psi /= ||psi|| sqrt(dX)
static int sw_tables(aw_state_s* h, double t) {
  const aw_config& c = h->cfg;
  TRY(build_tab(h, TAB_V1, 0, 0, t, 0.0, -0.5 * c.dt, 0.0, 0.0, c.absx_mode ? 1 : 0, t));
  return build_tab(h, TAB_K, 1, 0, t, 0.0, -c.dt, 0.0, 0.0, c.absp_mode ? 1 : 0, t);
}

static AwPassArgs sw_args(aw_state_s* h) {
  AwPassArgs a = pnone(h);
  a.nrows = h->sw_rows;
  a.ncols = h->nc;
  return a;
}

// 1-D table of N entries (slot) as a factor of a wave-function pass; lin selects how a long wave
// function's matrix view reads it (1: natural order, 2: the four-step spectrum order)
static AwFactor sw_tab(aw_state_s* h, int slot, int lin) {
  AwFactor f = ftab(h, slot);
  f.row_tab = nullptr;
  f.lin = h->sw_n1 ? lin : 0;
  return f;
}

// pre (x) -> FFT -> mid (p) -> [IFFT -> post (x)] on a wave function, in -> out.
//   Single tile (N <= 8192): one row pass.  Longer: psi as the N1 x N2 matrix n = n1 N2 + n2 and the
//   four-step FFT (Bailey, "FFTs in external or hierarchical memory", 1990): column FFTs of length
//   N1, the twiddle exp(-2 pi i n2 k1 / N), row FFTs of length N2; the spectrum sits in the order
//   k = k1 + N1 k2 at (k1, k2), which the mid factor reads its table in (lin = 2), and the inverse
//   retraces the steps.  fwd_only stops after mid; red_abs2 receives per-block sums of |out|^2.
//   Returns the number of norm partials in *nparts.
static int sw_run(aw_state_s* h, const void* in, void* out, const AwFactor& pre, const AwFactor& mid,
                  const AwFactor& post, bool fwd_only, double* red_abs2, int* nparts) {
  if (!h->sw_n1) {
    AwPassArgs a = sw_args(h);
    a.in = in;
    a.out = out;
    a.f0 = pre;
    a.d1 = +1;
    a.f1 = mid;
    if (!fwd_only) {
      a.d2 = -1;
      a.f3 = post;
    }
    if (red_abs2) {
      a.red_abs2 = red_abs2;
      a.abs2_end = 1;
    }
    TRY(row_pass(h, a, h->tw_r));
    if (nparts) *nparts = row_blocks(h, h->sw_rows, h->nc);
    return AW_OK;
  }
  const int n1 = h->sw_n1, n2 = h->sw_n2;
  auto twist = [&](bool inv) {
    AwFactor f = fnone();
    f.sh_hi = (inv ? h->swi_hi : h->swf_hi).p;
    f.sh_lo = (inv ? h->swi_lo : h->swf_lo).p;
    f.sh_lo_n = h->swt_lo_n;
    f.active = 1;
    return f;
  };
  AwPassArgs a = pnone(h);
  a.nrows = n1;
  a.ncols = n2;
  a.in = in;
  a.out = out;
  a.f0 = pre;
  a.d1 = +1;
  a.f1 = twist(false);
  TRY(col_pass(h, a, h->tw_l1));
  a = pnone(h);
  a.nrows = n1;
  a.ncols = n2;
  a.in = a.out = out;
  a.d1 = +1;
  a.f1 = mid;
  if (!fwd_only) a.d2 = -1;
  TRY(row_pass(h, a, h->tw_l2));
  if (fwd_only) return AW_OK;
  a = pnone(h);
  a.nrows = n1;
  a.ncols = n2;
  a.in = a.out = out;
  a.f0 = twist(true);
  a.d1 = -1;
  a.f1 = post;
  if (red_abs2) {
    a.red_abs2 = red_abs2;
    a.abs2_end = 1;
  }
  TRY(col_pass(h, a, h->tw_l1));
  if (nparts) *nparts = aw_col_pass_blocks(n1, n2, h->f32);
  return AW_OK;
}

static int sw_finalize(aw_state_s* h, double t, double* hrow) {
  const int N = h->nc;
  double* xm = (double*)h->red_line.p;    // |psi_j|^2
  double* pmar = (double*)h->red_cross.p; // |(fft psi)_k|^2
  KL(aw_k_abs2(h->W.p, h->f32, N, xm, h->st));
  if (h->sw_n1) {
    KL(aw_k_abs2_perm(h->tmp.p, h->f32, N, h->sw_n1, pmar, h->st));
  } else {
    KL(aw_k_abs2(h->tmp.p, h->f32, N, pmar, h->st));
  }
  FinalArgs f{xm, 1, N, pmar, 1, N, N / 2, nullptr, h->cfg.dX, dinv(h), 1, 1};
  return launch_finalize_args(h, f, t, hrow, 0);
}

int sw_propagate(aw_state_s* h, long long steps, double* t) {
  const aw_config& c = h->cfg;
  std::vector<double> times(steps + 2);
  times[0] = *t;
  for (long long n = 1; n <= steps + 1; ++n) times[n] = times[n - 1] + c.dt;
  TRY(ensure_hist(h, steps + 1));
  if (steps == 0) return AW_OK;
  const bool tdep = c.v_time_dependent || c.k_time_dependent || c.absx_mode == 2 || c.absp_mode == 2;
  KL(aw_k_set2(dinv(h), 1.0, 0.0, h->st));
  if (!tdep) TRY(sw_tables(h, times[1]));
  for (long long n = 1; n <= steps; ++n) {
    if (tdep) TRY(sw_tables(h, times[n]));
    AwFactor pre = sw_tab(h, TAB_V1, 1);
    pre.scale_ptr = dinv(h);
    const AwFactor mid = sw_tab(h, TAB_K, 2), post = sw_tab(h, TAB_V1, 1);
    int nb = 0;
    if (c.ehrenfest) {
      // psi' -> W buffer; its momentum representation -> tmp
      TRY(sw_run(h, h->rho.p, h->W.p, pre, mid, post, false, nullptr, nullptr));
      TRY(sw_run(h, h->W.p, h->tmp.p, fnone(), fnone(), fnone(), true, nullptr, nullptr));
      TRY(sw_finalize(h, times[n], (double*)h->hist.p + (size_t)(n - 1) * h->hist_cols));
      CK(cudaMemcpyAsync(h->rho.p, h->W.p, (size_t)h->sw_rows * h->nc * h->esz, cudaMemcpyDeviceToDevice, h->st));
    } else {
      TRY(sw_run(h, h->rho.p, h->rho.p, pre, mid, post, false, (double*)h->abs2.p, &nb));
      KL(aw_k_norm_finalize((const double*)h->abs2.p, nb, c.dX, dinv(h), nullptr, h->st));
    }
  }
  KL(aw_k_scale(h->rho.p, h->f32, h->nc, 1.0, 0.0, dinv(h), h->st));
  h->hist_rows = c.ehrenfest ? steps : 0;
  *t = times[steps];
  return AW_OK;
}

int sw_single_step(aw_state_s* h, double t) {
  TRY(sw_tables(h, t));
  const AwFactor pre = sw_tab(h, TAB_V1, 1), mid = sw_tab(h, TAB_K, 2), post = sw_tab(h, TAB_V1, 1);
  return sw_run(h, h->rho.p, h->rho.p, pre, mid, post, false, nullptr, nullptr);
}

// get_Ehrenfest of the Schrodinger propagator (schrodinger_wigner_cuda_1d.py:412-459) for the
// current wave function at time t: one row of observables (n_slots + 2 values).  The observables
// are ratios to the norms of psi and of its momentum representation, so psi itself is left as it
// is (the reference rescales it to sqrt(N) psi / |psi| on the way).
extern "C" int aw_sw_ehrenfest(aw_handle h, double t, double* row) {
  if (!h || !row) return fail(AW_E_ARG, "null argument");
  if (!h->kn.sw) return fail(AW_E_STATE, "aw_sw_ehrenfest needs the Schrodinger propagator");
  if (!h->cfg.ehrenfest) return fail(AW_E_STATE, "the propagator records no Ehrenfest observables");
  Settled guard{h};
  TRY(ensure_hist(h, 1));
  CK(cudaMemcpyAsync(h->W.p, h->rho.p, (size_t)h->sw_rows * h->nc * h->esz, cudaMemcpyDeviceToDevice, h->st));
  TRY(sw_run(h, h->rho.p, h->tmp.p, fnone(), fnone(), fnone(), true, nullptr, nullptr));
  TRY(sw_finalize(h, t, (double*)h->hist.p));
  CK(cudaMemcpyAsync(row, h->hist.p, (size_t)h->hist_cols * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  return AW_OK;
}

// get_wigner / get_wigner_blackman (schrodinger_wigner_cuda_1d.py:593-663)
static int sw_get_wigner(aw_state_s* h, int blackman) {
  const int N = h->nc;
  if (!h->wn) return fail(AW_E_STATE, "the Wigner function of a wave function longer than 8192 points (an N x N grid) is not formed");
  KL(aw_k_psi2rho(h->rho.p, h->f32, N, h->W.p, h->st));
  if (blackman) TRY(ensure_blackman(h, N, N));
  void* bcol = blackman ? h->blk_tabs.p : nullptr;
  void* brow = blackman ? (char*)h->blk_tabs.p + (size_t)N * h->esz : nullptr;
  AwFactor shx = fshear_x(h), shy = fshear_y(h);
  shx.sh_roll = N / 2;
  shy.sh_roll = N / 2;
  AwPassArgs a = pnone(h);
  a.nrows = a.ncols = N;
  a.in = a.out = h->W.p;
  if (blackman) { a.f0.col_tab = bcol; a.f0.active = 1; }
  a.d1 = +1; a.f1 = shx; a.d2 = -1;
  TRY(row_pass(h, a, h->tw_w));
  a = pnone(h);
  a.nrows = a.ncols = N;
  a.in = a.out = h->W.p;
  if (blackman) { a.f0.row_tab = brow; a.f0.active = 1; }
  a.d1 = +1; a.f1 = shy; a.d2 = -1;
  TRY(col_pass(h, a, h->tw_w));
  a = pnone(h);
  a.nrows = a.ncols = N;
  a.in = a.out = h->W.p;
  if (blackman) { a.f0.col_tab = bcol; a.f0.active = 1; }
  a.d1 = +1; a.f1 = shx; a.d2 = -1;
  TRY(row_pass(h, a, h->tw_w));
  a = pnone(h);
  a.nrows = a.ncols = N;
  a.in = a.out = h->W.p;
  a.f0 = fnone();
  a.f0.sign = 2;
  a.f0.active = 1;
  if (blackman) a.f0.row_tab = brow;
  a.d1 = -1;
  a.f3 = fnone();
  a.f3.sign = 2;
  a.f3.active = 1;
  TRY(col_pass(h, a, h->tw_w));
  double s[2];
  TRY(dsum(h, h->W.p, (long long)N * N, 0, 0, s));
  KL(aw_k_scale(h->W.p, h->f32, (long long)N * N, 1.0 / (s[0] * h->cfg.dXdP), 0.0, nullptr, h->st));
  return AW_OK;
}

// imaginary-time steps (set_ground_state / get_stationary_states, sw:484-591)
extern "C" int aw_sw_imag_steps(aw_handle h, int64_t steps, int32_t project) {
  if (!h) return fail(AW_E_ARG, "null handle");
  if (!h->kn.sw) return fail(AW_E_STATE, "imaginary-time wave-function steps need the Schrodinger propagator");
  const aw_config& c = h->cfg;
  // bloch_expV = exp(-dt/2 V(X, t_initial)), bloch_expK = exp(-dt K(P, t_initial))  (sw:834-854)
  TRY(build_tab(h, TAB_BV, 0, 1, c.t_initial, 0.0, -0.5 * c.dt, 0.0, 0.0, 0, 0.0));
  TRY(build_tab(h, TAB_BK, 1, 1, c.t_initial, 0.0, -c.dt, 0.0, 0.0, 0, 0.0));
  const int N = h->nc;
  for (long long n = 0; n < steps; ++n) {
    int nb = 0;
    TRY(sw_run(h, h->rho.p, h->rho.p, sw_tab(h, TAB_BV, 1), sw_tab(h, TAB_BK, 2), sw_tab(h, TAB_BV, 1), false,
               project ? nullptr : (double*)h->abs2.p, &nb));
    if (!project) {
      // psi /= norm(psi) sqrt(dX)
      KL(aw_k_norm_finalize((const double*)h->abs2.p, nb, c.dX, dinv(h), nullptr, h->st));
      KL(aw_k_scale(h->rho.p, h->f32, N, 1.0, 0.0, dinv(h), h->st));
    } else {
      // projectout_stationary_states (sw:505-550): normalise, subtract projections, normalise
      double s[2];
      TRY(dsum(h, h->rho.p, N, 2, 0, s));
      KL(aw_k_scale(h->rho.p, h->f32, N, 1.0 / sqrt(s[0]), 0.0, nullptr, h->st));
      std::vector<double2> proj(h->sw_states.size());
      for (size_t q = 0; q < h->sw_states.size(); ++q) {
        // <phi_q | psi>
        KL(aw_k_vdot(h->sw_states[q].p, h->rho.p, h->f32, N, (double2*)h->part.p, 256, h->st));
        std::vector<double2> hp(256);
        CK(cudaMemcpyAsync(hp.data(), h->part.p, 256 * sizeof(double2), cudaMemcpyDeviceToHost, h->st));
        CK(cudaStreamSynchronize(h->st));
        double re = 0, im = 0;
        for (auto& v : hp) { re += v.x; im += v.y; }
        proj[q] = make_double2(re, im);
      }
      for (size_t q = 0; q < h->sw_states.size(); ++q)
        KL(aw_k_axpy(h->rho.p, h->sw_states[q].p, h->f32, N, -proj[q].x, -proj[q].y, h->st));
      TRY(dsum(h, h->rho.p, N, 2, 0, s));
      KL(aw_k_scale(h->rho.p, h->f32, N, 1.0 / sqrt(s[0]), 0.0, nullptr, h->st));
    }
  }
  CK(cudaStreamSynchronize(h->st));
  return AW_OK;
}

extern "C" int aw_sw_store_state(aw_handle h) {
  if (!h || !h->kn.sw) return fail(AW_E_STATE, "stationary states need the Schrodinger propagator");
  DevBuf b;
  TRY(dalloc(b, (size_t)h->nc * h->esz));
  CK(cudaMemcpyAsync(b.p, h->rho.p, (size_t)h->nc * h->esz, cudaMemcpyDeviceToDevice, h->st));
  h->sw_states.push_back(b);
  return AW_OK;
}

extern "C" int aw_sw_clear_states(aw_handle h) {
  if (!h) return fail(AW_E_ARG, "null handle");
  for (DevBuf& b : h->sw_states) dfree(b);
  h->sw_states.clear();
  return AW_OK;
}

extern "C" int aw_sw_get_state(aw_handle h, int32_t index, void* dst_host) {
  if (!h || !dst_host) return fail(AW_E_ARG, "null argument");
  if (index < 0 || index >= (int)h->sw_states.size()) return fail(AW_E_ARG, "no stationary state %d", index);
  const void* src = h->sw_states[index].p;
  if (h->f32) {
    KL(aw_k_convert(src, 1, h->tmp.p, 0, h->nc, h->st));
    src = h->tmp.p;
  }
  CK(cudaMemcpyAsync(dst_host, src, (size_t)h->nc * 16, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  return AW_OK;
}

// get_energy (sw:461-482): <V> over |psi|^2 / Sum |psi|^2 plus <K> over |fft psi|^2 / Sum |fft psi|^2
extern "C" int aw_sw_energy(aw_handle h, double t, double* out) {
  if (!h || !out) return fail(AW_E_ARG, "null argument");
  if (!h->kn.sw) return fail(AW_E_STATE, "get_energy needs the Schrodinger propagator");
  double v, k, n1[2], n2[2];
  TRY(dsum(h, h->rho.p, h->nc, 2, 0, n1));
  TRY(aw_average(h, h->V.c_str(), t, &v));
  TRY(sw_run(h, h->rho.p, h->tmp.p, fnone(), fnone(), fnone(), true, nullptr, nullptr));
  const void* src = h->tmp.p;
  if (h->sw_n1) {
    // the four-step spectrum into natural order (the W buffer is scratch for a long wave function)
    KL(aw_k_unpermute(h->tmp.p, h->W.p, h->f32, h->nc, h->sw_n1, h->st));
    src = h->W.p;
  }
  TRY(dsum(h, src, h->nc, 2, 0, n2));
  // average of K over the momentum representation
  cudaKernel_t kern;
  TRY(get_obs_kernel(h, h->K.c_str(), &kern));
  int f32 = h->f32, nr = 1, nc = h->nc;
  double* part = (double*)h->part.p;
  double dX = h->cfg.dX, dP = h->cfg.dP;
  void* args[] = {&src, &f32, &t, &part, &nr, &nc, &dX, &dP};
  TRY(hjit(h, kern, dim3(256), dim3(256), args));
  std::vector<double> hp(256);
  CK(cudaMemcpyAsync(hp.data(), part, 256 * 8, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  k = 0;
  for (double x : hp) k += x;
  *out = v / n1[0] + k / n2[0];
  return AW_OK;
}

// ============================================================================ batches
// Independent instances of one propagator kind and grid, stepped together: every pass launch
// covers the view's instances (blockIdx.y), each with its own state, tables, parameters, norm,
// stop flag and observable rows; no instance reads another's data, so an instance's results do
// not depend on which others share the batch.
static int clear_stops(aw_state_s* h) {
  CK(cudaMemsetAsync(dstop(h, h->v0), 0, (size_t)h->vc * sizeof(int), h->st));
  return AW_OK;
}

extern "C" int aw_set_view(aw_handle h, int32_t first, int32_t count) {
  if (!h) return fail(AW_E_ARG, "null handle");
  if (first < 0 || count < 1 || first + count > h->ni)
    return fail(AW_E_ARG, "view [%d, %d) outside the %d instances", first, first + count, h->ni);
  TRY(settle(h));
  h->v0 = first;
  h->vc = count;
  return AW_OK;
}

extern "C" int aw_set_params(aw_handle h, int32_t inst, const double* values) {
  if (!h || (!values && h->np)) return fail(AW_E_ARG, "null argument");
  if (inst < 0 || inst >= h->ni) return fail(AW_E_ARG, "no instance %d", inst);
  if (!h->np) return AW_OK;
  CK(cudaMemcpyAsync((double*)h->params.p + (size_t)inst * h->np, values, (size_t)h->np * sizeof(double),
                     cudaMemcpyHostToDevice, h->st));
  CK(cudaStreamSynchronize(h->st));
  h->minima_ok[inst] = 0;
  h->maskx_ready = h->maskp_ready = false;  // masks may depend on the parameters
  h->maskx_sep = false;
  h->maskx_t[0] = h->maskx_t[1] = NAN;
  return AW_OK;
}

extern "C" int aw_set_active(aw_handle h, const int32_t* flags) {
  if (!h || !flags) return fail(AW_E_ARG, "null argument");
  for (int i = 0; i < h->ni; ++i) h->active[i] = flags[i] != 0;
  return AW_OK;
}

extern "C" int aw_bloch_min_of(aw_handle h, int32_t inst, double* v_min, double* k_min) {
  if (!h) return fail(AW_E_ARG, "null handle");
  if (inst < 0 || inst >= h->ni) return fail(AW_E_ARG, "no instance %d", inst);
  if (h->kind != AW_WIGNER_BLOCH && h->kind != AW_RHO_BLOCH) return fail(AW_E_STATE, "minima exist for Bloch propagators");
  if (!h->minima_ok[inst]) TRY(bloch_minima(h, inst));
  if (v_min) *v_min = h->vmin_i[inst];
  if (k_min) *k_min = h->kmin_i[inst];
  return AW_OK;
}

extern "C" int aw_init_state(aw_handle h) {
  if (!h) return fail(AW_E_ARG, "null handle");
  if (!h->k_binit) return fail(AW_E_STATE, "the handle was created without init_expr");
  if (h->kn.sw) return fail(AW_E_STATE, "aw_init_state exists for the grid propagators");
  Settled guard{h};
  const long long n = gsz(h);
  void* dst = h->kn.rotated ? h->W.p : h->rho.p;
  for (int i = h->v0; i < h->v0 + h->vc; ++i) {
    void* out = at_inst(dst, n, h->esz, i);
    int f32 = h->f32, nr = h->nr, nc = h->nc;
    double da = h->cfg.dX, db = h->kn.rotated ? h->cfg.dP : h->cfg.dX;
    const double* prm = h->np ? (const double*)h->params.p + (size_t)i * h->np : nullptr;
    void* args[] = {&out, &f32, &nr, &nc, &da, &db, &prm};
    TRY(hjit(h, h->k_binit, dim3((nc + 127) / 128, nr), dim3(128), args));
    double s[2];
    if (h->kn.rotated) {
      // set_wignerfunction: W /= Sum W dXdP (complex, wigner_moyal_cuda_1d.py:415)
      TRY(dsum(h, out, n, 0, 0, s));
      const double d = (s[0] * s[0] + s[1] * s[1]) * h->cfg.dXdP;
      KL(aw_k_scale(out, h->f32, n, s[0] / d, -s[1] / d, nullptr, h->st));
    } else {
      // set_rho: rho /= Re Tr(rho) dX (rho_vneumann_cuda_1d.py:382-384)
      TRY(dsum(h, out, h->nr, 3, h->nc + 1, s));
      KL(aw_k_scale(out, h->f32, n, 1.0 / (s[0] * h->cfg.dX), 0.0, nullptr, h->st));
    }
  }
  if (h->kn.rotated) {
    TRY(clear_stops(h));
    TRY(wm_wigner2rho(h));
  }
  CK(cudaStreamSynchronize(h->st));
  return AW_OK;
}
