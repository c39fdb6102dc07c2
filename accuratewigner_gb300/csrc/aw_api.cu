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
#include <mutex>
#include <string>
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
  std::vector<char> cubin(n);
  nvrtcGetCUBIN(prog, cubin.data());
  nvrtcDestroyProgram(&prog);
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

struct aw_state_s {
  aw_config cfg;
  std::string consts, V, K, absx, absp;
  std::vector<std::string> obs_x, obs_p;
  std::vector<int> tslot, tkind, tidx;
  std::vector<double> tcoef;
  awjit::KindNames kn;
  int kind = 0, f32 = 0, esz = 16;
  int df = 0;                          // complex128 state, passes in double-float arithmetic
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
  DevBuf tabs;                         // phase tables, slots of (nc + nr) complex
  DevBuf vseq, vtimes;                 // time-dependent kick tables of a run of time points, their times
  DevBuf maskx, maskp;                 // 2-D masks (rotated frame)
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
  DevBuf twist_hi, twist_lo;           // von Neumann momentum-diagonal twist exp(2 pi i k i / N) / N
  int twist_lo_n = 0;
  int sw_rows = 1;                     // Schrodinger: rows of the zero-padded psi tile
  int red_blocks = 0;                  // column blocks of the Wigner column pass
  int row_blocks = 0;                  // row blocks of the main row pass
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
  std::vector<ProfRec> prof;
};

// launch classes of the profiler
enum { PROF_ROW = 0, PROF_COL = 1, PROF_JIT = 2, PROF_UTIL = 3, PROF_NCLS = 4 };

static cudaEvent_t prof_mark(aw_state_s* h) {
  cudaEvent_t e = nullptr;
  if (!h->prof_on) return e;
  cudaEventCreate(&e);
  cudaEventRecord(e, h->st);
  return e;
}
static void prof_done(aw_state_s* h, int cls, double bytes, cudaEvent_t a) {
  if (!h->prof_on || !a) return;
  cudaEvent_t b;
  cudaEventCreate(&b);
  cudaEventRecord(b, h->st);
  h->prof.push_back({cls, bytes, a, b});
}
static void prof_clear(aw_state_s* h) {
  for (auto& r : h->prof) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  h->prof.clear();
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
  cudaStreamSynchronize(h->st);
  prof_clear(h);
  h->prof_on = enable != 0;
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
// (each FP64 number as the FP32 pair hi = rn(v), lo = rn(v - hi)).
static int tab_fmt(const aw_state_s* h) { return h->f32 ? 1 : (h->df ? 2 : 0); }

// upload real numbers (interleaved re, im for complex tables) in table format fmt
static int upload_reals(DevBuf& dst, const std::vector<double>& v, int fmt) {
  const size_t n = v.size();
  TRY(dalloc(dst, n * (fmt == 1 ? 4 : 8)));
  if (n == 0) return AW_OK;
  if (fmt == 0) {
    CK(cudaMemcpy(dst.p, v.data(), n * 8, cudaMemcpyHostToDevice));
  } else if (fmt == 1) {
    std::vector<float> g(v.begin(), v.end());
    CK(cudaMemcpy(dst.p, g.data(), n * 4, cudaMemcpyHostToDevice));
  } else {
    std::vector<float> g(2 * n);
    for (size_t k = 0; k < n; ++k) {
      const float hi = (float)v[k];
      g[2 * k] = hi;
      g[2 * k + 1] = (float)(v[k] - (double)hi);
    }
    CK(cudaMemcpy(dst.p, g.data(), n * 8, cudaMemcpyHostToDevice));
  }
  return AW_OK;
}

// twiddle table tw[m] = exp(-2 pi i m / n), built in extended precision
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
static int make_twist(DevBuf& hi, DevBuf& lo, int* lo_n, int n, int fmt) {
  const int LO = n < 32 ? n : 32;
  const int nhi = n / LO;
  const long double PI = 3.141592653589793238462643383279502884L;
  std::vector<double> H(2 * (size_t)n * nhi), L(2 * (size_t)n * LO);
  for (long long ln = 0; ln < n; ++ln) {
    for (int h = 0; h < nhi; ++h) {
      const long long m = (ln * (long long)(h * LO)) % n;
      const long double a = 2.0L * PI * (long double)m / (long double)n;
      H[2 * ((size_t)ln * nhi + h)] = (double)(cosl(a) / n);
      H[2 * ((size_t)ln * nhi + h) + 1] = (double)(sinl(a) / n);
    }
    for (int l = 0; l < LO; ++l) {
      const long long m = (ln * (long long)l) % n;
      const long double a = 2.0L * PI * (long double)m / (long double)n;
      L[2 * ((size_t)ln * LO + l)] = (double)cosl(a);
      L[2 * ((size_t)ln * LO + l) + 1] = (double)sinl(a);
    }
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
static AwPassArgs pnone(const aw_state_s* h) {
  AwPassArgs a;
  memset(&a, 0, sizeof a);
  a.f0 = a.f1 = a.f2 = a.f3 = a.fbr = fnone();
  a.nrows = h->nr;
  a.ncols = h->nc;
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

static int df_prepare(aw_state_s* h, AwPassArgs& a) {
  const long long n = (long long)a.nrows * a.ncols;
  if (a.in && !df_is_live(h, a.in)) {
    void* dst = a.out ? a.out : (void*)a.in;
    KL(aw_k_convert(a.in, 0, dst, 2, n, h->st));
    a.in = dst;
    df_mark(h, dst, n);
  }
  return AW_OK;
}
static void df_outputs(aw_state_s* h, const AwPassArgs& a) {
  const long long n = (long long)a.nrows * a.ncols;
  df_mark(h, a.out, n);
  df_mark(h, a.mid_out, n);
  df_mark(h, a.br_out, n);
}

static int launch_pass(aw_state_s* h, AwPassArgs& a, const DevBuf& tw, bool row) {
  a.tw = tw.p;
  if (h->df) TRY(df_prepare(h, a));
  cudaEvent_t pe = prof_mark(h);
  int r;
  if (h->df)
    r = row ? aw_launch_row_pass_df(&a, 1, h->st) : aw_launch_col_pass_df(&a, 1, h->st);
  else if (h->f32)
    r = row ? aw_launch_row_pass_f32(&a, 1, h->st) : aw_launch_col_pass_f32(&a, 1, h->st);
  else
    r = row ? aw_launch_row_pass_f64(&a, 1, h->st) : aw_launch_col_pass_f64(&a, 1, h->st);
  prof_done(h, row ? PROF_ROW : PROF_COL, pass_bytes(h, a), pe);
  ++g_launches;
  if (r)
    return fail(AW_E_CUDA, "%s pass launch failed (%d, %s), grid %d x %d", row ? "row" : "column", r,
                cudaGetErrorString(cudaGetLastError()), a.nrows, a.ncols);
  if (h->df) df_outputs(h, a);
  return AW_OK;
}
static int row_pass(aw_state_s* h, AwPassArgs& a, const DevBuf& tw) { return launch_pass(h, a, tw, true); }
static int col_pass(aw_state_s* h, AwPassArgs& a, const DevBuf& tw) { return launch_pass(h, a, tw, false); }

// phase table slots
enum { TAB_V1 = 0, TAB_V1B, TAB_V2, TAB_K, TAB_BV, TAB_BK, TAB_BLK, TAB_NSLOT };
static void* tab_col(aw_state_s* h, int slot) { return (char*)h->tabs.p + (size_t)slot * (h->nc + h->nr) * h->esz; }
static void* tab_row(aw_state_s* h, int slot) { return (char*)tab_col(h, slot) + (size_t)h->nc * h->esz; }

// build one table slot: fn 0 = V, 1 = K.  With tlist (device times, count of them), builds count
// tables of times tlist[s] + ta at col/row + s * (nc + nr) elements instead.
static int build_tab(aw_state_s* h, int slot, int fn, int mode, double ta, double tb, double ca, double cb,
                     double shift, int maskpow, double tmask, void* col_base = nullptr, const double* tlist = nullptr,
                     int count = 1) {
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
  void* col = col_base ? col_base : tab_col(h, slot);
  void* row = (char*)col + (size_t)h->nc * h->esz;
  int f32 = tab_fmt(h);
  long long tstride = (long long)h->nc + h->nr;
  void* args[] = {&col, &row, &f32, &fn, &mode, &ncol, &dcol, &roll, &nrow, &drow,
                  &ta, &tb, &ca, &cb, &shift, &maskpow, &tmask, &tlist, &tstride};
  const int n = ncol + nrow;
  return hjit(h, h->k_tab, dim3((n + 31) / 32, count), dim3(32), args);
}

static int build_mask2d(aw_state_s* h, int which, double t) {
  DevBuf& m = which == 0 ? h->maskx : h->maskp;
  void* out = m.p;
  int f32 = tab_fmt(h), nr = h->nr, nc = h->nc;
  double a = h->cfg.dXX, b = h->cfg.dXX_prime, c = h->cfg.dPP, d = h->cfg.dPP_prime;
  void* args[] = {&out, &f32, &which, &t, &nr, &nc, &a, &b, &c, &d};
  return hjit(h, h->k_mask2d, dim3((nc + 127) / 128, nr), dim3(128), args);
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

static double* dscal(aw_state_s* h, int k) { return (double*)h->scal.p + k; }

// ============================================================================ creation
// error message setter for the other translation units of the library (C++ linkage, not exported API)
void aw_internal_set_error(const char* msg) { g_err = msg ? msg : ""; }

extern "C" int32_t aw_version(void) { return AW_VERSION; }
extern "C" const char* aw_last_error(void) { return g_err.c_str(); }
extern "C" int64_t aw_launch_count(void) { return g_launches.load(); }

static std::string cstr(const char* s, const char* dflt) { return s ? std::string(s) : std::string(dflt); }

static int create_impl(const aw_config* cfg, aw_state_s* h) {
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
    h->sw_rows = aw_row_pass_lines(N, h->f32);
    if (h->sw_rows <= 0) return fail(AW_E_ARG, "unsupported wave-function length %d", N);
  }
  const int maxn = h->kn.sw ? 8192 : 8192;
  if (h->nc < 32 || h->nc > maxn || (!h->kn.sw && (h->nr < 32 || h->nr > maxn)) || (h->wn && h->wn > 8192))
    return fail(AW_E_ARG, "grid sides must be powers of two in [32, %d] (Wigner grid up to 8192)", maxn);

  CK(cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking));
  if (h->kn.rotated) {
    CK(cudaStreamCreateWithFlags(&h->st2, cudaStreamNonBlocking));
    for (int k = 0; k < 2; ++k) {
      CK(cudaEventCreateWithFlags(&h->ev_z[k], cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&h->ev_f[k], cudaEventDisableTiming));
    }
  }

  // user module
  std::string src = awjit::module_source(h->kn, h->consts, h->V, h->K, h->absx, h->absp, h->obs_x, h->obs_p);
  TRY(jit_compile(src, &h->lib));
  TRY(jit_kernel(h->lib, "aw_tab", &h->k_tab));
  TRY(jit_kernel(h->lib, "aw_values", &h->k_values));
  TRY(jit_kernel(h->lib, "aw_finalize", &h->k_final));
  if (h->kn.rotated) {
    TRY(jit_kernel(h->lib, "aw_mask2d", &h->k_mask2d));
    TRY(jit_kernel(h->lib, "aw_finalize_rot", &h->k_final_rot));
  }

  // buffers
  const size_t grid = (size_t)(h->kn.sw ? h->sw_rows : h->nr) * h->nc;
  const size_t wgrid = h->kn.rotated ? grid : (size_t)h->wn * h->wn;
  TRY(dalloc(h->rho, grid * h->esz));
  TRY(dalloc(h->W, wgrid * h->esz));
  TRY(dalloc(h->tmp, std::max(grid, wgrid) * 16));
  CK(cudaMemset(h->rho.p, 0, grid * h->esz));
  CK(cudaMemset(h->W.p, 0, wgrid * h->esz));
  TRY(dalloc(h->tabs, (size_t)TAB_NSLOT * (h->nc + h->nr) * h->esz));
  TRY(dalloc(h->scal, 2048 * sizeof(double)));
  TRY(dalloc(h->stop, 16 * sizeof(int)));
  TRY(dalloc(h->part, 1024 * sizeof(double2)));
  CK(cudaMemset(h->scal.p, 0, 2048 * sizeof(double)));
  CK(cudaMemset(h->stop.p, 0, 16 * sizeof(int)));
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
    CK(cudaMemcpy(h->terms.p, ti.data(), ti.size() * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy((char*)h->terms.p + 64 * 3 * sizeof(int), tc.data(), tc.size() * 8, cudaMemcpyHostToDevice));
  }

  // twiddles
  TRY(make_twiddles(h->tw_r, h->nc, tab_fmt(h)));
  if (!h->kn.sw) TRY(make_twiddles(h->tw_c, h->nr, tab_fmt(h)));
  if (h->wn) TRY(make_twiddles(h->tw_w, h->wn, tab_fmt(h)));

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
  } else if (h->kn.vn) {
    // rho_vneumann_cuda_1d.py:608-639 on the padded (2N)^2 grid, dXX = dX
    const int M = h->wn;
    std::vector<double> ax(M), ay(M);
    for (int i = 0; i < M; ++i) ax[i] = -a_shx * cfg->dPP * (cfg->dX * ((double)i - 0.5 * M));
    for (int j = 0; j < M; ++j) ay[j] = -b_shy * cfg->dPP * (cfg->dX * ((double)j - 0.5 * M));
    TRY(make_shear(h->shx_hi, h->shx_lo, &h->shx_lo_n, ax, M, 1.0 / M, tab_fmt(h)));
    TRY(make_shear(h->shy_hi, h->shy_lo, &h->shy_lo_n, ay, M, 1.0 / M, tab_fmt(h)));
  } else {
    // schrodinger_wigner_cuda_1d.py:695-726: P is fft-shifted along the sheared axis
    const int M = h->wn;
    std::vector<double> ax(M), ay(M);
    for (int i = 0; i < M; ++i) ax[i] = -a_shx * cfg->dP * (cfg->dX * ((double)i - 0.5 * M));
    for (int j = 0; j < M; ++j) ay[j] = -b_shy * cfg->dP * (cfg->dX * ((double)j - 0.5 * M));
    TRY(make_shear(h->shx_hi, h->shx_lo, &h->shx_lo_n, ax, M, 1.0 / M, tab_fmt(h)));
    TRY(make_shear(h->shy_hi, h->shy_lo, &h->shy_lo_n, ay, M, 1.0 / M, tab_fmt(h)));
  }

  if (h->kn.vn) TRY(make_twist(h->twist_hi, h->twist_lo, &h->twist_lo_n, h->nc, tab_fmt(h)));

  // reduction scratch of the Wigner column pass
  const int wr = h->kn.rotated ? h->nr : h->wn, wc = h->kn.rotated ? h->nc : h->wn;
  h->red_blocks = aw_col_pass_blocks(wr, wc, h->f32);
  if (h->red_blocks <= 0) return fail(AW_E_ARG, "unsupported Wigner grid %d x %d", wr, wc);
  TRY(dalloc(h->red_line, (size_t)wc * 8));
  TRY(dalloc(h->red_cross, (size_t)h->red_blocks * wr * 8));
  TRY(dalloc(h->red_sq, (size_t)h->red_blocks * 8));
  TRY(dalloc(h->rowsum, (size_t)std::max(wr, wc) * 8));
  TRY(dalloc(h->diag, (size_t)std::max(h->nr, h->nc) * 16));
  TRY(dalloc(h->abs2, 2 * (size_t)std::max(h->nr, 1) * 8));  // two parities, see rot_run
  if (h->kn.rotated) {
    // the marginal column pass: narrow slabs spread over every SM, row partials summed across
    // clusters of 8 blocks in distributed shared memory, so that z_blocks stays small
    h->z_lines = std::min(2, aw_col_pass_max_lines(h->nr, h->nc, h->f32));
    const size_t z_smem = (size_t)h->nr * h->z_lines * h->esz + (size_t)h->nr * 16;
    h->z_cluster = (h->nc / h->z_lines) % 8 == 0 && h->nr % 8 == 0 && z_smem <= 160 * 1024 ? 8 : 1;
    h->z_blocks = h->nc / h->z_lines / h->z_cluster;
    // two parities, so that step n's reduction can run while step n + 1 writes the other
    TRY(dalloc(h->zbuf, 2 * (size_t)(h->nc + h->nr) * 16));
    TRY(dalloc(h->altbuf, 2 * (size_t)h->z_blocks * h->nr * 16));
  }

  // 2-D absorbing masks of the rotated frame
  if (h->kn.rotated) {
    if (cfg->absx_mode) TRY(dalloc(h->maskx, grid * (h->f32 ? 4 : 8)));
    if (cfg->absp_mode) TRY(dalloc(h->maskp, grid * (h->f32 ? 4 : 8)));
  }

  // Bloch minima: min over (V(x) + V(x')) = min V(x) + min V(x') since rounding is monotone
  if (h->kind == AW_WIGNER_BLOCH || h->kind == AW_RHO_BLOCH) {
    double vm = 0.0, km = 0.0;
    const int nmax = std::max(h->nr, h->nc);
    TRY(dalloc(h->stage, (size_t)4 * nmax * 8));
    double* d = (double*)h->stage.p;
    auto eval = [&](int fn, int n, double dx, double* out) -> int {
      void* o = out;
      double tt = cfg->t_initial;
      void* args[] = {&o, &fn, &n, &dx, &tt};
      return hjit(h, h->k_values, dim3((n + 255) / 256), dim3(256), args);
    };
    std::vector<double> a(nmax), b(nmax);
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
    for (int i = 0; i < h->nr; ++i) v2 = std::min(v2, hv[nmax + i]);
    for (int j = 0; j < h->nc; ++j) { k1 = std::min(k1, hv[2 * nmax + j]); knan |= !std::isfinite(hv[2 * nmax + j]); }
    for (int i = 0; i < h->nr; ++i) { k2 = std::min(k2, hv[3 * nmax + i]); knan |= !std::isfinite(hv[3 * nmax + i]); }
    vm = v1 + v2;
    km = k1 + k2;
    if (h->kind == AW_RHO_BLOCH) km = knan ? NAN : 0.0;  // fill_K multiplies a zeroed array (rho_bloch_cuda_1d.py:370)
    h->V_min = define_round(vm);
    h->K_min = define_round(km);
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

extern "C" int aw_destroy(aw_handle h) {
  if (!h) return AW_OK;
  if (h->st) cudaStreamSynchronize(h->st);
  DevBuf* bufs[] = {&h->vseq, &h->vtimes, &h->zbuf, &h->altbuf, &h->twist_hi, &h->twist_lo, &h->rho, &h->W, &h->snap, &h->tmp, &h->stage, &h->tw_r, &h->tw_c, &h->tw_w, &h->shx_hi,
                    &h->shx_lo, &h->shy_hi, &h->shy_lo, &h->tabs, &h->maskx, &h->maskp, &h->red_line,
                    &h->red_cross, &h->red_sq, &h->rowsum, &h->diag, &h->abs2, &h->scal, &h->stop, &h->hist,
                    &h->terms, &h->part, &h->blk_tabs};
  for (DevBuf* b : bufs) dfree(*b);
  for (DevBuf& b : h->sw_states) dfree(b);
  if (h->st) cudaStreamDestroy(h->st);
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

extern "C" int aw_sync(aw_handle h) {
  if (!h) return fail(AW_E_ARG, "null handle");
  CK(cudaStreamSynchronize(h->st));
  return AW_OK;
}

extern "C" int aw_bloch_min(aw_handle h, double* v_min, double* k_min) {
  if (!h) return fail(AW_E_ARG, "null handle");
  if (v_min) *v_min = h->V_min;
  if (k_min) *k_min = h->K_min;
  return AW_OK;
}

// ============================================================================ buffers
static DevBuf* buf_of(aw_state_s* h, int which, long long* rows, long long* cols) {
  switch (which) {
    case AW_BUF_RHO:
    case AW_BUF_PSI:
      if ((which == AW_BUF_PSI) != h->kn.sw) return nullptr;
      *rows = h->nr;
      *cols = h->nc;
      return &h->rho;
    case AW_BUF_WIGNER:
      *rows = h->kn.rotated ? h->nr : h->wn;
      *cols = h->kn.rotated ? h->nc : h->wn;
      return &h->W;
    case AW_BUF_SNAPSHOT:
      *rows = h->nr;
      *cols = h->nc;
      return &h->snap;
    default:
      return nullptr;
  }
}

extern "C" int aw_buffer(aw_handle h, int32_t which, void** dptr, int64_t* rows, int64_t* cols, int32_t* elem_bytes) {
  if (!h) return fail(AW_E_ARG, "null handle");
  long long r, c;
  DevBuf* b = buf_of(h, which, &r, &c);
  if (!b) return fail(AW_E_ARG, "no buffer %d for this propagator", which);
  if (dptr) *dptr = b->p;
  if (rows) *rows = r;
  if (cols) *cols = c;
  if (elem_bytes) *elem_bytes = h->esz;
  return AW_OK;
}

extern "C" int aw_set_buffer(aw_handle h, int32_t which, const void* src, int32_t src_on_device) {
  if (!h || !src) return fail(AW_E_ARG, "null argument");
  long long r, c;
  DevBuf* b = buf_of(h, which, &r, &c);
  if (!b) return fail(AW_E_ARG, "no buffer %d for this propagator", which);
  if (which == AW_BUF_SNAPSHOT) TRY(dalloc(h->snap, (size_t)r * c * h->esz));
  const size_t n = (size_t)r * c;
  if (!h->f32) {
    CK(cudaMemcpyAsync(b->p, src, n * 16, src_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, h->st));
  } else {
    CK(cudaMemcpyAsync(h->tmp.p, src, n * 16, src_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, h->st));
    KL(aw_k_convert(h->tmp.p, 0, b->p, 1, (long long)n, h->st));
  }
  CK(cudaStreamSynchronize(h->st));
  return AW_OK;
}

extern "C" int aw_get_buffer(aw_handle h, int32_t which, void* dst, int32_t dst_on_device) {
  if (!h || !dst) return fail(AW_E_ARG, "null argument");
  long long r, c;
  DevBuf* b = buf_of(h, which, &r, &c);
  if (!b || !b->p) return fail(AW_E_ARG, "no buffer %d for this propagator", which);
  const size_t n = (size_t)r * c;
  const void* from = b->p;
  if (h->f32) {
    KL(aw_k_convert(b->p, 1, h->tmp.p, 0, (long long)n, h->st));
    from = h->tmp.p;
  }
  CK(cudaMemcpyAsync(dst, from, n * 16, dst_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  return AW_OK;
}

extern "C" int aw_copy_buffer(aw_handle h, int32_t from, int32_t to) {
  if (!h) return fail(AW_E_ARG, "null handle");
  long long r1, c1, r2, c2;
  DevBuf* a = buf_of(h, from, &r1, &c1);
  DevBuf* b = buf_of(h, to, &r2, &c2);
  if (!a || !b || r1 * c1 != r2 * c2) return fail(AW_E_ARG, "incompatible buffers %d -> %d", from, to);
  if (to == AW_BUF_SNAPSHOT) TRY(dalloc(h->snap, (size_t)r2 * c2 * h->esz));
  if (!a->p) return fail(AW_E_STATE, "buffer %d is empty", from);
  CK(cudaMemcpyAsync(b->p, a->p, (size_t)r1 * c1 * h->esz, cudaMemcpyDeviceToDevice, h->st));
  return AW_OK;
}

extern "C" int aw_fill_const(aw_handle h, int32_t which, double re, double im) {
  if (!h) return fail(AW_E_ARG, "null handle");
  long long r, c;
  DevBuf* b = buf_of(h, which, &r, &c);
  if (!b) return fail(AW_E_ARG, "no buffer %d", which);
  KL(aw_k_fill(b->p, h->f32, r * c, re, im, h->st));
  return AW_OK;
}

extern "C" int aw_fill_expr(aw_handle h, int32_t which, const char* expr) {
  if (!h || !expr) return fail(AW_E_ARG, "null argument");
  long long r, c;
  DevBuf* b = buf_of(h, which, &r, &c);
  if (!b) return fail(AW_E_ARG, "no buffer %d", which);
  cudaLibrary_t lib;
  TRY(jit_compile(awjit::init_source(h->kn, h->consts, expr), &lib));
  cudaKernel_t k;
  TRY(jit_kernel(lib, "aw_init", &k));
  void* out = b->p;
  int f32 = h->f32, nr = (int)r, nc = (int)c;
  double dX = h->cfg.dX, dP = h->cfg.dP;
  void* args[] = {&out, &f32, &nr, &nc, &dX, &dP};
  TRY(hjit(h, k, dim3((nc + 127) / 128, h->kn.sw ? 1 : nr), dim3(128), args));
  return AW_OK;
}

extern "C" int aw_sum(aw_handle h, int32_t which, double* re, double* im) {
  if (!h) return fail(AW_E_ARG, "null handle");
  long long r, c;
  DevBuf* b = buf_of(h, which, &r, &c);
  if (!b) return fail(AW_E_ARG, "no buffer %d", which);
  double s[2];
  TRY(dsum(h, b->p, r * c, 0, 0, s));
  if (re) *re = s[0];
  if (im) *im = s[1];
  return AW_OK;
}

extern "C" int aw_trace(aw_handle h, double* re, double* im) {
  if (!h) return fail(AW_E_ARG, "null handle");
  if (h->nr != h->nc) return fail(AW_E_STATE, "trace of a non-square grid");
  double s[2];
  TRY(dsum(h, h->rho.p, h->nr, 3, h->nc + 1, s));
  if (re) *re = s[0];
  if (im) *im = s[1];
  return AW_OK;
}

extern "C" int aw_scale(aw_handle h, int32_t which, double re, double im) {
  if (!h) return fail(AW_E_ARG, "null handle");
  long long r, c;
  DevBuf* b = buf_of(h, which, &r, &c);
  if (!b) return fail(AW_E_ARG, "no buffer %d", which);
  KL(aw_k_scale(b->p, h->f32, r * c, re, im, nullptr, h->st));
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
  f.active = 1;
  return f;
}
static AwFactor fshear_y(aw_state_s* h) {
  AwFactor f = fnone();
  f.sh_hi = h->shy_hi.p;
  f.sh_lo = h->shy_lo.p;
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

static int launch_finalize_args(aw_state_s* h, const FinalArgs& f, double t, double* hist_row, int stop_on_purity) {
  const double* colsum = f.colsum;
  const double* rowpart = f.rowpart;
  int nparts = f.nparts;
  const double* sqpart = f.sqpart;
  double* rowsum = (double*)h->rowsum.p;
  double* inv = f.inv;
  int* stop = (int*)h->stop.p;
  int ncol = f.ncol, nrow = f.nrow;
  double dX = h->cfg.dX, dP = h->cfg.dP, dXdP = f.dXdP;
  const int* ts = (const int*)h->terms.p;
  const int* tk = ts + 64;
  const int* ti = ts + 128;
  const double* tc = (const double*)((const char*)h->terms.p + 64 * 3 * sizeof(int));
  int nterms = (int)h->tslot.size(), nslots = h->cfg.n_slots;
  int cstride = f.cstride, proll = f.proll, pown = f.pnorm_own, sq = f.sqrt_norm;
  void* args[] = {&colsum, &rowpart, &nparts, &sqpart, &rowsum, &hist_row, &inv, &stop, &stop_on_purity, &t,
                  &ncol, &nrow, &dX, &dP, &dXdP, &ts, &tk, &ti, &tc, &nterms, &nslots, &cstride, &proll, &pown, &sq};
  return hjit(h, h->k_final, dim3(1), dim3(256), args);
}

// rotated frame: marginals of W from the reducing column pass
static int launch_finalize(aw_state_s* h, double t, double* hist_row, int stop_on_purity) {
  FinalArgs f{(const double*)h->red_line.p, 1, h->nc, (const double*)h->red_cross.p, h->red_blocks, h->nr, 0,
              (const double*)h->red_sq.p, h->cfg.dXdP, dscal(h, 0), 0, 0};
  return launch_finalize_args(h, f, t, hist_row, stop_on_purity);
}

// marginal buffers of parity par (zbuf, altbuf, abs2 hold two sets)
static double2* zbuf_of(aw_state_s* h, int par) { return (double2*)h->zbuf.p + (size_t)par * (h->nc + h->nr); }
static double2* altbuf_of(aw_state_s* h, int par) { return (double2*)h->altbuf.p + (size_t)par * h->z_blocks * h->nr; }
static double* abs2_of(aw_state_s* h, int par) { return (double*)h->abs2.p + (size_t)par * std::max(h->nr, 1); }

static int launch_finalize_rot(aw_state_s* h, double t, double* hist_row, int stop_on_purity, int par = 0,
                               cudaStream_t st = nullptr) {
  const double2* z = zbuf_of(h, par);
  const double2* wpart = altbuf_of(h, par);
  int nparts = h->z_blocks;
  const double* abs2 = abs2_of(h, par);
  int nb2 = aw_row_pass_blocks(h->nr, h->nc, h->f32);
  double* tv = dscal(h, 16);
  unsigned int* counter = (unsigned int*)h->stop.p + 1;
  double* inv = dscal(h, 0);
  int* stop = (int*)h->stop.p;
  int ncol = h->nc, nrow = h->nr;
  double dX = h->cfg.dX, dP = h->cfg.dP, dXdP = h->cfg.dXdP;
  const int* ts = (const int*)h->terms.p;
  const int* tk = ts + 64;
  const int* ti = ts + 128;
  const double* tc = (const double*)((const char*)h->terms.p + 64 * 3 * sizeof(int));
  int nterms = (int)h->tslot.size(), nslots = h->cfg.n_slots;
  // chunks per term: enough blocks to spread the FP64 expression work over the SMs
  int nchunk = 16;
  while (nchunk > 1 && ((std::min(ncol, nrow) % nchunk) || (nterms + 2) * nchunk > 1024)) nchunk >>= 1;
  void* args[] = {&z, &wpart, &nparts, &abs2, &nb2, &tv, &counter, &hist_row, &inv, &stop, &stop_on_purity, &t,
                  &ncol, &nrow, &dX, &dP, &dXdP, &ts, &tk, &ti, &tc, &nterms, &nslots, &nchunk};
  return hjit_on(h, h->k_final_rot, dim3((nterms + 2) * nchunk), dim3(128), args, st ? st : h->st);
}

static int ensure_hist(aw_state_s* h, long long rows) {
  h->hist_cols = h->cfg.n_slots + 2;
  const size_t need = (size_t)std::max(rows, 1LL) * h->hist_cols * 8;
  if (h->hist.bytes < need) TRY(dalloc(h->hist, need));
  h->hist_rows = 0;
  h->hist_cap = rows;
  return AW_OK;
}

// normalize_rho_wigner (wigner_moyal_cuda_1d.py:608-622): W = rho2wigner(rho); norm; W, rho /= norm
static int wm_normalize(aw_state_s* h, double* hist_row) {
  WignerGrid g{h->W.p, h->nr, h->nc, &h->tw_r, &h->tw_c};
  TRY(wigner_passes(h, g, h->rho.p, fsign(), false, true, true));
  TRY(launch_finalize(h, 0.0, hist_row, 0));
  TRY(settle(h));
  KL(aw_k_scale(h->W.p, h->f32, (long long)h->nr * h->nc, 1.0, 0.0, dscal(h, 0), h->st));
  KL(aw_k_scale(h->rho.p, h->f32, (long long)h->nr * h->nc, 1.0, 0.0, dscal(h, 0), h->st));
  return AW_OK;
}

extern "C" int aw_wigner2rho(aw_handle h) {
  if (!h) return fail(AW_E_ARG, "null handle");
  Settled guard{h};
  if (!h->kn.rotated) return fail(AW_E_STATE, "wigner2rho exists for the Wigner-Moyal / Wigner-Bloch propagators");
  return wm_wigner2rho(h);
}

extern "C" int aw_normalize_rho_wigner(aw_handle h) {
  if (!h) return fail(AW_E_ARG, "null handle");
  Settled guard{h};
  if (!h->kn.rotated) return fail(AW_E_STATE, "normalize_rho_wigner exists for the Wigner-Moyal propagators");
  TRY(ensure_hist(h, 1));
  return wm_normalize(h, (double*)h->hist.p);
}

static int vn_get_wigner(aw_state_s* h, int blackman);
static int sw_get_wigner(aw_state_s* h, int blackman);

extern "C" int aw_rho2wigner(aw_handle h, int32_t blackman) {
  if (!h) return fail(AW_E_ARG, "null handle");
  Settled guard{h};
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
};

static AwFactor ftab(aw_state_s* h, int slot) {
  AwFactor f = fnone();
  f.col_tab = tab_col(h, slot);
  f.row_tab = tab_row(h, slot);
  f.active = 1;
  return f;
}

static int rot_tables_V(aw_state_s* h, const StepPlan& p, double tn, double tn1, bool pair) {
  const aw_config& c = h->cfg;
  if (p.bloch) {
    // bloch_expV: exp(-dbeta/4 (V(XX) + V(XX') - V_min)), split evenly over the two factors
    return build_tab(h, TAB_BV, 0, 1, c.t_initial, 0.0, -0.25 * p.dbeta, 0.0, 0.5 * h->V_min, 0, 0.0);
  }
  const double half = 0.5 * c.dt;
  TRY(build_tab(h, TAB_V1, 0, 0, tn + half, 0.0, -half, 0.0, 0.0, 0, 0.0));
  if (pair) TRY(build_tab(h, TAB_V1B, 0, 0, tn1 + half, 0.0, -half, 0.0, 0.0, 0, 0.0));
  return AW_OK;
}

static int rot_tables_K(aw_state_s* h, const StepPlan& p, double tn) {
  const aw_config& c = h->cfg;
  if (p.bloch)
    return build_tab(h, TAB_BK, 1, 1, c.t_initial, 0.0, -0.5 * p.dbeta, 0.0, 0.5 * h->K_min, 0, 0.0);
  return build_tab(h, TAB_K, 1, 0, tn + 0.5 * c.dt, 0.0, -c.dt, 0.0, 0.0, 0, 0.0);
}

// V-kick factor; `mask_t` >= 0 evaluates a time-dependent mask at that time
static int vkick(aw_state_s* h, const StepPlan& p, int slot, bool sign, double t_mask, AwFactor* f) {
  *f = ftab(h, p.bloch ? TAB_BV : slot);
  f->sign = sign;
  if (!p.bloch && h->cfg.absx_mode) {
    if (h->cfg.absx_mode == 2 || !h->maskx_ready) {
      TRY(build_mask2d(h, 0, t_mask));
      h->maskx_ready = true;
    }
    f->mask = h->maskx.p;
    f->mask_pow = 1;
  }
  return AW_OK;
}

// Run `steps` steps of the rotated-frame propagator on rho.
//   times[n] (n = 1..steps) are the reference's self.t values after the increment.
//   rows of observables go to hist (one per step) when p.ehrenfest.
static int rot_run(aw_state_s* h, const StepPlan& p, long long steps, const std::vector<double>& times, double* hist) {
  const aw_config& c = h->cfg;
  if (!p.bloch && (c.absx_mode == 2 || c.absp_mode == 2))
    return fail(AW_E_ARG, "time-dependent abs_boundary_x / abs_boundary_p are not supported by the rotated-frame passes");
  const bool vdep = !p.bloch && (c.v_time_dependent || c.absx_mode == 2);
  const bool kdep = !p.bloch && (c.k_time_dependent || c.absp_mode == 2);
  const long long grid = (long long)h->nr * h->nc;
  const double inv_n2 = p.bloch ? 1.0 : 1.0 / (double)grid;  // WM divides by N^2 (wm:557); Bloch does not
  // Real-time propagation is linear and every recorded observable is a ratio to the norm of the
  // same step (sum f W / sum W, purity sum W^2 / (sum W)^2), so the per-step normalisation of
  // normalize_rho_wigner (wm:608-622) is deferred to the end of the call: the step loop does not
  // wait for the reduction, which runs on a side stream.  Bloch steps normalise every step.
  const bool defer = !p.bloch && p.ehrenfest && h->st2;
  // scale applied in the column pass: 1/N^2 and, for Bloch steps, 1/norm of the previous step
  KL(aw_k_set2(dscal(h, 0), 1.0, 0.0, h->st));
  CK(cudaMemsetAsync(h->stop.p, 0, sizeof(int), h->st));  // a stop raised by an earlier call must not persist
  const int* stop = p.stop_on_purity ? (const int*)h->stop.p : nullptr;

  if (!vdep) TRY(rot_tables_V(h, p, times[1], times[1], false));
  if (!kdep) TRY(rot_tables_K(h, p, times[1]));
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
    TRY(vkick(h, p, TAB_V1, sign, times[n], f));
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
  for (long long n = 1; n <= steps; ++n) {
    const bool last = n == steps;
    const int par = defer ? (int)(n & 1) : 0;
    // the reduction of step n - 2 read this parity's buffers
    if (defer && n >= 3) CK(cudaStreamWaitEvent(h->st, h->ev_f[par], 0));
    // column pass: scale, ifft0, K-kick, fft0
    {
      if (kdep) TRY(rot_tables_K(h, p, times[n]));
      AwPassArgs a = pnone(h);
      a.in = a.out = h->rho.p;
      a.f0 = fnone();
      a.f0.scale = inv_n2;
      a.f0.scale_ptr = p.ehrenfest && !defer ? dscal(h, 0) : nullptr;
      a.f0.active = 1;
      a.d1 = -1;
      a.f1 = ftab(h, p.bloch ? TAB_BK : TAB_K);
      if (!p.bloch && c.absp_mode) {
        if (c.absp_mode == 2 || !h->maskp_ready) {
          TRY(build_mask2d(h, 1, times[n]));
          h->maskp_ready = true;
        }
        a.f1.mask = h->maskp.p;
        a.f1.mask_pow = 1;
      }
      a.d2 = +1;
      a.stop = stop;
      TRY(col_pass(h, a, h->tw_c));
    }
    // row pass: ifft1, V-kick(t_n) [branch: Wigner transform] [next kick(t_{n+1}), fft1 | S]
    {
      AwPassArgs a = pnone(h);
      a.in = a.out = h->rho.p;
      a.d1 = -1;
      TRY(vfactor(n, false, &a.f1));
      if (p.ehrenfest) {
        a.br_out = h->W.p;
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
      a.in = h->W.p;
      a.d1 = +1;
      a.f1 = fshear_y(h);
      a.col_alt = zbuf_of(h, par);
      a.alt_cross = altbuf_of(h, par);
      a.lines_hint = h->z_lines;
      a.cluster = h->z_cluster;
      a.stop = stop;
      TRY(col_pass(h, a, h->tw_c));
      double* hrow = hist + (size_t)(n - 1) * h->hist_cols;
      if (defer) {
        CK(cudaEventRecord(h->ev_z[par], h->st));
        CK(cudaStreamWaitEvent(h->st2, h->ev_z[par], 0));
        TRY(launch_finalize_rot(h, times[n], hrow, 0, par, h->st2));
        CK(cudaEventRecord(h->ev_f[par], h->st2));
      } else {
        TRY(launch_finalize_rot(h, times[n], hrow, p.stop_on_purity));
      }
      if (last) {
        WignerGrid g{h->W.p, h->nr, h->nc, &h->tw_r, &h->tw_c};
        TRY(wigner_passes(h, g, h->W.p, fnone(), false, false, true, true));
      }
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
    if (!c.ehrenfest) TRY(wm_normalize(h, (double*)h->hist.p));
    return AW_OK;
  }
  StepPlan p{false, 0.0, c.ehrenfest != 0, false, 0};
  TRY(rot_run(h, p, steps, times, (double*)h->hist.p));
  if (c.ehrenfest) {
    // the last step's normalisation, applied to both arrays
    TRY(settle(h));
    KL(aw_k_scale(h->W.p, h->f32, (long long)h->nr * h->nc, 1.0, 0.0, dscal(h, 0), h->st));
    KL(aw_k_scale(h->rho.p, h->f32, (long long)h->nr * h->nc, 1.0, 0.0, dscal(h, 0), h->st));
    h->hist_rows = steps;
  } else {
    TRY(wm_normalize(h, (double*)h->hist.p + (size_t)steps * h->hist_cols));
    h->hist_rows = 0;
  }
  *t = times[steps];
  return AW_OK;
}

extern "C" int aw_history(aw_handle h, double* out, int64_t max_rows, int64_t* rows, int32_t* cols) {
  if (!h) return fail(AW_E_ARG, "null handle");
  const long long n = std::min<long long>(h->hist_rows, max_rows);
  if (rows) *rows = h->hist_rows;
  if (cols) *cols = h->hist_cols;
  if (out && n > 0) {
    CK(cudaMemcpyAsync(out, h->hist.p, (size_t)n * h->hist_cols * 8, cudaMemcpyDeviceToHost, h->st));
  }
  CK(cudaStreamSynchronize(h->st));
  return AW_OK;
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
  const void* src = h->kn.rotated ? h->W.p : h->rho.p;
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
    TRY(dsum(h, h->W.p, (long long)h->nr * h->nc, 1, 0, s));
    *out = 2.0 * M_PI * s[0] * h->cfg.dXdP;
  } else if (h->kn.vn) {
    TRY(dsum(h, h->rho.p, (long long)h->nr * h->nc, 2, 0, s));
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
  std::vector<double> times(3, 0.0);
  TRY(rot_run(h, p, 1, times, (double*)h->hist.p));
  TRY(settle(h));
  KL(aw_k_scale(h->W.p, h->f32, (long long)h->nr * h->nc, 1.0, 0.0, dscal(h, 0), h->st));
  KL(aw_k_scale(h->rho.p, h->f32, (long long)h->nr * h->nc, 1.0, 0.0, dscal(h, 0), h->st));
  if (out) {
    CK(cudaMemcpyAsync(out, h->hist.p, (size_t)h->hist_cols * 8, cudaMemcpyDeviceToHost, h->st));
  }
  CK(cudaStreamSynchronize(h->st));
  return AW_OK;
}

extern "C" int aw_gibbs(aw_handle h, double dbeta, int64_t steps, int64_t* done, double* purity) {
  if (!h) return fail(AW_E_ARG, "null handle");
  Settled guard{h};
  int vn_gibbs(aw_state_s*, double, long long, long long*, double*);
  if (h->kind == AW_RHO_BLOCH) {
    long long d = 0;
    TRY(vn_gibbs(h, dbeta, steps, &d, purity));
    if (done) *done = d;
    return AW_OK;
  }
  if (h->kind != AW_WIGNER_BLOCH) return fail(AW_E_STATE, "get_gibbs_state needs a Bloch propagator");
  if (steps <= 0) {
    if (done) *done = 0;
    return AW_OK;
  }
  TRY(ensure_hist(h, steps + 1));
  CK(cudaMemsetAsync(h->hist.p, 0, (size_t)(steps + 1) * h->hist_cols * 8, h->st));
  TRY(dalloc(h->snap, (size_t)h->nr * h->nc * h->esz));
  StepPlan p{true, dbeta, true, true, 1};
  std::vector<double> times(steps + 2, 0.0);
  TRY(rot_run(h, p, steps, times, (double*)h->hist.p));
  // how many steps ran: rows with a non-zero norm
  std::vector<double> hh((size_t)steps * h->hist_cols);
  CK(cudaMemcpyAsync(hh.data(), h->hist.p, hh.size() * 8, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  long long ran = 0;
  const int cols = h->hist_cols;
  // rows are written in order until the stop flag is raised; the finalize of the stopping step still writes
  // (the flag is checked at entry), so count rows whose norm entry was written
  for (long long n = 0; n < steps; ++n) {
    if (hh[(size_t)n * cols + cols - 1] == 0.0) break;
    ran = n + 1;
  }
  if (done) *done = ran;
  if (purity && ran > 0) *purity = hh[(size_t)(ran - 1) * cols + cols - 2];
  // rho_n of the last executed step (position representation, unnormalised) and its W
  TRY(settle(h));
  CK(cudaMemcpyAsync(h->rho.p, h->snap.p, (size_t)h->nr * h->nc * h->esz, cudaMemcpyDeviceToDevice, h->st));
  {
    WignerGrid g{h->W.p, h->nr, h->nc, &h->tw_r, &h->tw_c};
    TRY(wigner_passes(h, g, h->rho.p, fsign(), false, false, true));
  }
  TRY(settle(h));
  KL(aw_k_scale(h->W.p, h->f32, (long long)h->nr * h->nc, 1.0, 0.0, dscal(h, 0), h->st));
  KL(aw_k_scale(h->rho.p, h->f32, (long long)h->nr * h->nc, 1.0, 0.0, dscal(h, 0), h->st));
  CK(cudaStreamSynchronize(h->st));
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
};

static int vn_tables(aw_state_s* h, const VnPlan& p, double tn, bool kfirst) {
  const aw_config& c = h->cfg;
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
// so that Tr[g(p) rho] dX = Sum_k g(P_k) M_k dX (the p branch of get_average, vn:548-561)
static int vn_run(aw_state_s* h, const VnPlan& p, long long steps, const std::vector<double>& times, double* hist,
                  int hist_stride) {
  const aw_config& c = h->cfg;
  const bool vdep = !p.bloch && c.v_time_dependent;
  const bool kdep = !p.bloch && c.k_time_dependent;
  const int N = h->nc;
  KL(aw_k_set2(dscal(h, 0), 1.0, 0.0, h->st));
  CK(cudaMemsetAsync(h->stop.p, 0, sizeof(int), h->st));  // a stop raised by an earlier call must not persist
  const int* stop = p.stop_on_purity ? (const int*)h->stop.p : nullptr;
  const int row_blocks = aw_row_pass_blocks(h->nr, h->nc, h->f32);
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
      AwPassArgs a = pnone(h);
      a.in = a.out = h->rho.p;
      a.f0 = fnone();
      a.f0.scale_ptr = dscal(h, 0);
      a.f0.active = 1;
      a.d1 = -1;
      a.f1 = ftab(h, kslot);
      a.d2 = +1;
      a.stop = stop;
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
      a.f1 = ftab(h, vslot);
      a.diag_out = (double2*)h->diag.p;
      if (p.stop_on_purity || p.bloch) a.red_abs2 = (double*)h->abs2.p;
      if (p.keep_rho) {
        a.mid_out = h->snap.p;
        a.mid_sign = 1;
      }
      if (p.observables) {
        a.br_out = h->tmp.p;
        a.br_d1 = +1;
        a.fbr = fnone();
        a.fbr.sh_hi = h->twist_hi.p;
        a.fbr.sh_lo = h->twist_lo.p;
        a.fbr.sh_lo_n = h->twist_lo_n;
        a.fbr.active = 1;
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
      // column sums of the twisted branch: Re M_k
      AwPassArgs a = pnone(h);
      a.in = h->tmp.p;
      a.red_line = (double*)h->red_line.p;
      a.stop = stop;
      TRY(col_pass(h, a, h->tw_c));
    }
    if (p.bloch || !p.observables) {
      KL(aw_k_trace_finalize((const double2*)h->diag.p, N, (const double*)h->abs2.p, row_blocks, c.dX,
                             p.complex_trace, dscal(h, 0), p.observables ? nullptr : hrow, (int*)h->stop.p,
                             p.stop_on_purity, h->st));
    }
    if (p.observables) {
      FinalArgs f{(const double*)h->diag.p, 2, N, (const double*)h->red_line.p, 1, N, 0, nullptr, c.dX,
                  p.bloch ? nullptr : dscal(h, 0), 0, 0};
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
  TRY(vn_run(h, p, steps, times, c.ehrenfest ? (double*)h->hist.p : nullptr, h->hist_cols));
  TRY(settle(h));
  KL(aw_k_scale(h->rho.p, h->f32, (long long)h->nr * h->nc, 1.0, 0.0, dscal(h, 0), h->st));
  h->hist_rows = c.ehrenfest ? steps : 0;
  *t = times[steps];
  return AW_OK;
}

int vn_bloch_step(aw_state_s* h, double dbeta, double* out) {
  TRY(ensure_hist(h, 2));
  CK(cudaMemsetAsync(h->hist.p, 0, 2 * (size_t)h->hist_cols * 8, h->st));
  const bool obs = h->cfg.n_slots > 0;
  VnPlan p{true, dbeta, obs, false, 0, 1};
  std::vector<double> times(3, 0.0);
  // observables go to row 0, the trace finalize (purity, trace) to row 1
  TRY(vn_run(h, p, 1, times, (double*)h->hist.p, h->hist_cols));
  if (obs)
    KL(aw_k_trace_finalize((const double2*)h->diag.p, h->nc, (const double*)h->abs2.p,
                           aw_row_pass_blocks(h->nr, h->nc, h->f32), h->cfg.dX, 1, dscal(h, 2),
                           (double*)h->hist.p + h->hist_cols, nullptr, 0, h->st));
  TRY(settle(h));
  KL(aw_k_scale(h->rho.p, h->f32, (long long)h->nr * h->nc, 1.0, 0.0, dscal(h, 0), h->st));
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

int vn_gibbs(aw_state_s* h, double dbeta, long long steps, long long* done, double* purity) {
  *done = 0;
  if (steps <= 0) return AW_OK;
  TRY(ensure_hist(h, steps + 1));
  const int hc = 3;
  TRY(dalloc(h->hist, (size_t)(steps + 1) * hc * 8));
  CK(cudaMemsetAsync(h->hist.p, 0, (size_t)(steps + 1) * hc * 8, h->st));
  TRY(dalloc(h->snap, (size_t)h->nr * h->nc * h->esz));
  VnPlan p{true, dbeta, false, true, 1, 1};
  std::vector<double> times(steps + 2, 0.0);
  TRY(vn_run(h, p, steps, times, (double*)h->hist.p, hc));
  std::vector<double> hh((size_t)steps * hc);
  CK(cudaMemcpyAsync(hh.data(), h->hist.p, hh.size() * 8, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  long long ran = 0;
  for (long long n = 0; n < steps; ++n) {
    if (hh[(size_t)n * hc + 1] == 0.0) break;
    ran = n + 1;
  }
  *done = ran;
  if (purity && ran > 0) *purity = hh[(size_t)(ran - 1) * hc];
  TRY(settle(h));
  CK(cudaMemcpyAsync(h->rho.p, h->snap.p, (size_t)h->nr * h->nc * h->esz, cudaMemcpyDeviceToDevice, h->st));
  KL(aw_k_scale(h->rho.p, h->f32, (long long)h->nr * h->nc, 1.0, 0.0, dscal(h, 0), h->st));
  CK(cudaStreamSynchronize(h->st));
  h->hist_rows = 0;
  return AW_OK;
}

// get_wignerfunction (rho_vneumann_cuda_1d.py:387-427): embed rho in the centre of a zeroed
// (2N)^2 grid, sign flip, three shears, ifft0, sign flip, normalise by Re Sum W dXdP_wigner
static int vn_get_wigner(aw_state_s* h, int blackman) {
  const int N = h->nc, M = h->wn, pad = N / 2;
  KL(aw_k_embed(h->rho.p, h->f32, N, h->W.p, M, pad, h->st));
  if (blackman) TRY(ensure_blackman(h, M, M));
  WignerGrid g{h->W.p, M, M, &h->tw_w, &h->tw_w};
  TRY(wigner_passes(h, g, h->W.p, fsign(), blackman != 0, false, true));
  TRY(settle(h));
  double s[2];
  TRY(dsum(h, h->W.p, (long long)M * M, 0, 0, s));
  KL(aw_k_scale(h->W.p, h->f32, (long long)M * M, 1.0 / (s[0] * h->cfg.dXdP), 0.0, nullptr, h->st));
  return AW_OK;
}

extern "C" int aw_average_ops(aw_handle h, const char* const* ops, int32_t n_ops, double t, double* out) {
  if (!h || !out) return fail(AW_E_ARG, "null argument");
  if (!h->kn.vn) return fail(AW_E_STATE, "ordered operator averages are defined for density matrices");
  Settled guard{h};
  const long long n = (long long)h->nr * h->nc;
  CK(cudaMemcpyAsync(h->tmp.p, h->rho.p, n * h->esz, cudaMemcpyDeviceToDevice, h->st));
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

static int sw_finalize(aw_state_s* h, double t, double* hrow) {
  const int N = h->nc;
  double* xm = (double*)h->red_line.p;    // |psi_j|^2
  double* pmar = (double*)h->red_cross.p; // |(fft psi)_k|^2
  KL(aw_k_abs2(h->W.p, h->f32, N, xm, h->st));
  KL(aw_k_abs2(h->tmp.p, h->f32, N, pmar, h->st));
  FinalArgs f{xm, 1, N, pmar, 1, N, N / 2, nullptr, h->cfg.dX, dscal(h, 0), 1, 1};
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
  KL(aw_k_set2(dscal(h, 0), 1.0, 0.0, h->st));
  if (!tdep) TRY(sw_tables(h, times[1]));
  const int nb = aw_row_pass_blocks(h->sw_rows, h->nc, h->f32);
  for (long long n = 1; n <= steps; ++n) {
    if (tdep) TRY(sw_tables(h, times[n]));
    AwPassArgs a = sw_args(h);
    a.in = h->rho.p;
    a.out = c.ehrenfest ? h->W.p : h->rho.p;
    a.f0 = ftab(h, TAB_V1);
    a.f0.row_tab = nullptr;
    a.f0.scale_ptr = dscal(h, 0);
    a.d1 = +1;
    a.f1 = ftab(h, TAB_K);
    a.f1.row_tab = nullptr;
    a.d2 = -1;
    a.f3 = ftab(h, TAB_V1);
    a.f3.row_tab = nullptr;
    if (!c.ehrenfest) {
      a.red_abs2 = (double*)h->abs2.p;
      a.abs2_end = 1;
    } else {
      // psi' -> W buffer; its momentum representation -> tmp
      a.br_out = nullptr;
    }
    TRY(row_pass(h, a, h->tw_r));
    if (c.ehrenfest) {
      AwPassArgs b = sw_args(h);
      b.in = h->W.p;
      b.out = h->tmp.p;
      b.d1 = +1;
      TRY(row_pass(h, b, h->tw_r));
      TRY(sw_finalize(h, times[n], (double*)h->hist.p + (size_t)(n - 1) * h->hist_cols));
      CK(cudaMemcpyAsync(h->rho.p, h->W.p, (size_t)h->sw_rows * h->nc * h->esz, cudaMemcpyDeviceToDevice, h->st));
    } else {
      KL(aw_k_norm_finalize((const double*)h->abs2.p, nb, c.dX, dscal(h, 0), nullptr, h->st));
    }
  }
  KL(aw_k_scale(h->rho.p, h->f32, h->nc, 1.0, 0.0, dscal(h, 0), h->st));
  h->hist_rows = c.ehrenfest ? steps : 0;
  *t = times[steps];
  return AW_OK;
}

// get_wigner / get_wigner_blackman (schrodinger_wigner_cuda_1d.py:593-663)
static int sw_get_wigner(aw_state_s* h, int blackman) {
  const int N = h->nc;
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
  const int nb = aw_row_pass_blocks(h->sw_rows, h->nc, h->f32);
  const int N = h->nc;
  for (long long n = 0; n < steps; ++n) {
    AwPassArgs a = sw_args(h);
    a.in = a.out = h->rho.p;
    a.f0 = ftab(h, TAB_BV);
    a.f0.row_tab = nullptr;
    a.d1 = +1;
    a.f1 = ftab(h, TAB_BK);
    a.f1.row_tab = nullptr;
    a.d2 = -1;
    a.f3 = ftab(h, TAB_BV);
    a.f3.row_tab = nullptr;
    if (!project) {
      a.red_abs2 = (double*)h->abs2.p;
      a.abs2_end = 1;
    }
    TRY(row_pass(h, a, h->tw_r));
    if (!project) {
      // psi /= norm(psi) sqrt(dX)
      KL(aw_k_norm_finalize((const double*)h->abs2.p, nb, c.dX, dscal(h, 0), nullptr, h->st));
      KL(aw_k_scale(h->rho.p, h->f32, N, 1.0, 0.0, dscal(h, 0), h->st));
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
  AwPassArgs a = sw_args(h);
  a.in = h->rho.p;
  a.out = h->tmp.p;
  a.d1 = +1;
  TRY(row_pass(h, a, h->tw_r));
  TRY(dsum(h, h->tmp.p, h->nc, 2, 0, n2));
  // average of K over the momentum representation held in tmp
  cudaKernel_t kern;
  TRY(get_obs_kernel(h, h->K.c_str(), &kern));
  const void* src = h->tmp.p;
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
