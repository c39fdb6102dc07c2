// Stockham FFT over a tile of independent lines, registers + shared memory.
//
// Replaces the reference's batched cuFFT Z2Z plans (cufft.py:274-343): a
// row-pass tile holds whole rows (the Axis1 plan), a column-pass tile holds
// whole columns (the Axis0 plan).  Transforms are unnormalised in both
// directions, like cuFFT: forward uses exp(-2 pi i jk/N), inverse exp(+...).
//
// Algorithm: the radix-R Stockham autosort FFT (Govindaraju et al., SC08,
// "High Performance Discrete Fourier Transforms on Graphics Processors"),
// mixed radix 8/4/2.  Twiddles come from a per-N table
// tw[m] = exp(-2 pi i m / N) built on the host in extended precision; the
// inverse transform uses their conjugates.  The direction is a run-time
// argument so that a pass kernel holds one copy of the FFT code: the
// double-float form of a 1024-point FFT alone is tens of kilobytes of
// instructions, and several inlined copies overflow the instruction cache.
//
// Data placement.  Each thread owns E elements of the tile, all on one line:
//   line = tid % LINES,  position p_k = tid / LINES + k * (N / E),  k = 0..E-1.
// Every stage has radix min(8, E) (less for the remainder), so the first
// Stockham stage (span 1) reads exactly these elements and the last stage
// writes exactly these positions, so an FFT starts from
// and ends in registers; only the stages in between go through shared memory
// (read all inputs, synchronise, write all outputs).  Element-wise factors,
// global loads and stores and reductions all work on the registers.
#pragma once
#include <type_traits>

#include "aw_common.cuh"

// Tile geometry: a row tile holds L lines of N contiguous elements (padded by
// one element per line when L > 1 so that lanes on different lines fall in
// different banks); a column tile holds B lines interleaved (element e of line
// c sits at e*B + c), the layout of a B-column slab of a row-major grid.
// In both, consecutive work items walk across lines first.
template <int N_, int L_> struct RowTile {
  static constexpr int N = N_;
  static constexpr int LINES = L_;
  static constexpr bool IS_ROW = true;
  static constexpr int STRIDE = L_ > 1 ? N_ + 1 : N_;
  static constexpr int SMEM_ELEMS = STRIDE * L_;
  __device__ __forceinline__ static int addr(int line, int e) { return line * STRIDE + e; }
};

template <int N_, int B_> struct ColTile {
  static constexpr int N = N_;
  static constexpr int LINES = B_;
  static constexpr bool IS_ROW = false;
  static constexpr int SMEM_ELEMS = N_ * B_;
  __device__ __forceinline__ static int addr(int line, int e) { return e * B_ + line; }
};

// work item u -> (line, butterfly index b): lines first
template <class Tile>
__device__ __forceinline__ void split_item(int u, int& line, int& b) {
  line = u % Tile::LINES;
  b = u / Tile::LINES;
}

// ---------------------------------------------------------------- radix kernels
// inv: 0 forward, 0x80000000 inverse (sign-bit mask, see aw_common.cuh)
template <int R, typename V> struct Dft;

// run: outputs renormalised (double-float); run_lazy: sums left unrenormalised for an enclosing butterfly
template <typename V> struct Dft<2, V> {
  __device__ __forceinline__ static void run(V* v, unsigned) {
    V a = v[0], b = v[1];
    v[0] = cnorm(cadd_l(a, b));
    v[1] = cnorm(csub_l(a, b));
  }
};

template <typename V> struct Dft<4, V> {
  __device__ __forceinline__ static void run_lazy(V* v, unsigned inv) {
    V t0 = cadd_l(v[0], v[2]);
    V t1 = csub_l(v[0], v[2]);
    V t2 = cadd_l(v[1], v[3]);
    V t3 = cmul_mi_dir(csub_l(v[1], v[3]), inv);
    v[0] = cadd_l(t0, t2);
    v[2] = csub_l(t0, t2);
    v[1] = cadd_l(t1, t3);
    v[3] = csub_l(t1, t3);
  }
  __device__ __forceinline__ static void run(V* v, unsigned inv) {
    run_lazy(v, inv);
#pragma unroll
    for (int q = 0; q < 4; ++q) v[q] = cnorm(v[q]);
  }
};

template <typename V> struct Dft<8, V> {
  __device__ __forceinline__ static void run(V* v, unsigned inv) {
    // y[2q]   = DFT4(a[n] + a[n+4])
    // y[2q+1] = DFT4((a[n] - a[n+4]) * w8^n)
    V b[4], c[4];
#pragma unroll
    for (int n = 0; n < 4; ++n) {
      b[n] = cadd_l(v[n], v[n + 4]);
      c[n] = csub_l(v[n], v[n + 4]);
    }
    c[1] = cmul_w8_1_dir(c[1], inv);
    c[2] = cmul_mi_dir(c[2], inv);
    c[3] = cmul_w8_3_dir(c[3], inv);
    Dft<4, V>::run_lazy(b, inv);
    Dft<4, V>::run_lazy(c, inv);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      v[2 * q] = cnorm(b[q]);
      v[2 * q + 1] = cnorm(c[q]);
    }
  }
};

// Native FP64, the first (twiddle-free) radix-8 stage: the odd outputs as two tangent-form butterflies
// (see below).  With c_n = v_n - v_(n+4) and W4 = -i (forward; +i inverse):
//   y_(2q+1) = g + W8^(2q+1) h,  g = c0 + W4^(2q+1) c2,  h = c1 + W4^(2q+1) c3
// so y1, y5 pair g_e = c0 + W4 c2, h_e = c1 + W4 c3 under W8 = m (1 + i q) with m = 1/sqrt2, q = -1, and
// y3, y7 pair g_o = c0 - W4 c2, h_o = c1 - W4 c3 under W8^3 = -m (1 - i) (the inverse conjugates q):
// 52 FP64 instructions for the 8 points instead of 56 (the products by W8 and W8^3, then a radix-4).
template <> struct Dft<8, double2> {
  __device__ __forceinline__ static void run(double2* v, unsigned inv) {
    double2 b[4], c[4];
#pragma unroll
    for (int n = 0; n < 4; ++n) {
      b[n] = cadd_l(v[n], v[n + 4]);
      c[n] = csub_l(v[n], v[n + 4]);
    }
    Dft<4, double2>::run_lazy(b, inv);
    const double2 c2 = cmul_mi_dir(c[2], inv), c3 = cmul_mi_dir(c[3], inv);
    const double2 ge = cadd_l(c[0], c2), go = csub_l(c[0], c2);
    const double2 he = cadd_l(c[1], c3), ho = csub_l(c[1], c3);
    // u = h (1 + i q): q = -1 (forward) or +1 for the pair of W8, the opposite for W8^3
    const double ue_x = he.x + flip(he.y, inv), ue_y = he.y - flip(he.x, inv);
    const double uo_x = ho.x - flip(ho.y, inv), uo_y = ho.y + flip(ho.x, inv);
    const double r = rsqrt2<double>();
#pragma unroll
    for (int q = 0; q < 4; ++q) v[2 * q] = b[q];
    v[1] = make_double2(fma(r, ue_x, ge.x), fma(r, ue_y, ge.y));
    v[5] = make_double2(fma(-r, ue_x, ge.x), fma(-r, ue_y, ge.y));
    v[3] = make_double2(fma(-r, uo_x, go.x), fma(-r, uo_y, go.y));
    v[7] = make_double2(fma(r, uo_x, go.x), fma(r, uo_y, go.y));
  }
};

// ---------------------------------------------------------------- native FP64: tangent-form butterflies
// The native FP64 passes are bound by the FP64 pipe, so their FFT is written to need the fewest FP64
// instructions.  A radix-R stage with twiddle w = exp(-+2 pi i k / (NS R)) is computed as log2 R
// levels of twiddled radix-2 butterflies (decimation in time on the stage's R inputs), each
//   a, b  ->  a + t b, a - t b
// with its twiddle in tangent form t = i^e m (1 + i q), |q| <= 1 (m = cos, q = tan when |cos| >= |sin|;
// m = sin, q = -cot and e = 1 otherwise): u = b (1 + i q) is two FMAs, the factor i^e a swap and sign
// flips on the integer pipe, and a +- m i^e u four FMAs: 6 FP64 instructions a butterfly where a
// complex product and two complex sums take 8, and two roundings per output instead of three
// (Linzer and Feig, "Implementation of efficient FFT algorithms on fused multiply-add
// architectures", IEEE Trans. Signal Processing 41, 1993).  A 1024-point transform of radix-8, 8, 8,
// 2 stages needs 27.5 FP64 instructions a point instead of 32: 6.5 in the first stage (w = 1: plain
// sums, its W8 pair in tangent form, Dft<8, double2> above), 9 a radix-8 stage, 3 the radix-2 one.
//
// Table (built on the host in extended precision, one per line length N): for R in {2, 4, 8}, span
// NS in {1, 2, .., N / 2} and k < NS, the entries of w = exp(-2 pi i k / (NS R)):
//   R = 8: w^4, w^2, w, w W8     R = 4: w^2, w     R = 2: w          (W8 = exp(-i pi / 4))
// at tan_off<R, N>(NS, k): (m, q) pairs in `mq`, the exponent e in `te`; the inverse transform uses the
// conjugates (q -> -q, e -> -e mod 4), and the factors W4 = -i of the radix's inner levels are
// further powers of i.
template <int R> struct TanEnt {
  static constexpr int n = R == 8 ? 4 : (R == 4 ? 2 : 1);
};
template <int R, int N> __host__ __device__ constexpr int tan_base() {
  return R == 2 ? 0 : (R == 4 ? (N - 1) : 3 * (N - 1));
}
template <int R, int N> __device__ __forceinline__ int tan_off(int ns, int k) {
  return tan_base<R, N>() + (ns - 1 + k) * TanEnt<R>::n;
}

// a, b -> a + t b, a - t b with t = i^e m (1 + i q) (forward), its conjugate for the inverse
__device__ __forceinline__ void bf_tan(double2& a, double2& b, double2 mq, int e, unsigned inv) {
  const double q = flip(mq.y, inv);
  e = (inv ? -e : e) & 3;
  const double ux = fma(-q, b.y, b.x), uy = fma(q, b.x, b.y);
  // v = i^e u by bit operations on the integer pipe (a swap when e is odd, then sign flips): e varies
  // across the lanes of a row tile, and a data-dependent select there left FP64 instructions issued
  // for part of a warp (23.7 of 32 lanes active on average in the headline's row pass)
  const unsigned long long xb = (unsigned long long)__double_as_longlong(ux);
  const unsigned long long yb = (unsigned long long)__double_as_longlong(uy);
  const unsigned long long t = (xb ^ yb) & (0ull - (unsigned long long)(e & 1));
  const double vx = __longlong_as_double((long long)(xb ^ t ^ ((unsigned long long)((e ^ (e >> 1)) & 1) << 63)));
  const double vy = __longlong_as_double((long long)(yb ^ t ^ ((unsigned long long)((e >> 1) & 1) << 63)));
  const double m = mq.x;
  const double2 a0 = a;
  a = make_double2(fma(m, vx, a0.x), fma(m, vy, a0.y));
  b = make_double2(fma(-m, vx, a0.x), fma(-m, vy, a0.y));
}

// X_q = sum_r v_r w^r W_R^(rq), from the stage's table entries; outputs in natural order
template <int R> struct DftTan;
template <> struct DftTan<2> {
  __device__ __forceinline__ static void run(double2* v, const double2* mq, const unsigned char* te, unsigned inv) {
    bf_tan(v[0], v[1], mq[0], te[0], inv);
  }
};
template <> struct DftTan<4> {
  __device__ __forceinline__ static void run(double2* v, const double2* mq, const unsigned char* te, unsigned inv) {
    const double2 t2 = mq[0], t1 = mq[1];
    const int e2 = te[0], e1 = te[1];
    bf_tan(v[0], v[2], t2, e2, inv);
    bf_tan(v[1], v[3], t2, e2, inv);
    bf_tan(v[0], v[1], t1, e1, inv);            // X0, X2
    bf_tan(v[2], v[3], t1, (e1 + 3) & 3, inv);  // X1, X3 (twiddle w W4)
    const double2 x1 = v[2];
    v[2] = v[1];
    v[1] = x1;
  }
};
template <> struct DftTan<8> {
  __device__ __forceinline__ static void run(double2* v, const double2* mq, const unsigned char* te, unsigned inv) {
    const double2 t4 = mq[0], t2 = mq[1], t1 = mq[2], t18 = mq[3];
    const int e4 = te[0], e2 = te[1], e1 = te[2], e18 = te[3];
#pragma unroll
    for (int j = 0; j < 4; ++j) bf_tan(v[j], v[j + 4], t4, e4, inv);
    // even outputs from (v0..v3) with w, odd ones from (v4..v7) with w W8
    bf_tan(v[0], v[2], t2, e2, inv);
    bf_tan(v[1], v[3], t2, e2, inv);
    bf_tan(v[4], v[6], t2, (e2 + 3) & 3, inv);
    bf_tan(v[5], v[7], t2, (e2 + 3) & 3, inv);
    bf_tan(v[0], v[1], t1, e1, inv);             // X0, X4
    bf_tan(v[2], v[3], t1, (e1 + 3) & 3, inv);   // X2, X6
    bf_tan(v[4], v[5], t18, e18, inv);           // X1, X5
    bf_tan(v[6], v[7], t18, (e18 + 3) & 3, inv); // X3, X7
    const double2 x4 = v[1], x1 = v[4], x2 = v[2], x6 = v[3], x5 = v[5], x3 = v[6];
    v[1] = x1;
    v[2] = x2;
    v[3] = x3;
    v[4] = x4;
    v[5] = x5;
    v[6] = x6;
  }
};

// radix of a stage with REM points left to combine: at most MAXR, the number of elements a thread
// owns when it is below 8 (every stage then gives each thread whole butterflies)
template <int REM, int MAXR = 8> struct RadixChoice {
  static constexpr int R = REM >= MAXR ? MAXR : REM;
};
template <class Tile, int NT> struct MaxRadix {
  static constexpr int E = Tile::N * Tile::LINES / NT;
  static constexpr int value = E < 8 ? E : 8;
};

// Middle Stockham stage with span NS: shared memory to shared memory, in place
// (all inputs are read before the barrier, all outputs written after it).
template <class Tile, int NT, int NS, typename V>
__device__ __forceinline__ void stockham_stage(V* __restrict__ s, const V* __restrict__ tw, int tid, unsigned inv,
                                               const double2* __restrict__ tmq, const unsigned char* __restrict__ te) {
  constexpr int N = Tile::N;
  constexpr int R = RadixChoice<N / NS, MaxRadix<Tile, NT>::value>::R;
  constexpr int NB = N / R;
  constexpr int TOT = Tile::LINES * NB;
  static_assert(TOT % NT == 0, "work items must divide evenly over the threads");
  constexpr int PER = TOT / NT;
  V v[PER][R];
#pragma unroll
  for (int m = 0; m < PER; ++m) {
    int line, b;
    split_item<Tile>(tid + m * NT, line, b);
#pragma unroll
    for (int r = 0; r < R; ++r) v[m][r] = s[Tile::addr(line, b + r * NB)];
  }
  __syncthreads();
#pragma unroll
  for (int m = 0; m < PER; ++m) {
    int line, b;
    split_item<Tile>(tid + m * NT, line, b);
    const int k = b & (NS - 1);
    if constexpr (std::is_same<V, double2>::value) {
      const int off = tan_off<R, N>(NS, k);
      DftTan<R>::run(v[m], tmq + off, te + off, inv);
    } else {
#pragma unroll
      for (int r = 1; r < R; ++r) v[m][r] = cmul_l(v[m][r], cconj_if(tw[r * k * (N / (NS * R))], inv));
      Dft<R, V>::run(v[m], inv);
    }
    const int base = (b / NS) * NS * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) s[Tile::addr(line, base + r * NS)] = v[m][r];
  }
  __syncthreads();
}

template <class Tile, int NT, int NS, typename V> struct MiddleStages {
  // applies stages NS, NS*R, ... up to but excluding the last one
  __device__ __forceinline__ static void run(V* s, const V* tw, int tid, unsigned inv, const double2* tmq,
                                             const unsigned char* te) {
    constexpr int R = RadixChoice<Tile::N / NS, MaxRadix<Tile, NT>::value>::R;
    if constexpr (NS * R < Tile::N) {
      stockham_stage<Tile, NT, NS, V>(s, tw, tid, inv, tmq, te);
      MiddleStages<Tile, NT, NS * R, V>::run(s, tw, tid, inv, tmq, te);
    }
  }
};

template <int N, int NS, int MAXR> struct LastSpan {
  static constexpr int R = RadixChoice<N / NS, MAXR>::R;
  static constexpr int value = NS * R >= N ? NS : LastSpan<N, NS * R, MAXR>::value;
};
template <int N, int MAXR> struct LastSpan<N, N, MAXR> {
  static constexpr int value = N;
};

// Full FFT of every line of the tile, registers in and out; inv selects the direction.
//   r[k] holds the thread's element at position tid / LINES + k * (N / E) of line tid % LINES.
// tmq / te: the tangent-form twiddle table of the line length (native FP64 only)
template <class Tile, int NT, typename V>
__device__ __forceinline__ void tile_fft_regs(V* r, V* __restrict__ s, const V* __restrict__ tw, int tid, unsigned inv,
                                              const double2* __restrict__ tmq = nullptr,
                                              const unsigned char* __restrict__ te = nullptr) {
  constexpr int N = Tile::N;
  constexpr int L = Tile::LINES;
  constexpr int E = N * L / NT;
  constexpr int MAXR = MaxRadix<Tile, NT>::value;
  constexpr int R1 = RadixChoice<N, MAXR>::R;
  static_assert(R1 == MAXR && E % R1 == 0, "the first stage combines the thread's own elements");
  constexpr int PER1 = E / R1;
  // the previous use of the tile may still be read by other threads
  __syncthreads();
  // stage 1 (span 1): inputs are the thread's own elements, no twiddles
#pragma unroll
  for (int m = 0; m < PER1; ++m) {
    V v[R1];
#pragma unroll
    for (int q = 0; q < R1; ++q) v[q] = r[m + q * PER1];
    Dft<R1, V>::run(v, inv);
    int line, b;
    split_item<Tile>(tid + m * NT, line, b);
#pragma unroll
    for (int q = 0; q < R1; ++q) s[Tile::addr(line, b * R1 + q)] = v[q];
  }
  __syncthreads();
  MiddleStages<Tile, NT, R1, V>::run(s, tw, tid, inv, tmq, te);
  // last stage: span NSL = N / RL; outputs land on the thread's own positions
  constexpr int NSL = LastSpan<N, R1, MAXR>::value;
  constexpr int RL = N / NSL;
  constexpr int NBL = N / RL;
  constexpr int PERL = L * NBL / NT;
  V v[PERL][RL];
#pragma unroll
  for (int m = 0; m < PERL; ++m) {
    int line, b;
    split_item<Tile>(tid + m * NT, line, b);
#pragma unroll
    for (int q = 0; q < RL; ++q) v[m][q] = s[Tile::addr(line, b + q * NBL)];
  }
#pragma unroll
  for (int m = 0; m < PERL; ++m) {
    int line, b;
    split_item<Tile>(tid + m * NT, line, b);
    // b < NSL here, so the twiddle exponent is q * b and the outputs go to b + q * NSL
    if constexpr (std::is_same<V, double2>::value) {
      const int off = tan_off<RL, N>(NSL, b);
      DftTan<RL>::run(v[m], tmq + off, te + off, inv);
    } else {
#pragma unroll
      for (int q = 1; q < RL; ++q) v[m][q] = cmul_l(v[m][q], cconj_if(tw[q * b], inv));
      Dft<RL, V>::run(v[m], inv);
    }
#pragma unroll
    for (int q = 0; q < RL; ++q) r[m + q * PERL] = v[m][q];
  }
}
