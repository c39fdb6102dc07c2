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
__device__ __forceinline__ void stockham_stage(V* __restrict__ s, const V* __restrict__ tw, int tid, unsigned inv) {
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
#pragma unroll
    for (int r = 1; r < R; ++r) v[m][r] = cmul_l(v[m][r], cconj_if(tw[r * k * (N / (NS * R))], inv));
    Dft<R, V>::run(v[m], inv);
    const int base = (b / NS) * NS * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) s[Tile::addr(line, base + r * NS)] = v[m][r];
  }
  __syncthreads();
}

template <class Tile, int NT, int NS, typename V> struct MiddleStages {
  // applies stages NS, NS*R, ... up to but excluding the last one
  __device__ __forceinline__ static void run(V* s, const V* tw, int tid, unsigned inv) {
    constexpr int R = RadixChoice<Tile::N / NS, MaxRadix<Tile, NT>::value>::R;
    if constexpr (NS * R < Tile::N) {
      stockham_stage<Tile, NT, NS, V>(s, tw, tid, inv);
      MiddleStages<Tile, NT, NS * R, V>::run(s, tw, tid, inv);
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
template <class Tile, int NT, typename V>
__device__ __forceinline__ void tile_fft_regs(V* r, V* __restrict__ s, const V* __restrict__ tw, int tid, unsigned inv) {
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
  MiddleStages<Tile, NT, R1, V>::run(s, tw, tid, inv);
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
#pragma unroll
    for (int q = 1; q < RL; ++q) v[m][q] = cmul_l(v[m][q], cconj_if(tw[q * b], inv));
    Dft<RL, V>::run(v[m], inv);
#pragma unroll
    for (int q = 0; q < RL; ++q) r[m + q * PERL] = v[m][q];
  }
}
