// Shared-memory Stockham FFT over a tile of independent lines.
//
// Replaces the reference's batched cuFFT Z2Z plans (cufft.py:274-343): a
// row-pass tile holds whole rows (the Axis1 plan), a column-pass tile holds
// whole columns (the Axis0 plan).  Transforms are unnormalised in both
// directions, like cuFFT: forward uses exp(-2 pi i jk/N), inverse exp(+...).
//
// Algorithm: the radix-R Stockham autosort FFT (Govindaraju et al., SC08,
// "High Performance Discrete Fourier Transforms on Graphics Processors"),
// mixed radix 8/4/2, in place in shared memory: every stage reads all of its
// inputs into registers, synchronises, then writes its outputs.  Twiddles
// come from a per-N table tw[m] = exp(-2 pi i m / N) built on the host in
// extended precision and rounded once.
#pragma once
#include "aw_common.cuh"

// Tile geometry: a row tile holds L lines of N contiguous elements; a column
// tile holds B lines interleaved (element e of line c sits at e*B + c), which
// is exactly the layout of a B-column slab of a row-major grid.
template <int N_, int L_> struct RowTile {
  static constexpr int N = N_;
  static constexpr int LINES = L_;
  static constexpr bool IS_ROW = true;
  __device__ __forceinline__ static int addr(int line, int e) { return line * N + e; }
  // consecutive work items walk along a line
  __device__ __forceinline__ static void split(int u, int nb, int& line, int& b) {
    line = u / nb;
    b = u - line * nb;
  }
  // element index in the tile -> (line, position)
  __device__ __forceinline__ static void elem(int e, int& line, int& pos) {
    line = e / N;
    pos = e - line * N;
  }
};

template <int N_, int B_> struct ColTile {
  static constexpr int N = N_;
  static constexpr int LINES = B_;
  static constexpr bool IS_ROW = false;
  __device__ __forceinline__ static int addr(int line, int e) { return e * B_ + line; }
  // consecutive work items walk across lines (neighbouring columns)
  __device__ __forceinline__ static void split(int u, int nb, int& line, int& b) {
    b = u / B_;
    line = u - b * B_;
  }
  __device__ __forceinline__ static void elem(int e, int& line, int& pos) {
    pos = e / B_;
    line = e - pos * B_;
  }
};

// ---------------------------------------------------------------- radix kernels
template <int R, bool FWD, typename V> struct Dft;

template <bool FWD, typename V> struct Dft<2, FWD, V> {
  __device__ __forceinline__ static void run(V* v) {
    V a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};

template <bool FWD, typename V> struct Dft<4, FWD, V> {
  __device__ __forceinline__ static void run(V* v) {
    V t0 = cadd(v[0], v[2]);
    V t1 = csub(v[0], v[2]);
    V t2 = cadd(v[1], v[3]);
    V d = csub(v[1], v[3]);
    V t3 = FWD ? cmul_mi(d) : cmul_pi(d);
    v[0] = cadd(t0, t2);
    v[2] = csub(t0, t2);
    v[1] = cadd(t1, t3);
    v[3] = csub(t1, t3);
  }
};

template <bool FWD, typename V> struct Dft<8, FWD, V> {
  __device__ __forceinline__ static void run(V* v) {
    // y[2q]   = DFT4(a[n] + a[n+4])
    // y[2q+1] = DFT4((a[n] - a[n+4]) * w8^n)
    V b[4], c[4];
#pragma unroll
    for (int n = 0; n < 4; ++n) {
      b[n] = cadd(v[n], v[n + 4]);
      c[n] = csub(v[n], v[n + 4]);
    }
    c[1] = cmul_w8_1<V, FWD>(c[1]);
    c[2] = FWD ? cmul_mi(c[2]) : cmul_pi(c[2]);
    c[3] = cmul_w8_3<V, FWD>(c[3]);
    Dft<4, FWD, V>::run(b);
    Dft<4, FWD, V>::run(c);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      v[2 * q] = b[q];
      v[2 * q + 1] = c[q];
    }
  }
};

template <int REM> struct RadixChoice {
  static constexpr int R = REM >= 8 ? 8 : REM;
};

// One Stockham stage with span NS (product of the radices already applied).
template <class Tile, int NT, int NS, bool FWD, typename V>
__device__ __forceinline__ void stockham_stage(V* __restrict__ s, const V* __restrict__ tw, int tid) {
  constexpr int N = Tile::N;
  constexpr int R = RadixChoice<N / NS>::R;
  constexpr int NB = N / R;
  constexpr int TOT = Tile::LINES * NB;
  static_assert(TOT % NT == 0, "work items must divide evenly over the threads");
  constexpr int PER = TOT / NT;
  V v[PER][R];
#pragma unroll
  for (int m = 0; m < PER; ++m) {
    int line, b;
    Tile::split(tid + m * NT, NB, line, b);
#pragma unroll
    for (int r = 0; r < R; ++r) v[m][r] = s[Tile::addr(line, b + r * NB)];
  }
  __syncthreads();
#pragma unroll
  for (int m = 0; m < PER; ++m) {
    int line, b;
    Tile::split(tid + m * NT, NB, line, b);
    const int k = b & (NS - 1);
    if (NS > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) {
        V w = tw[r * k * (N / (NS * R))];
        v[m][r] = FWD ? cmul(v[m][r], w) : cmulc(v[m][r], w);
      }
    }
    Dft<R, FWD, V>::run(v[m]);
    const int base = (b / NS) * NS * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) s[Tile::addr(line, base + r * NS)] = v[m][r];
  }
  __syncthreads();
}

template <class Tile, int NT, int NS, bool FWD, typename V> struct StockhamRun {
  __device__ __forceinline__ static void run(V* s, const V* tw, int tid) {
    stockham_stage<Tile, NT, NS, FWD, V>(s, tw, tid);
    StockhamRun<Tile, NT, NS * RadixChoice<Tile::N / NS>::R, FWD, V>::run(s, tw, tid);
  }
};

// terminates when the span reaches N
template <int N, int L, int NT, bool FWD, typename V> struct StockhamRun<RowTile<N, L>, NT, N, FWD, V> {
  __device__ __forceinline__ static void run(V*, const V*, int) {}
};
template <int N, int B, int NT, bool FWD, typename V> struct StockhamRun<ColTile<N, B>, NT, N, FWD, V> {
  __device__ __forceinline__ static void run(V*, const V*, int) {}
};

// Full in-place FFT of every line of the tile.  Expects the tile to be
// complete in shared memory (caller synchronised); returns synchronised.
template <class Tile, int NT, bool FWD, typename V>
__device__ __noinline__ void tile_fft(V* s, const V* tw, int tid) {
  StockhamRun<Tile, NT, 1, FWD, V>::run(s, tw, tid);
}
