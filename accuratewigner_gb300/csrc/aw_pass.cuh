// Fused FFT pass kernels for sm_103a.  See aw_pass.h for the pass program.
//
// A row pass owns L whole rows of the grid (contiguous in HBM); a column pass
// owns a slab of B whole columns (B * element size >= 64-128 bytes per grid row,
// so every row segment is a full set of DRAM sectors).  Each pass reads its
// tile from HBM once, keeps it in shared memory for every FFT, phase multiply
// and reduction of its program, and writes it once.
#pragma once
#include "aw_common.cuh"
#include "aw_fft.cuh"
#include "aw_pass.h"

template <typename V> struct PassShape;

// complex128: 32 KB row tiles, 128 KB column slabs, 8 elements per thread
template <> struct PassShape<double2> {
  template <int N> struct Row {
    static constexpr int L = N >= 2048 ? 1 : 2048 / N;
    static constexpr int TILE = L * N;
    static constexpr int E = TILE / 1024 > 8 ? TILE / 1024 : 8;
    static constexpr int NT = TILE / E;
  };
  template <int N> struct Col {
    static constexpr int B = N <= 1024 ? 8 : (8192 / N);
    static constexpr int TILE = B * N;
    static constexpr int E = TILE / 1024 > 8 ? TILE / 1024 : 8;
    static constexpr int NT = TILE / E;
  };
};

// complex64: 32 KB row tiles, 128 KB column slabs
template <> struct PassShape<float2> {
  template <int N> struct Row {
    static constexpr int L = N >= 4096 ? 1 : 4096 / N;
    static constexpr int TILE = L * N;
    static constexpr int E = TILE / 1024 > 8 ? TILE / 1024 : 8;
    static constexpr int NT = TILE / E;
  };
  template <int N> struct Col {
    static constexpr int B = N <= 1024 ? 16 : (16384 / N);
    static constexpr int TILE = B * N;
    static constexpr int E = TILE / 1024 > 8 ? TILE / 1024 : 8;
    static constexpr int NT = TILE / E;
  };
};

template <typename V> struct RealOf;
template <> struct RealOf<double2> { typedef double type; };
template <> struct RealOf<float2> { typedef float type; };

// apply one AwFactor to the thread's own elements of the tile
template <typename V, class Tile, int NT>
__device__ __forceinline__ void apply_factor(V* s, const AwFactor& f, int line0, int ncols, int tid,
                                             long long tab_off, long long elem_off, int inst) {
  typedef typename RealOf<V>::type T;
  constexpr int TILE = Tile::N * Tile::LINES;
  const V* ct = (const V*)f.col_tab;
  const V* rt = (const V*)f.row_tab;
  const T* mk = (const T*)f.mask;
  const V* sh = (const V*)f.sh_hi;
  const V* sl = (const V*)f.sh_lo;
  if (ct) ct += tab_off;
  if (rt) rt += tab_off;
  if (mk) mk += elem_off;
  T sc = (T)f.scale;
  T sci = T(0);
  if (f.scale_ptr) {
    sc = (T)(f.scale * f.scale_ptr[2 * inst]);
    sci = (T)(f.scale * f.scale_ptr[2 * inst + 1]);
  }
  const int nhi = f.sh_lo_n ? Tile::N / f.sh_lo_n : 0;
#pragma unroll 4
  for (int e = tid; e < TILE; e += NT) {
    int line, pos;
    Tile::elem(e, line, pos);
    const int i = Tile::IS_ROW ? line0 + line : pos;
    const int j = Tile::IS_ROW ? pos : line0 + line;
    V v = s[e];
    T m = T(1);
    if (f.sign && ((f.sign == 1 ? i + j : (f.sign == 2 ? i : j)) & 1)) m = -m;
    if (mk) {
      T q = mk[(long long)i * ncols + j];
      m *= q;
      if (f.mask_pow == 2) m *= q;
    }
    v = sci == T(0) ? cscale(v, m * sc) : cmul(v, cmake<V>(m * sc, m * sci));
    if (ct) v = cmul(v, ct[j]);
    if (rt) v = cmulc(v, rt[i]);
    if (f.sh_lo_n) {
      const int lg = line0 + line;
      const int q = (pos + f.sh_roll) & (Tile::N - 1);
      V w = cmul(sh[(long long)lg * nhi + q / f.sh_lo_n], sl[(long long)lg * f.sh_lo_n + (q % f.sh_lo_n)]);
      v = cmul(v, w);
    }
    s[e] = v;
  }
}

template <class Tile, int NT, typename V>
__device__ __forceinline__ void run_fft(V* s, const V* tw, int dir, int tid) {
  if (dir == 0) return;
  __syncthreads();
  if (dir > 0)
    tile_fft<Tile, NT, true, V>(s, tw, tid);
  else
    tile_fft<Tile, NT, false, V>(s, tw, tid);
}

// global element offset of tile element e
template <class Tile>
__device__ __forceinline__ long long gofs(int e, int line0, int ncols) {
  int line, pos;
  Tile::elem(e, line, pos);
  return Tile::IS_ROW ? (long long)(line0 + line) * ncols + pos : (long long)pos * ncols + line0 + line;
}

template <typename V, class Tile, int NT>
__device__ __forceinline__ void store_tile(V* __restrict__ dst, const V* s, int line0, int ncols, int tid, bool sgn) {
  constexpr int TILE = Tile::N * Tile::LINES;
#pragma unroll 4
  for (int e = tid; e < TILE; e += NT) {
    V v = s[e];
    if (sgn) {
      int line, pos;
      Tile::elem(e, line, pos);
      const int i = Tile::IS_ROW ? line0 + line : pos;
      const int j = Tile::IS_ROW ? pos : line0 + line;
      if ((i + j) & 1) v = cmake<V>(-v.x, -v.y);
    }
    dst[gofs<Tile>(e, line0, ncols)] = v;
  }
}

// deterministic per-block sum of |v|^2 over the tile (row passes)
template <typename V, class Tile, int NT>
__device__ __forceinline__ void row_abs2(const V* s, const AwPassArgs& a, int tid, int inst) {
  constexpr int TILE = Tile::N * Tile::LINES;
  constexpr int E = TILE / NT;
  __shared__ double red2[NT];
  double acc = 0.0;
#pragma unroll 4
  for (int k = 0; k < E; ++k) {
    V v = s[tid + k * NT];
    acc += (double)v.x * (double)v.x + (double)v.y * (double)v.y;
  }
  red2[tid] = acc;
  __syncthreads();
  for (int w = NT / 2; w > 0; w >>= 1) {
    if (tid < w) red2[tid] += red2[tid + w];
    __syncthreads();
  }
  if (tid == 0) a.red_abs2[(long long)inst * gridDim.x + blockIdx.x] = red2[0];
  __syncthreads();
}

template <typename V, class Tile, int NT>
__global__ void __launch_bounds__(NT) aw_pass_kernel(const AwPassArgs a) {
  extern __shared__ __align__(16) unsigned char aw_smem[];
  V* s = reinterpret_cast<V*>(aw_smem);
  constexpr int TILE = Tile::N * Tile::LINES;
  constexpr int E = TILE / NT;
  const int inst = blockIdx.y;
  if (a.stop && a.stop[inst]) return;
  const int tid = threadIdx.x;
  const int line0 = blockIdx.x * Tile::LINES;
  const int ncols = a.ncols;
  const long long eoff = (long long)inst * a.batch_elems;
  const long long toff = (long long)inst * a.batch_tab;
  const V* in = (const V*)a.in + eoff;
  const V* tw = (const V*)a.tw;

#pragma unroll 4
  for (int e = tid; e < TILE; e += NT) s[e] = in[gofs<Tile>(e, line0, ncols)];

  if (a.f0.active) apply_factor<V, Tile, NT>(s, a.f0, line0, ncols, tid, toff, eoff, inst);
  run_fft<Tile, NT>(s, tw, a.d1, tid);
  if (a.f1.active) apply_factor<V, Tile, NT>(s, a.f1, line0, ncols, tid, toff, eoff, inst);

  if (a.mid_out) store_tile<V, Tile, NT>((V*)a.mid_out + eoff, s, line0, ncols, tid, a.mid_sign != 0);
  if (Tile::IS_ROW && a.diag_out) {
    // element (i, i) of each row at the branch point
#pragma unroll 4
    for (int e = tid; e < TILE; e += NT) {
      int line, pos;
      Tile::elem(e, line, pos);
      if (line0 + line == pos) {
        V v = s[e];
        a.diag_out[(long long)inst * a.nrows + pos] = make_double2((double)v.x, (double)v.y);
      }
    }
  }
  if (Tile::IS_ROW && a.red_abs2 && !a.abs2_end) row_abs2<V, Tile, NT>(s, a, tid, inst);
  if (a.br_out) {
    V keep[E];
#pragma unroll
    for (int k = 0; k < E; ++k) keep[k] = s[tid + k * NT];
    run_fft<Tile, NT>(s, tw, a.br_d1, tid);
    if (a.fbr.active) apply_factor<V, Tile, NT>(s, a.fbr, line0, ncols, tid, toff, eoff, inst);
    run_fft<Tile, NT>(s, tw, a.br_d2, tid);
    store_tile<V, Tile, NT>((V*)a.br_out + eoff, s, line0, ncols, tid, false);
    __syncthreads();
#pragma unroll
    for (int k = 0; k < E; ++k) s[tid + k * NT] = keep[k];
  }

  if (a.f2.active) apply_factor<V, Tile, NT>(s, a.f2, line0, ncols, tid, toff, eoff, inst);
  run_fft<Tile, NT>(s, tw, a.d2, tid);
  if (a.f3.active) apply_factor<V, Tile, NT>(s, a.f3, line0, ncols, tid, toff, eoff, inst);
  if (a.out) store_tile<V, Tile, NT>((V*)a.out + eoff, s, line0, ncols, tid, false);
  if (Tile::IS_ROW && a.red_abs2 && a.abs2_end) row_abs2<V, Tile, NT>(s, a, tid, inst);

  if (!Tile::IS_ROW && (a.red_line || a.red_cross || a.red_sq)) {
    // deterministic reductions over the column slab (fixed order, no atomics)
    constexpr int B = Tile::LINES;
    __shared__ double red[NT];
    double lsum = 0.0, sq = 0.0;
#pragma unroll 4
    for (int k = 0; k < E; ++k) {
      const int e = tid + k * NT;
      V v = s[e];
      const double re = (double)v.x, im = (double)v.y;
      lsum += re;
      sq += re * re - im * im;
      if (a.red_cross) {
        // the B values of one grid row sit in B consecutive lanes
        double c = re;
#pragma unroll
        for (int o = B / 2; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o, B);
        if ((tid & (B - 1)) == 0)
          a.red_cross[((long long)inst * gridDim.x + blockIdx.x) * a.nrows + e / B] = c;
      }
    }
    if (a.red_line) {
      red[tid] = lsum;
      __syncthreads();
      if (tid < B) {
        double acc = 0.0;
        for (int m = tid; m < NT; m += B) acc += red[m];
        a.red_line[(long long)inst * ncols + line0 + tid] = acc;
      }
      __syncthreads();
    }
    if (a.red_sq) {
      red[tid] = sq;
      __syncthreads();
      for (int w = NT / 2; w > 0; w >>= 1) {
        if (tid < w) red[tid] += red[tid + w];
        __syncthreads();
      }
      if (tid == 0) a.red_sq[(long long)inst * gridDim.x + blockIdx.x] = red[0];
    }
  }
}

// ------------------------------------------------------------------ dispatch
template <typename V, int N>
static int launch_row_n(const AwPassArgs* a, int batch, cudaStream_t st) {
  typedef typename PassShape<V>::template Row<N> S;
  typedef RowTile<N, S::L> Tile;
  if (a->nrows % S::L) return -2;
  const size_t smem = sizeof(V) * S::TILE;
  auto kern = aw_pass_kernel<V, Tile, S::NT>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return -3;
  }
  dim3 grid(a->nrows / S::L, batch);
  kern<<<grid, S::NT, smem, st>>>(*a);
  return cudaGetLastError() == cudaSuccess ? 0 : -4;
}

template <typename V, int N>
static int launch_col_n(const AwPassArgs* a, int batch, cudaStream_t st) {
  typedef typename PassShape<V>::template Col<N> S;
  typedef ColTile<N, S::B> Tile;
  if (a->ncols % S::B) return -2;
  const size_t smem = sizeof(V) * S::TILE;
  auto kern = aw_pass_kernel<V, Tile, S::NT>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return -3;
  }
  dim3 grid(a->ncols / S::B, batch);
  kern<<<grid, S::NT, smem, st>>>(*a);
  return cudaGetLastError() == cudaSuccess ? 0 : -4;
}

template <typename V> static int launch_row(const AwPassArgs* a, int batch, cudaStream_t st) {
  switch (a->ncols) {
    case 64: return launch_row_n<V, 64>(a, batch, st);
    case 128: return launch_row_n<V, 128>(a, batch, st);
    case 256: return launch_row_n<V, 256>(a, batch, st);
    case 512: return launch_row_n<V, 512>(a, batch, st);
    case 1024: return launch_row_n<V, 1024>(a, batch, st);
    case 2048: return launch_row_n<V, 2048>(a, batch, st);
    case 4096: return launch_row_n<V, 4096>(a, batch, st);
    case 8192: return launch_row_n<V, 8192>(a, batch, st);
    default: return -1;
  }
}

template <typename V> static int launch_col(const AwPassArgs* a, int batch, cudaStream_t st) {
  switch (a->nrows) {
    case 64: return launch_col_n<V, 64>(a, batch, st);
    case 128: return launch_col_n<V, 128>(a, batch, st);
    case 256: return launch_col_n<V, 256>(a, batch, st);
    case 512: return launch_col_n<V, 512>(a, batch, st);
    case 1024: return launch_col_n<V, 1024>(a, batch, st);
    case 2048: return launch_col_n<V, 2048>(a, batch, st);
    case 4096: return launch_col_n<V, 4096>(a, batch, st);
    case 8192: return launch_col_n<V, 8192>(a, batch, st);
    default: return -1;
  }
}

template <typename V> static int row_lines(int ncols) {
  switch (ncols) {
#define AW_RL(NN) \
  case NN: return PassShape<V>::template Row<NN>::L;
    AW_RL(64) AW_RL(128) AW_RL(256) AW_RL(512) AW_RL(1024) AW_RL(2048) AW_RL(4096) AW_RL(8192)
#undef AW_RL
    default: return -1;
  }
}

template <typename V> static int col_blocks(int nrows, int ncols) {
  switch (nrows) {
#define AW_CB(NN) \
  case NN: return ncols / PassShape<V>::template Col<NN>::B;
    AW_CB(64) AW_CB(128) AW_CB(256) AW_CB(512) AW_CB(1024) AW_CB(2048) AW_CB(4096) AW_CB(8192)
#undef AW_CB
    default: return -1;
  }
}
