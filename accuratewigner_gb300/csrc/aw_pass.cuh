// Fused FFT pass kernels for sm_103a.  See aw_pass.h for the pass program.
//
// A row pass owns L whole rows of the grid (contiguous in HBM); a column pass
// owns a slab of B whole columns (B * element size >= 64-128 bytes per grid row,
// so every row segment is a full set of DRAM sectors).  Each pass reads its
// tile from HBM once, keeps it in shared memory for every FFT, phase multiply
// and reduction of its program, and writes it once.
#pragma once
#include <cooperative_groups.h>
#include <cudaTypedefs.h>

#include <atomic>
#include <type_traits>

#include "aw_common.cuh"
#include "aw_fft.cuh"
#include "aw_pass.h"
#include "aw_tma.cuh"

namespace cg = cooperative_groups;

// Tile shapes.  A row tile holds LINES whole rows, a column tile a slab of
// LINES whole columns; a thread keeps E elements (8, more for tiles above
// 4096 elements so that a block stays at or below 512 threads and 128
// registers a thread).  The number of lines per tile is chosen at run time
// (aw_row_pass_lines / aw_col_pass_lines) so that a launch spreads over all
// 152 SMs; column tiles hold at most 4096 elements.
// A double-float row of 1024 elements is spread over 256 threads of 4 elements (radix-4 stages, 64
// registers, 4 blocks a SM): more warps for the latency-bound row pass, whose branch point keeps a
// second copy of the elements in registers (measured: 0.174 -> 0.170 ms a step; tiles of several
// shorter rows spill at 64 registers and keep 8 elements a thread).
// Complex64 tiles of 4096 elements and more keep 16 elements a thread (two radix-8 butterflies a thread
// a stage, half the threads): 4096^2 von Neumann 0.608 -> 0.573 ms a step.  Smaller tiles keep 8, so
// that their other shape (4 elements, radix-4 stages) exists at every column width: a width then
// never changes the radix a grid's tuned shape sets.
// ALT: the other number of elements a thread (4 where the rule above gives 8, 8 where it gives 4), so
// the other FFT radix (stages of radix min(8, E)); offered to the autotuner for lines of 256 to 2048
// points where the block stays within 512 threads (ALT_OK).
template <typename V, int N, int LINES, bool ROW = false, bool ALT = false> struct Shape {
  static constexpr int TILE = N * LINES;
  static constexpr int E0 = (ROW && std::is_same<V, dfc>::value && N == 1024 && LINES == 1) ? 4
                            : ((std::is_same<V, float2>::value && TILE >= 4096) ? (TILE / 512 > 16 ? TILE / 512 : 16)
                                                                                  : (TILE / 512 > 8 ? TILE / 512 : 8));
  static constexpr int E1 = E0 == 4 ? 8 : (E0 == 8 ? 4 : E0);
  static constexpr bool ALT_OK = N >= 256 && N <= 2048 && E1 != E0 && TILE / E1 <= 512 && TILE % E1 == 0;
  static constexpr int E = ALT ? E1 : E0;
  static constexpr int NT = TILE / E;
  // the tile fits the 128 KB a block is given: rows are padded by one element when LINES > 1
  static constexpr bool FITS_ROW = (LINES > 1 ? (N + 1) * LINES : N) * (int)sizeof(V) <= 128 * 1024;
  // column tiles above 4096 elements keep 16 (complex64: 8-byte) elements a thread; the 16-byte types
  // hold a single column there
  static constexpr bool FITS_COL = N * LINES * (int)sizeof(V) <= 128 * 1024 &&
                                   (N * LINES <= 4096 || LINES == 1 || (sizeof(V) == 8 && N * LINES <= 8192));
};

template <typename V> struct RealOf;
template <> struct RealOf<double2> { typedef double type; };
template <> struct RealOf<float2> { typedef float type; };
template <> struct RealOf<dfc> { typedef dfr type; };

// The thread's own elements (see aw_fft.cuh): line tid % LINES, positions pos0 + k * STEP.
template <class Tile, int NT> struct Own {
  static constexpr int E = Tile::N * Tile::LINES / NT;
  static constexpr int STEP = Tile::N / E;
};

// global index of the element at (global line lg, position pos)
template <class Tile>
__device__ __forceinline__ long long gidx(int lg, int pos, int ncols) {
  return Tile::IS_ROW ? (long long)lg * ncols + pos : (long long)pos * ncols + lg;
}

// apply one AwFactor to the thread's own elements
template <typename V, class Tile, int NT>
__device__ __forceinline__ void apply_factor(V* r, const AwFactor& f, int lg, int pos0, int nrows, int ncols,
                                             long long tab_off, long long elem_off, int inst) {
  typedef typename RealOf<V>::type T;
  constexpr int E = Own<Tile, NT>::E;
  constexpr int STEP = Own<Tile, NT>::STEP;
  const V* ct = (const V*)f.col_tab;
  const V* rt = (const V*)f.row_tab;
  const T* mk = (const T*)f.mask;
  const V* sh = (const V*)f.sh_hi;
  const V* sl = (const V*)f.sh_lo;
  if (ct) ct += tab_off;
  if (rt) rt += tab_off;
  if (mk) mk += elem_off;
  // every factor that depends only on the line, folded into one complex constant:
  //   row tile: conj(row_tab[line]) * scale,  column tile: col_tab[line] * scale
  // (the FP64 scale is converted only when there is one: conversions run at the FP64 rate)
  const V* lt = f.lin ? nullptr : (Tile::IS_ROW ? rt : ct);
  const bool scaled = f.scale_ptr || f.scale != 1.0;
  V c;
  if (scaled) {
    double scr = f.scale, sci = 0.0;
    if (f.scale_ptr) {
      scr = f.scale * f.scale_ptr[2 * inst];
      sci = f.scale * f.scale_ptr[2 * inst + 1];
    }
    c = cmake<V>(from_double<T>(scr), from_double<T>(sci));
    if (lt) c = Tile::IS_ROW ? cmulc(c, lt[lg]) : cmul(c, lt[lg]);
  } else if (lt) {
    c = Tile::IS_ROW ? cconj_if(lt[lg], 0x80000000u) : lt[lg];
  }
  const bool have_c = lt || scaled;
  const V* et = f.lin ? nullptr : (Tile::IS_ROW ? ct : rt);  // table along the line
  const int lo_n = f.sh_lo_n;
  const int nhi = lo_n ? Tile::N / lo_n : 0;
  const int sgn = f.sign;
  // One uniform branch around each component's loop over the thread's elements (the same operations
  // in the same order as an element-by-element chain, so the same bits): tested inside the element
  // loop, the optional products were compiled as predicated instructions, and FP64 instructions
  // whose predicate is off still occupy GB300's FP64 pipe (16 cycles a warp instruction).  Measured on
  // the headline's passes: 24-30 of 32 lanes active per FP64 instruction before.
  if (sgn) {
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int pos = pos0 + k * STEP;
      const int i = Tile::IS_ROW ? lg : pos;
      const int j = Tile::IS_ROW ? pos : lg;
      r[k] = cflip(r[k], ((sgn == 1 ? i + j : (sgn == 2 ? i : j)) & 1) ? 0x80000000u : 0u);
    }
  }
  if (mk) {
    const bool sq = f.mask_pow == 2;
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int pos = pos0 + k * STEP;
      const int i = Tile::IS_ROW ? lg : pos;
      const int j = Tile::IS_ROW ? pos : lg;
      T q = mk[(long long)i * ncols + j];
      if (sq) q = q * q;
      r[k] = cscale(r[k], q);
    }
  }
  if (et) {
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int pos = pos0 + k * STEP;
      r[k] = Tile::IS_ROW ? cmul_l(r[k], et[pos]) : cmulc_l(r[k], et[pos]);
    }
  }
  if (f.lin) {
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int pos = pos0 + k * STEP;
      const int i = Tile::IS_ROW ? lg : pos;
      const int j = Tile::IS_ROW ? pos : lg;
      r[k] = cmul_l(r[k], ct[f.lin == 1 ? (long long)i * ncols + j : i + (long long)nrows * j]);
    }
  }
  if (have_c) {
#pragma unroll
    for (int k = 0; k < E; ++k) r[k] = cmul_l(r[k], c);
  }
  if (f.sh_full) {
    const V* sf = (const V*)f.sh_full + (long long)lg * Tile::N;
#pragma unroll
    for (int k = 0; k < E; ++k) r[k] = cmul_l(r[k], sf[(pos0 + k * STEP + f.sh_roll) & (Tile::N - 1)]);
  } else if (lo_n) {
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int q = (pos0 + k * STEP + f.sh_roll) & (Tile::N - 1);
      const V w = cmul_l(sh[(long long)lg * nhi + q / lo_n], sl[(long long)lg * lo_n + (q % lo_n)]);
      r[k] = cmul_l(r[k], w);
    }
  }
#pragma unroll
  for (int k = 0; k < E; ++k) r[k] = cnorm(r[k]);
}

template <class Tile, int NT, typename V>
__device__ __forceinline__ void run_fft(V* r, V* s, const AwPassArgs& a, int dir, int tid) {
  if (dir == 0) return;
  tile_fft_regs<Tile, NT, V>(r, s, (const V*)a.tw, tid, dir > 0 ? 0u : 0x80000000u, (const double2*)a.twt_mq,
                             a.twt_e);
}

template <typename V, class Tile, int NT>
__device__ __forceinline__ void store_regs(V* __restrict__ dst, const V* r, int lg, int pos0, int ncols, bool sgn) {
  constexpr int E = Own<Tile, NT>::E;
  constexpr int STEP = Own<Tile, NT>::STEP;
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const int pos = pos0 + k * STEP;
    V v = r[k];
    if (sgn) v = cflip(v, ((lg + pos) & 1) ? 0x80000000u : 0u);
    dst[gidx<Tile>(lg, pos, ncols)] = v;
  }
}

// the branch store of a row tile rotated: element (lg, pos) to (lg, (pos - lg) mod N), times (-1)^lg
template <typename V, class Tile, int NT>
__device__ __forceinline__ void store_regs_rot(V* __restrict__ dst, const V* r, int lg, int pos0, int ncols) {
  constexpr int E = Own<Tile, NT>::E;
  constexpr int STEP = Own<Tile, NT>::STEP;
  static_assert(Tile::IS_ROW, "rotated stores are row-tile stores");
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const int pos = pos0 + k * STEP;
    V v = r[k];
    if (lg & 1) v = cflip(v, 0x80000000u);
    dst[(long long)lg * ncols + ((pos - lg) & (Tile::N - 1))] = v;
  }
}

// deterministic block sum of one double per thread (NT a power of two); result valid in thread 0:
// a fixed shuffle tree inside each warp, then the warp sums in index order (two barriers instead of
// one per halving)
template <int NT>
__device__ __forceinline__ double block_sum(double x, double* red, int tid) {
  constexpr int W = NT < 32 ? NT : 32;
#pragma unroll
  for (int o = W / 2; o > 0; o >>= 1) x += __shfl_down_sync(lane_mask<NT>(), x, o, W);
  if constexpr (NT <= 32) {
    return x;
  } else {
    if ((tid & 31) == 0) red[tid >> 5] = x;
    __syncthreads();
    double out = 0.0;
    if (tid == 0)
#pragma unroll
      for (int w = 0; w < NT / 32; ++w) out += red[w];
    __syncthreads();
    return out;
  }
}

// Register budget: 5 blocks of 128 threads (96 registers a thread) or 2 blocks of 256 per SM, and 4
// blocks of 256 (64 registers) for 4 elements a thread.  The double-float passes are latency-bound
// and the occupancy gained beats the few spills (measured on the 1024-point passes: 4 blocks of 128
// threads 0.180 ms a step, 5 blocks 0.174, 6 blocks 0.183).  Complex64 passes over lines of 512 points
// and more with at most 8 elements a thread get 64 registers (1024 threads a SM; no spills in the main
// passes): the 1024^2 Wigner-Moyal step 0.088 -> 0.074 ms, 4096^2 von Neumann 1.43 -> 1.26 ms, the
// 64 x 512^2 Gibbs batch +16 %; at 256 points it lost 5 %.
// REDUCE_ONLY: the reduction-only column pass (load, FFT d1, f1, column reductions, nothing stored),
// compiled without the segment loop so that its code is a fraction of the full pass's; it needs
// fewer registers and runs 3 blocks of 256 threads a SM (0.1555 -> 0.1537 ms a step).
// TMA: (column tiles) the tile arrives in shared memory by tensor copies and `out` leaves it the same
// way (aw_tma.cuh); everything between is the register-resident program of the direct form, so the
// two forms give bit-identical results.
// LEAN: (grouped launches) compiled without the branch segments, the mid-point and |v|^2 outputs and the
// column reductions, which a grouped pass never asks for (the host refuses them): six tile lengths of
// the full program in one kernel spill 700-800 bytes a thread, the lean ones 0-90.
// The pass program on the tile of logical block (bx, by) of a launch of gx x ... blocks; the kernel
// below runs it for its own block, the grouped kernel (aw_group.cuh) for the work items it walks.
template <typename V, class Tile, int NT, bool REDUCE_ONLY = false, bool TMA = false, bool LEAN = false>
__device__ __forceinline__ void aw_pass_body(const AwPassArgs& a, const int bx, const int by, const int gx,
                                             unsigned char* aw_smem) {
  typedef typename RealOf<V>::type T;
  V* s = reinterpret_cast<V*>(aw_smem);
  constexpr int L = Tile::LINES;
  constexpr int E = Own<Tile, NT>::E;
  constexpr int STEP = Own<Tile, NT>::STEP;
  __shared__ double red[NT];
  const int inst = by + a.inst0;
  if (a.stop && a.stop[inst]) return;
  const int tid = threadIdx.x;
  const int line = tid % L;
  const int pos0 = tid / L;
  const int line0 = bx * L;
  const int lg = line0 + line;
  const int ncols = a.ncols;
  const long long eoff = (long long)inst * a.batch_elems;
  const long long toff = (long long)inst * a.batch_tab;
  const V* in = (const V*)a.in + eoff;

  // TMA geometry: 8-byte words per element, rows per box, boxes per tile; tensor row of this
  // instance's row 0 (the instances of the launch are stacked rows of one tensor)
  constexpr int TW = sizeof(V) / 8;
  constexpr int TR = Tile::N < 256 ? Tile::N : 256;
  constexpr int TBOX = Tile::N / TR;
  const int ty0 = a.batch_elems ? inst * a.nrows : 0;

  V r[E];
  if constexpr (TMA && !Tile::IS_ROW) {
    __shared__ __align__(8) uint64_t tma_bar;
    // box destinations must be 128-byte aligned: a block whose tile is not records it and copies nothing
    if (aw_smem_addr(s) & 127) {
      if (tid == 0 && a.err) atomicExch(a.err, AW_TMA_MISALIGNED);
      return;
    }
    if (tid == 0) {
      aw_mbar_init(&tma_bar, 1);
      aw_fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0) {
      aw_mbar_arrive_expect_tx(&tma_bar, (uint32_t)(sizeof(V) * Tile::SMEM_ELEMS));
#pragma unroll 1
      for (int b = 0; b < TBOX; ++b) aw_tma_load_2d(s + b * TR * L, a.tmap_in, line0 * TW, ty0 + b * TR, &tma_bar);
    }
    if (!__syncthreads_and(aw_mbar_wait(&tma_bar, 0))) {
      // the copies did not arrive in time: record it, give them a second bounded wait (they write into
      // this block's shared memory) and leave
      if (tid == 0 && a.err) atomicExch(a.err, AW_TMA_TIMEOUT);
      aw_mbar_wait(&tma_bar, 0);
      return;
    }
#pragma unroll
    for (int k = 0; k < E; ++k) r[k] = s[Tile::addr(line, pos0 + k * STEP)];
  } else {
#pragma unroll
    for (int k = 0; k < E; ++k) r[k] = in[gidx<Tile>(lg, pos0 + k * STEP, ncols)];
  }

  if constexpr (REDUCE_ONLY) {
    run_fft<Tile, NT>(r, s, a, a.d1, tid);
    if (a.f1.active) apply_factor<V, Tile, NT>(r, a.f1, lg, pos0, a.nrows, ncols, toff, eoff, inst);
  } else {
  // The pass as a loop over FFT segments, so that the kernel holds one copy of the FFT and of
  // the factor code:
  //   0: f0, FFT d1, f1        then mid_out, diag_out, red_abs2 (start)
  //   1: keep, FFT br_d1, fbr  (branch, with br_out)
  //   2: FFT br_d2, store br_out, restore
  //   3: f2, FFT d2, f3
  V keep[E];
#pragma unroll 1
  for (int seg = 0; seg < 4; ++seg) {
    // column passes never branch (the host refuses it), so their kernels carry no branch code
    if ((seg == 1 || seg == 2) && (LEAN || !Tile::IS_ROW || !a.br_out)) continue;
    if (seg == 1) {
#pragma unroll
      for (int k = 0; k < E; ++k) keep[k] = r[k];
    }
    const AwFactor* pre = seg == 0 ? &a.f0 : (seg == 3 ? &a.f2 : nullptr);
    const AwFactor* post = seg == 0 ? &a.f1 : (seg == 1 ? &a.fbr : (seg == 3 ? &a.f3 : nullptr));
    const int dir = seg == 0 ? a.d1 : (seg == 1 ? a.br_d1 : (seg == 2 ? a.br_d2 : a.d2));
    if (pre && pre->active) apply_factor<V, Tile, NT>(r, *pre, lg, pos0, a.nrows, ncols, toff, eoff, inst);
    run_fft<Tile, NT>(r, s, a, dir, tid);
    if (post && post->active) apply_factor<V, Tile, NT>(r, *post, lg, pos0, a.nrows, ncols, toff, eoff, inst);
    if (seg == 0) {
      if (!LEAN && Tile::IS_ROW && a.mid_out) store_regs<V, Tile, NT>((V*)a.mid_out + eoff, r, lg, pos0, ncols, a.mid_sign != 0);
      if (Tile::IS_ROW && a.diag_out) {
        // the element (lg, lg), when this thread holds it: picked by selects, then one conversion
        // under a real branch (per-element conditional conversions were predicated FP64 work)
        const int kd = (lg - pos0) / STEP;
        if (lg >= pos0 && (lg - pos0) % STEP == 0 && kd < E) {
          V d = r[0];
#pragma unroll
          for (int k = 1; k < E; ++k) d = k == kd ? r[k] : d;
          a.diag_out[(long long)inst * a.nrows + lg] = make_double2(to_d(cre(d)), to_d(cim(d)));
        }
      }
      if (!LEAN && a.red_abs2 && !a.abs2_end) {
        T acc = from_double<T>(0.0);
#pragma unroll
        for (int k = 0; k < E; ++k) acc += cabs2(r[k]);
        const double tot = block_sum<NT>(to_d(acc), red, tid);
        if (tid == 0) a.red_abs2[(long long)inst * gx + bx] = tot;
      }
    }
    if (seg == 2) {
      if constexpr (Tile::IS_ROW) {
        if (a.br_rot)
          store_regs_rot<V, Tile, NT>((V*)a.br_out + eoff, r, lg, pos0, ncols);
        else
          store_regs<V, Tile, NT>((V*)a.br_out + eoff, r, lg, pos0, ncols, false);
      }
#pragma unroll
      for (int k = 0; k < E; ++k) r[k] = keep[k];
    }
  }
  if (a.out) {
    if constexpr (TMA && !Tile::IS_ROW) {
      __syncthreads();  // every thread has read the tile's last FFT stage
#pragma unroll
      for (int k = 0; k < E; ++k) s[Tile::addr(line, pos0 + k * STEP)] = r[k];
      aw_fence_proxy_async_smem();
      __syncthreads();
      if (tid == 0) {
#pragma unroll 1
        for (int b = 0; b < TBOX; ++b) aw_tma_store_2d(a.tmap_out, line0 * TW, ty0 + b * TR, s + b * TR * L);
        aw_bulk_commit();
        aw_bulk_wait_read();  // the block's shared memory stays until the copies have read it
      }
    } else {
      store_regs<V, Tile, NT>((V*)a.out + eoff, r, lg, pos0, ncols, false);
    }
  }
  if (!LEAN && a.red_abs2 && a.abs2_end) {
    T acc = from_double<T>(0.0);
#pragma unroll
    for (int k = 0; k < E; ++k) acc += cabs2(r[k]);
    const double tot = block_sum<NT>(to_d(acc), red, tid);
    if (tid == 0) a.red_abs2[(long long)inst * gx + bx] = tot;
  }
  }

  if constexpr (!Tile::IS_ROW && !LEAN) {
    constexpr int B = L;
    // per-thread partials over the thread's E elements of its column (working precision), then
    // FP64 across threads in a fixed order
    if (a.col_alt || a.alt_cross) {
      __shared__ typename cpart<V>::type cred[NT];
      // each reduction in its own loop under one uniform branch (no predicated arithmetic, see
      // apply_factor); every accumulator adds its terms in the same order as before
      T cr = from_double<T>(0.0), ci = from_double<T>(0.0);
      if (a.col_alt) {
#pragma unroll
        for (int k = 0; k < E; ++k) {
          // (-1)^pos by a sign-bit flip, not a branch: pos differs across the lanes of a warp
          const unsigned sp = ((pos0 + k * STEP) & 1) ? 0x80000000u : 0u;
          cr += flip(cre(r[k]), sp);
          ci += flip(cim(r[k]), sp);
        }
      }
      if (a.alt_cross) {
        // across the block's B columns in working precision (B <= 16 terms), FP64 beyond
        const unsigned sl = (lg & 1) ? 0x80000000u : 0u;
#pragma unroll
        for (int k = 0; k < E; ++k) {
          const int pos = pos0 + k * STEP;
          T xr = flip(cre(r[k]), sl), xi = flip(cim(r[k]), sl);
#pragma unroll
          for (int o = B / 2; o > 0; o >>= 1) {
            xr += shfl_xor(lane_mask<NT>(), xr, o, B);
            xi += shfl_xor(lane_mask<NT>(), xi, o, B);
          }
          if (line == 0) {
            if (a.cluster > 1)
              reinterpret_cast<typename cpart<V>::type*>(aw_smem + sizeof(V) * Tile::SMEM_ELEMS)[pos] =
                  cpart<V>::make(xr, xi);
            else
              a.alt_cross[((long long)inst * gx + bx) * a.nrows + pos] = make_double2(to_d(xr), to_d(xi));
          }
        }
      }
      if (a.col_alt) {
        // the lanes of one column in a warp (equal lane mod B) by a fixed shuffle tree, then the
        // warps in index order
        constexpr int W = NT < 32 ? NT : 32;
        typename cpart<V>::type acc = cpart<V>::make(cr, ci);
#pragma unroll
        for (int o = W / 2; o >= B; o >>= 1) acc = cpart<V>::add(acc, cpart<V>::shfl_xor(lane_mask<NT>(), acc, o, W));
        if ((tid % W) < B) cred[(tid / W) * B + (tid % W)] = acc;
        __syncthreads();
        if (tid < B) {
          typename cpart<V>::type sum = cpart<V>::zero();
          for (int w = 0; w < NT / W; ++w) sum = cpart<V>::add(sum, cred[w * B + tid]);
          a.col_alt[(long long)inst * ncols + line0 + tid] = cpart<V>::to_d2(sum);
        }
        __syncthreads();
      }
      if (a.alt_cross && a.cluster > 1) {
        // sum the cluster's per-block row partials through distributed shared memory, rank order
        cg::cluster_group cl = cg::this_cluster();
        cl.sync();
        const int rank = (int)cl.block_rank();
        const int ncl = (int)cl.num_blocks();
        const int n = a.nrows;
        const int lo = rank * (n / ncl), hi = lo + n / ncl;
        typedef typename cpart<V>::type P;
        P* mine = reinterpret_cast<P*>(aw_smem + sizeof(V) * Tile::SMEM_ELEMS);
        for (int k = lo + tid; k < hi; k += NT) {
          P acc = cpart<V>::zero();
          for (int q = 0; q < ncl; ++q) acc = cpart<V>::add(acc, cl.map_shared_rank(mine, q)[k]);
          a.alt_cross[((long long)inst * (gx / ncl) + bx / ncl) * n + k] = cpart<V>::to_d2(acc);
        }
        cl.sync();
      }
    }
    if (a.red_line || a.red_cross || a.red_sq) {
      typedef typename acc_of<V>::type A;
      A lsum = to_acc<A>(0.0), sq = to_acc<A>(0.0);
      if (a.red_line) {
#pragma unroll
        for (int k = 0; k < E; ++k) lsum += to_acc<A>(cre(r[k]));
      }
      if (a.red_sq) {
#pragma unroll
        for (int k = 0; k < E; ++k) {
          const A re = to_acc<A>(cre(r[k])), im = to_acc<A>(cim(r[k]));
          sq += re * re - im * im;
        }
      }
      if (a.red_cross) {
#pragma unroll
        for (int k = 0; k < E; ++k) {
          // across the block's B columns: FP32 for complex64 (B <= 16 terms), FP64 otherwise
          const A re = to_acc<A>(cre(r[k]));
          typedef typename std::conditional<std::is_same<A, float>::value, float, double>::type C;
          C c;
          if constexpr (std::is_same<C, float>::value) c = re; else c = to_d(re);
#pragma unroll
          for (int o = B / 2; o > 0; o >>= 1) c += shfl_xor(lane_mask<NT>(), c, o, B);
          if (line == 0) a.red_cross[((long long)inst * gx + bx) * a.nrows + pos0 + k * STEP] = (double)c;
        }
      }
      if (a.red_line) {
        // as the marginal sums: shuffle tree over a column's lanes, then the warps in order
        constexpr int W = NT < 32 ? NT : 32;
        double acc = to_d(lsum);
#pragma unroll
        for (int o = W / 2; o >= B; o >>= 1) acc += __shfl_xor_sync(lane_mask<NT>(), acc, o, W);
        if ((tid % W) < B) red[(tid / W) * B + (tid % W)] = acc;
        __syncthreads();
        if (tid < B) {
          double sum = 0.0;
          for (int w = 0; w < NT / W; ++w) sum += red[w * B + tid];
          a.red_line[(long long)inst * ncols + line0 + tid] = sum;
        }
        __syncthreads();
      }
      if (a.red_sq) {
        const double tot = block_sum<NT>(to_d(sq), red, tid);
        if (tid == 0) a.red_sq[(long long)inst * gx + bx] = tot;
      }
    }
  }
}

template <typename V, class Tile, int NT, bool REDUCE_ONLY = false, bool TMA = false>
__global__ void __launch_bounds__(NT, (std::is_same<V, float2>::value && Tile::N >= 512 && NT >= 64 &&
                                       (Own<Tile, NT>::E <= 8 || TMA || REDUCE_ONLY)) ? 1024 / NT
                                      : (Own<Tile, NT>::E == 4 ? (NT <= 256 ? 4 : 1)
                                                              : (NT <= 128 ? 5 : (NT <= 256 ? (REDUCE_ONLY ? 3 : 2) : 1))))
    aw_pass_kernel(const __grid_constant__ AwPassArgs a) {
  extern __shared__ __align__(128) unsigned char aw_smem[];
  aw_pass_body<V, Tile, NT, REDUCE_ONLY, TMA>(a, blockIdx.x, blockIdx.y, gridDim.x, aw_smem);
}


// ------------------------------------------------------------------ dispatch
// Grids are sized by the SM count of the device the launch goes to (aw_sm_count, aw_common.cuh).

// rows per row-pass block: tiles of about 1024 elements
inline int choose_row_lines(int ncols, int esz) {
  int l = 1024 / ncols;
  if (l < 1) l = 1;
  return l;
}

// rows per row-pass block for a grid of nrows rows: tiles of about 1024 elements, or one row a
// block when that would leave fewer than two blocks per SM (small grids; not the zero-padded tile
// of a wave function, whose nrows equals the tile)
inline int choose_row_lines(int nrows, int ncols, int esz) {
  const int l = choose_row_lines(ncols, esz);
  return (l > 1 && nrows > l && nrows / l < 2 * aw_sm_count()) ? 1 : l;
}

// columns per column-pass block: as many as fit (<= 16, <= 128 KB of shared memory, <= 512
// threads so that the 16-byte element types keep their registers)
inline int max_col_lines(int nrows, int ncols, int esz) {
  int b = 16;
  const long long most = esz == 8 ? 8192 : 4096;  // elements of a tile (Shape::FITS_COL)
  while (b > 1 && ((long long)nrows * b * esz > 128 * 1024 || (long long)nrows * b > most || ncols % b))
    b >>= 1;
  return b;
}

inline int choose_col_lines(int nrows, int ncols, int batch, int esz) {
  // as many columns as fit while the launch keeps at least 4 blocks per SM
  int b = max_col_lines(nrows, ncols, esz);
  while (b > 1 && (long long)(ncols / b) * batch < 4 * aw_sm_count()) b >>= 1;
  return b;
}

// Opt a kernel in to the dynamic shared memory its launches can ask for (tile plus, for a clustered
// column pass, one row of FP64 partials), within the 227 KB per block of sm_103a.  The attribute
// belongs to the device that is current, so it is set once per device: `slots` is the kernel's own
// per-device record of the size granted (0: not yet set).
template <typename K>
static int prepare_smem(K kern, size_t max_dynamic, std::atomic<int>* slots) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= AW_MAX_DEVICES) return -3;
  const int have = slots[dev].load(std::memory_order_acquire);
  if (have > 0) return have;
  cudaFuncAttributes fa;
  if (cudaFuncGetAttributes(&fa, kern) != cudaSuccess) return -3;
  const size_t cap = 227 * 1024 - fa.sharedSizeBytes;
  const size_t want = max_dynamic < cap ? max_dynamic : cap;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)want) != cudaSuccess) return -3;
  slots[dev].store((int)want, std::memory_order_release);
  return (int)want;
}

template <typename V, int N, int LINES, bool ALT = false>
static int launch_row_t(const AwPassArgs* a, int batch, cudaStream_t st) {
  typedef Shape<V, N, LINES, true, ALT> S;
  if constexpr (!S::FITS_ROW || (ALT && !S::ALT_OK)) {
    return ALT ? -9 : -5;
  } else {
    typedef RowTile<N, LINES> Tile;
    if (a->nrows % LINES) return -2;
    const size_t smem = sizeof(V) * Tile::SMEM_ELEMS;
    auto kern = aw_pass_kernel<V, Tile, S::NT>;
    static std::atomic<int> granted[AW_MAX_DEVICES];
    if (prepare_smem(kern, smem, granted) < (int)smem) return -3;
    dim3 grid(a->nrows / LINES, batch);
    kern<<<grid, S::NT, smem, st>>>(*a);
    return cudaGetLastError() == cudaSuccess ? 0 : -4;
  }
}

// cuTensorMapEncodeTiled from the driver, looked up once through the runtime
static PFN_cuTensorMapEncodeTiled_v12000 aw_encode_tiled() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = []() -> PFN_cuTensorMapEncodeTiled_v12000 {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return nullptr;
    return (PFN_cuTensorMapEncodeTiled_v12000)p;
  }();
  return fn;
}

// Tensor map of a column slab source or destination: `rows` rows (every instance of the launch,
// stacked) of ncols elements of esz bytes, seen as 8-byte words; boxes of `lines` columns by `box_rows`
// rows.  0 on success.
static int aw_column_tmap(void* map, const void* base, int ncols, long long rows, int esz, int lines, int box_rows) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = aw_encode_tiled();
  if (!enc) return -8;
  const cuuint64_t dim[2] = {(cuuint64_t)ncols * (esz / 8), (cuuint64_t)rows};
  const cuuint64_t stride[1] = {(cuuint64_t)ncols * esz};
  const cuuint32_t box[2] = {(cuuint32_t)(lines * esz / 8), (cuuint32_t)box_rows};
  const cuuint32_t es[2] = {1, 1};
  const CUresult r = enc((CUtensorMap*)map, CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, const_cast<void*>(base), dim, stride,
                         box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : -8;
}

// whether a column pass of LINES columns of V can be staged by TMA: every box row a multiple of 16
// bytes (so that each box starts on a 16-byte boundary), contiguous instances, 16-byte aligned
// buffers, one store target
template <typename V, int LINES>
static bool col_tma_ok(const AwPassArgs* a) {
  if ((LINES * (int)sizeof(V)) % 16 || !a->out || a->mid_out || a->br_out) return false;
  if (a->batch_elems != 0 && a->batch_elems != (long long)a->nrows * a->ncols) return false;
  if (((uintptr_t)a->in | (uintptr_t)a->out) & 15) return false;
  return true;
}

template <typename V, int N, int LINES, bool ALT = false>
static int launch_col_t(const AwPassArgs* a, int batch, cudaStream_t st) {
  typedef Shape<V, N, LINES, false, ALT> S;
  if constexpr (!S::FITS_COL || (ALT && !S::ALT_OK)) {
    return ALT ? -9 : -5;
  } else {
    // the other shape serves the storing passes only (the reduction-only and clustered passes keep
    // the rule's)
    if (ALT && (!a->out || (a->alt_cross && a->cluster > 1))) return -9;
    typedef ColTile<N, LINES> Tile;
    if (a->ncols % LINES) return -2;
    const bool clustered = a->alt_cross && a->cluster > 1;
    if (a->tma && !clustered && col_tma_ok<V, LINES>(a)) {
      // TMA-staged form of the pass (its program has no cluster reductions)
      AwPassArgs b = *a;
      const long long rows = a->batch_elems ? (long long)(a->inst0 + batch) * N : (long long)N;
      constexpr int R = N < 256 ? N : 256;
      if (aw_column_tmap(b.tmap_in, a->in, a->ncols, rows, (int)sizeof(V), LINES, R) ||
          aw_column_tmap(b.tmap_out, a->out, a->ncols, rows, (int)sizeof(V), LINES, R))
        return -8;
      const size_t smem = sizeof(V) * Tile::SMEM_ELEMS;
      auto kern = aw_pass_kernel<V, Tile, S::NT, false, true>;
      static std::atomic<int> granted_t[AW_MAX_DEVICES];
      if (prepare_smem(kern, smem, granted_t) < (int)smem) return -3;
      dim3 grid(a->ncols / LINES, batch);
      kern<<<grid, S::NT, smem, st>>>(b);
      return cudaGetLastError() == cudaSuccess ? 0 : -4;
    }
    if constexpr (ALT) {
      // the other shape: plain storing passes, unclustered
      const size_t smem = sizeof(V) * Tile::SMEM_ELEMS;
      auto kern = aw_pass_kernel<V, Tile, S::NT, false>;
      static std::atomic<int> granted_a[AW_MAX_DEVICES];
      if (prepare_smem(kern, smem, granted_a) < (int)smem) return -3;
      kern<<<dim3(a->ncols / LINES, batch), S::NT, smem, st>>>(*a);
      return cudaGetLastError() == cudaSuccess ? 0 : -4;
    } else {
    // a clustered launch keeps one row of partials (N complex FP64) behind the tile
    const size_t smem = sizeof(V) * Tile::SMEM_ELEMS + (clustered ? sizeof(double2) * N : 0);
    const bool reduce_only = !a->out && !a->mid_out && !a->br_out && !a->f0.active && !a->d2 && !a->f2.active &&
                             !a->f3.active && !a->red_abs2 && (a->col_alt || a->alt_cross || a->red_line);
    auto kern = reduce_only ? aw_pass_kernel<V, Tile, S::NT, true> : aw_pass_kernel<V, Tile, S::NT, false>;
    static std::atomic<int> granted[AW_MAX_DEVICES], granted_r[AW_MAX_DEVICES];
    const size_t most = sizeof(V) * Tile::SMEM_ELEMS + sizeof(double2) * N;
    const int max_dyn = reduce_only ? prepare_smem(aw_pass_kernel<V, Tile, S::NT, true>, most, granted_r)
                                    : prepare_smem(aw_pass_kernel<V, Tile, S::NT, false>, most, granted);
    if (max_dyn < (int)smem) return -3;
    dim3 grid(a->ncols / LINES, batch);
    if (!clustered) {
      kern<<<grid, S::NT, smem, st>>>(*a);
      return cudaGetLastError() == cudaSuccess ? 0 : -4;
    }
    if ((a->ncols / LINES) % a->cluster || N % a->cluster || a->cluster > 8) return -6;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = dim3(S::NT);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = a->cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&cfg, kern, *a);
    return e == cudaSuccess ? 0 : -4;
    }
  }
}

template <typename V, int N, bool ALT> static int launch_row_s(const AwPassArgs* a, int batch, cudaStream_t st) {
  constexpr int L = 1024 / N >= 1 ? 1024 / N : 1;
  const int l = a->row_lines ? a->row_lines : choose_row_lines(a->nrows, N, (int)sizeof(V));
  if constexpr (L > 1) {
    if (l == 1) return launch_row_t<V, N, 1, ALT>(a, batch, st);
  }
  return l == L ? launch_row_t<V, N, L, ALT>(a, batch, st) : -7;
}

template <typename V, int N> static int launch_row_n(const AwPassArgs* a, int batch, cudaStream_t st) {
  return a->shape ? launch_row_s<V, N, true>(a, batch, st) : launch_row_s<V, N, false>(a, batch, st);
}

template <typename V, int N, bool ALT> static int launch_col_s(const AwPassArgs* a, int batch, cudaStream_t st) {
  switch (a->lines_hint ? a->lines_hint : choose_col_lines(a->nrows, a->ncols, batch, (int)sizeof(V))) {
    case 1: return launch_col_t<V, N, 1, ALT>(a, batch, st);
    case 2: return launch_col_t<V, N, 2, ALT>(a, batch, st);
    case 4: return launch_col_t<V, N, 4, ALT>(a, batch, st);
    case 8: return launch_col_t<V, N, 8, ALT>(a, batch, st);
    case 16: return launch_col_t<V, N, 16, ALT>(a, batch, st);
    default: return -1;
  }
}

template <typename V, int N> static int launch_col_n(const AwPassArgs* a, int batch, cudaStream_t st) {
  return a->shape ? launch_col_s<V, N, true>(a, batch, st) : launch_col_s<V, N, false>(a, batch, st);
}

#define AW_FOR_SIZES(M) M(32) M(64) M(128) M(256) M(512) M(1024) M(2048) M(4096) M(8192)

// Per-size launchers, so that the heavier element types can spread their instantiations over
// several translation units that compile in parallel.
#define AW_SIZE_LAUNCHERS(V, TAG, NN)                                                   \
  int aw_##TAG##_row_##NN(const AwPassArgs* a, int batch, cudaStream_t st) {           \
    return launch_row_n<V, NN>(a, batch, st);                                          \
  }                                                                                    \
  int aw_##TAG##_col_##NN(const AwPassArgs* a, int batch, cudaStream_t st) {           \
    return launch_col_n<V, NN>(a, batch, st);                                          \
  }

template <typename V> static int launch_row(const AwPassArgs* a, int batch, cudaStream_t st) {
  switch (a->ncols) {
#define AW_CASE(NN) \
  case NN: return launch_row_n<V, NN>(a, batch, st);
    AW_FOR_SIZES(AW_CASE)
#undef AW_CASE
    default: return -1;
  }
}

template <typename V> static int launch_col(const AwPassArgs* a, int batch, cudaStream_t st) {
  switch (a->nrows) {
#define AW_CASE(NN) \
  case NN: return launch_col_n<V, NN>(a, batch, st);
    AW_FOR_SIZES(AW_CASE)
#undef AW_CASE
    default: return -1;
  }
}
