// Grouped passes: the row (or column) passes of several propagators of different grid sizes in one
// persistent launch.  A block walks the work items blockIdx.x, blockIdx.x + gridDim.x, ...; item u
// belongs to the member m with start[m] <= u < start[m + 1] and is that member's tile
// (u - start[m]) % tiles_x of instance (u - start[m]) / tiles_x, on which the block runs the same pass
// program as the member's own launch (aw_pass_body, in its lean form).  Tiles hold AW_GROUP_TILE
// elements on AW_GROUP_NT threads of 8 (radix-8 stages) at every length: AW_GROUP_TILE / n lines.
#pragma once
#include "aw_pass.cuh"

static_assert(AW_GROUP_TILE == 8 * AW_GROUP_NT, "8 elements a thread");
static_assert(AW_GROUP_TILE >= AW_GROUP_LONGEST, "a tile holds a whole line of the longest grouped length");

template <typename V, bool ROW, int N>
__device__ __forceinline__ void aw_group_tile(const AwPassArgs& a, int bx, int by, int gx, unsigned char* smem) {
  constexpr int L = AW_GROUP_TILE / N;
  if constexpr (ROW)
    aw_pass_body<V, RowTile<N, L>, AW_GROUP_NT, false, false, true>(a, bx, by, gx, smem);
  else
    aw_pass_body<V, ColTile<N, L>, AW_GROUP_NT, false, false, true>(a, bx, by, gx, smem);
}

template <typename V, bool ROW>
__global__ void __launch_bounds__(AW_GROUP_NT, 512 / AW_GROUP_NT) aw_group_kernel(const __grid_constant__ AwGroupArgs g) {
  extern __shared__ __align__(128) unsigned char aw_smem[];
  const int total = g.start[g.count];
  for (int item = blockIdx.x; item < total; item += gridDim.x) {
    int m = 0;
    while (m + 1 < g.count && item >= g.start[m + 1]) ++m;
    const AwPassArgs& a = g.a[m];
    const int local = item - g.start[m];
    const int gx = g.tiles_x[m];
    const int bx = local % gx, by = local / gx;
    switch (ROW ? a.ncols : a.nrows) {
      case 64: aw_group_tile<V, ROW, 64>(a, bx, by, gx, aw_smem); break;
      case 128: aw_group_tile<V, ROW, 128>(a, bx, by, gx, aw_smem); break;
      case 256: aw_group_tile<V, ROW, 256>(a, bx, by, gx, aw_smem); break;
      default: break;
    }
    __syncthreads();  // the next item reuses the block's shared memory
  }
}

// dynamic shared memory of a grouped launch: the largest tile (rows of a multi-row tile are padded)
template <typename V> constexpr size_t aw_group_smem() { return sizeof(V) * (AW_GROUP_TILE + AW_GROUP_TILE / 64); }

template <typename V> static int aw_group_launch(const AwGroupArgs* g, int row, cudaStream_t st) {
  for (int m = 0; m < g->count; ++m) {
    const int n = row ? g->a[m].ncols : g->a[m].nrows;
    if (n < 64 || n > AW_GROUP_LONGEST || (n & (n - 1))) return -1;
  }
  auto kern = row ? aw_group_kernel<V, true> : aw_group_kernel<V, false>;
  const size_t smem = aw_group_smem<V>();
  static std::atomic<int> granted_r[AW_MAX_DEVICES], granted_c[AW_MAX_DEVICES];
  if (prepare_smem(kern, smem, row ? granted_r : granted_c) < (int)smem) return -3;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, AW_GROUP_NT, smem) != cudaSuccess || per_sm < 1)
    return -3;
  const int total = g->start[g->count];
  const int grid = total < per_sm * aw_sm_count() ? total : per_sm * aw_sm_count();
  if (grid < 1) return 0;
  kern<<<grid, AW_GROUP_NT, smem, st>>>(*g);
  return cudaGetLastError() == cudaSuccess ? 0 : -4;
}

#define AW_GROUP_LAUNCHER(V, TAG)                                                   \
  extern "C" int aw_launch_group_##TAG(const AwGroupArgs* g, int row, void* stream) { \
    return aw_group_launch<V>(g, row, (cudaStream_t)stream);                        \
  }
