// Tensor-memory-access (TMA) staging of column tiles for sm_103a: inline PTX for the mbarrier, the
// tiled bulk tensor copies global <-> shared memory and their fences.
//
// A column tile is a slab of B whole columns of an nrows x ncols row-major grid (element e of column
// c at smem offset e * B + c).  Seen as a 2-D tensor of 8-byte words (dimension 0: ncols * W words a
// row, W = element bytes / 8; dimension 1: the rows of every instance stacked), the slab is a stack of
// boxes of B * W words by R rows, and a box lands in shared memory exactly in the tile's layout.  One
// thread issues the box copies; the block waits on one mbarrier for their bytes.  Every wait is
// bounded: a wait that runs out records AW_TMA_TIMEOUT in the pass's error word and the block leaves
// after a second bounded wait for its copies in flight.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#define AW_TMA_TIMEOUT 1
#define AW_TMA_MISALIGNED 2
// iterations of mbarrier.try_wait before a wait gives up (each try may suspend the thread for a
// hardware-chosen interval of under a microsecond; the limit, about a second, is far beyond the few
// microseconds a tile's copies take)
#define AW_TMA_SPIN_LIMIT (1u << 22)

__device__ __forceinline__ uint32_t aw_smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void aw_mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(aw_smem_addr(bar)), "r"(count) : "memory");
}

// makes the initialised barrier visible to the asynchronous (TMA) proxy
__device__ __forceinline__ void aw_fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void aw_mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(aw_smem_addr(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool aw_mbar_try_wait(uint64_t* bar, uint32_t phase) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(aw_smem_addr(bar)), "r"(phase)
      : "memory");
  return done != 0;
}

// bounded wait for the phase `phase` of the barrier; false when the limit ran out
__device__ __forceinline__ bool aw_mbar_wait(uint64_t* bar, uint32_t phase) {
  for (uint32_t it = 0; it < AW_TMA_SPIN_LIMIT; ++it)
    if (aw_mbar_try_wait(bar, phase)) return true;
  return false;
}

// box copy global -> shared (tensor coordinates x: 8-byte words in a row, y: rows), completing
// its bytes on the barrier
__device__ __forceinline__ void aw_tma_load_2d(void* dst, const void* tmap, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          aw_smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(tmap)), "r"(x), "r"(y), "r"(aw_smem_addr(bar))
      : "memory");
}

// box copy shared -> global, in the thread's current bulk group
__device__ __forceinline__ void aw_tma_store_2d(const void* tmap, int x, int y, const void* src) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                   reinterpret_cast<uint64_t>(tmap)),
               "r"(x), "r"(y), "r"(aw_smem_addr(src))
               : "memory");
}

__device__ __forceinline__ void aw_bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }

// the bulk groups of this thread have finished reading shared memory
__device__ __forceinline__ void aw_bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }

// generic-proxy writes to shared memory made visible to the asynchronous proxy (before a TMA store)
__device__ __forceinline__ void aw_fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
