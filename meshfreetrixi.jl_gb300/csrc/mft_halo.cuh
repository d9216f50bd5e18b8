// Shared-memory staging of a row group's neighbour records (the halos of EllView): used by
// the staged variants of the gathers.
#pragma once

#include <cuda_runtime.h>

#include "mft_internal.cuh"

namespace mft {
namespace {

// 16-byte asynchronous copy global -> shared (bypasses registers), and the wait for all
// of this thread's copies.
static __device__ __forceinline__ void cp_async16(float4* smem, const float4* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
static __device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}
static __device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
// Waits until at most N of this thread's committed copy groups are still in flight.
template <int N>
static __device__ __forceinline__ void cp_async_wait_group() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Per-warp ring of the streamed arrays of a sliced-ELL gather: for slot j of the warp's
// slice, NA double-word weight arrays (32 lanes x 8 bytes = 16 chunks each) and the 16-bit
// positions (32 x 2 bytes = 4 chunks), copied into shared memory WST - 1 slots ahead of
// use, so that their DRAM latency is covered without registers.  Slot layout (float4):
// [array a: 16 chunks] x NA, then the positions.  Every lane of the warp takes part in
// every issue / wait (rows past n included: their slice exists, padded).
template <int NA, int WST>
struct WarpRing {
  static constexpr int kSlot = 16 * NA + 4;  // float4 per slot
  float4* ring;
  int64_t s0;    // first ELL element of the slice
  int m;         // slots of the slice
  int lane;
  const float2* const* arrays;
  const uint16_t* lcol;
  __device__ __forceinline__ void issue(int j) {
    if (j < m) {
      float4* dst = ring + (j % WST) * kSlot;
      const int64_t e0 = s0 + ((int64_t)j << 5);
#pragma unroll
      for (int q = lane; q < kSlot; q += 32) {
        const float4* src = q < 16 * NA
                                ? reinterpret_cast<const float4*>(arrays[q >> 4] + e0) + (q & 15)
                                : reinterpret_cast<const float4*>(lcol + e0) + (q - 16 * NA);
        cp_async16(dst + q, src);
      }
    }
    cp_async_commit();
  }
  // weight pair of array a and the position of this lane in slot j (after wait + sync)
  __device__ __forceinline__ float2 weight(int j, int a) const {
    return reinterpret_cast<const float2*>(ring + (j % WST) * kSlot)[a * 32 + lane];
  }
  __device__ __forceinline__ int pos(int j) const {
    return reinterpret_cast<const uint16_t*>(ring + (j % WST) * kSlot + 16 * NA)[lane];
  }
};

// Stages the neighbour records of this block's row group (the group's halo list) into
// shared memory: NCH 16-byte chunks per record, chunk k of list entry q at
// sm[k * ell.halo_stride + q] (chunk-major, so that lanes reading one chunk of different
// records spread over the banks).  chunk(k, c) is the address of chunk k of node c's
// record.  Consecutive threads copy consecutive chunks of one record, so each record
// arrives in whole sectors.  Returns false (nothing staged) when the group has no list.
// Every thread of the block must call it (it ends with a block barrier); the block is one
// group (blockDim.x = ell.halo_rows).
template <int NCH, typename Chunk>
__device__ __forceinline__ bool stage_halo(const EllView& ell, float4* sm, Chunk chunk) {
  const int h0 = __ldg(ell.halo_off + blockIdx.x);
  const int nh = __ldg(ell.halo_off + blockIdx.x + 1) - h0;
  if (nh <= 0) return false;  // block-uniform
  for (int q = threadIdx.x; q < nh * NCH; q += blockDim.x) {
    const int rec = q / NCH, k = q - rec * NCH;
    cp_async16(sm + k * ell.halo_stride + rec,
               chunk(k, (int64_t)__ldg(ell.halo_col + h0 + rec)));
  }
  cp_async_wait_all();
  __syncthreads();
  return true;
}

}  // namespace
}  // namespace mft
