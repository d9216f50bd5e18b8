// Shared-memory staging of a row group's neighbour records (the halos of EllView): used by
// the staged variants of the gathers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

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

// L2 eviction-priority hints (createpolicy + .L2::cache_hint): evict_first for the streamed
// operator arrays, read once per launch, and evict_last for the intermediates a gather
// writes for the next one (t, q, the partial du), so that the stream does not push the
// intermediates out of L2 before they are read back.
static __device__ __forceinline__ uint64_t l2_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;\n" : "=l"(p));
  return p;
}
static __device__ __forceinline__ uint64_t l2_evict_last() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;\n" : "=l"(p));
  return p;
}
static __device__ __forceinline__ float2 ldg_hint(const float2* ptr, uint64_t pol) {
  float2 v;
  asm("ld.global.nc.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;\n"
      : "=f"(v.x), "=f"(v.y)
      : "l"(ptr), "l"(pol));
  return v;
}
static __device__ __forceinline__ int ldg_hint(const uint16_t* ptr, uint64_t pol) {
  unsigned short v;
  asm("ld.global.nc.L2::cache_hint.u16 %0, [%1], %2;\n" : "=h"(v) : "l"(ptr), "l"(pol));
  return (int)v;
}
static __device__ __forceinline__ void st_hint(float4* ptr, float4 v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.v4.f32 [%0], {%1, %2, %3, %4}, %5;\n"
               ::"l"(ptr), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w), "l"(pol)
               : "memory");
}
static __device__ __forceinline__ void st_hint(double2* ptr, double2 v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.v2.f64 [%0], {%1, %2}, %3;\n"
               ::"l"(ptr), "d"(v.x), "d"(v.y), "l"(pol)
               : "memory");
}

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
