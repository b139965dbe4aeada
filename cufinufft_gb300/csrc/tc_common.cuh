// tc_common.cuh -- 5th-generation tensor-core (tcgen05) building blocks in
// inline PTX: tensor-memory allocation, shared-memory matrix and
// instruction descriptors, the MMA, its commit to an mbarrier, and the
// accumulator read-back.  Used by the tensor-core cell-run spread.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "device_common.cuh"

namespace cfg {

// Tensor memory: `ncols` columns (a power of two >= 32) x 128 lanes of 32
// bits, allocated by one whole warp; the base address lands in *holder.
__device__ __forceinline__ void tmem_alloc(unsigned* holder, unsigned ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(holder)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(unsigned taddr, unsigned ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes made visible to the tensor core
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Shared-memory matrix descriptor, no swizzle: a K-major tile made of core
// matrices of 8 rows x 16 bytes (row stride 16 bytes), lbo bytes apart along
// K and sbo bytes apart along the rows (M or N).
__device__ __forceinline__ uint64_t umma_sdesc(const void* p, unsigned lbo, unsigned sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((smem_u32(p) >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version of sm_100 and later
  return d;                // base offset 0, layout type 0 (no swizzle)
}

// Offset (elements) of (row r, k) in such a tile of 32-bit elements, 8 K per
// core-matrix pair: core matrices 256 bytes apart along the rows, 128 along K.
__device__ __forceinline__ int umma_kmaj_off(int r, int k) {
  return (r >> 3) * 64 + (k >> 2) * 32 + (r & 7) * 4 + (k & 3);
}
constexpr unsigned kUmmaLbo = 128, kUmmaSbo = 256;

// Instruction descriptor of kind::tf32: FP32 accumulator, TF32 A and B, both
// K-major, M x N.
__host__ __device__ constexpr unsigned umma_idesc_tf32(unsigned M, unsigned N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

// D[tmem] (+)= A[smem] B[smem]^T, K = 8 TF32; one thread issues it.
__device__ __forceinline__ void umma_tf32(unsigned taddr, uint64_t adesc, uint64_t bdesc, unsigned idesc,
                                          unsigned accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(taddr),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// The MMAs issued so far by this thread arrive on `bar` when complete.
__device__ __forceinline__ void umma_commit(unsigned long long* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// 16 consecutive 32-bit columns of this warp's 32 TMEM lanes (lane = the
// warp's quadrant, 32 (warp % 4) + lane), then wait for the load.
__device__ __forceinline__ void tmem_ld16(unsigned taddr, float* out) {
  unsigned r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int c = 0; c < 16; ++c) out[c] = __uint_as_float(r[c]);
}

// TF32 split of an FP32 value: hi keeps the 19 bits the tensor core reads,
// lo = v - hi (exact); hi*hi' + hi*lo' + lo*hi' carries FP32 accuracy.
__device__ __forceinline__ void tf32_split(float v, float& hi, float& lo) {
  hi = __uint_as_float(__float_as_uint(v) & 0xffffe000u);
  lo = v - hi;
}

}  // namespace cfg
