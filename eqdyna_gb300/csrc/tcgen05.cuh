// Blackwell 5th-generation tensor-core primitives (tcgen05, sm_100a / sm_103a): tensor-memory
// allocation, shared-memory operand descriptors, the kind::f16 MMA with BF16 operands and FP32
// accumulators in tensor memory, its completion on an mbarrier, and accumulator loads.
//
// Operand layout used throughout: K-major, no swizzle, "row-group major".  The element (r, k) of an
// R x K bf16 operand lives at byte
//     kmaj_off(r, k, K) = (r / 8) * (16 K) + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2,
// i.e. 8 x 8 core matrices of 128 contiguous bytes, the K/8 core matrices of one 8-row group next
// to each other.  Its descriptor has leading-dimension offset 128 B (next core matrix along K) and
// stride-dimension offset 16 K B (next 8-row group); the K-step kk of 16 starts 256 kk bytes in.
// Both offsets are small against the operand, so the bytes one MMA can address stay inside the
// operand whichever way the two offsets are applied.
#pragma once
#include <cstdint>

#include "elem32_common.cuh"

namespace eqd {
namespace tc {

__host__ __device__ constexpr int kmaj_off(int r, int k, int K) {
  return (r >> 3) * (K * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

// Shared-memory matrix descriptor: start address, leading / stride byte offsets (16-byte units),
// the fixed version field of tcgen05 descriptors (bits 46-48 = 1), base offset 0, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(const void *p, uint32_t lbo, uint32_t sbo) {
  const uint32_t a = e32::smem_addr(p);
  return (uint64_t)((a & 0x3FFFFu) >> 4) | (uint64_t)((lbo >> 4) & 0x3FFFu) << 16 |
         (uint64_t)((sbo >> 4) & 0x3FFFu) << 32 | (uint64_t)1 << 46;
}
// Descriptor of the K-step kk of an operand with K columns in the layout above.
__device__ __forceinline__ uint64_t kmaj_desc(const void *base, int K, int kk) {
  return smem_desc(static_cast<const unsigned char *>(base) + 256 * kk, 128u, (uint32_t)(16 * K));
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), A and B both BF16 (bits
// 7-9 = 1, bits 10-12 = 1), both K-major (bits 15, 16 = 0), N / 8 in bits 17-22, M / 16 in bits
// 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// D (tensor memory) = A B^T (+ D when accumulate): A M x 16 and B N x 16 from shared memory.
// Issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         bool accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"((int)accumulate)
      : "memory");
}
// The mbarrier completes a phase when every MMA this thread issued before has completed.
__device__ __forceinline__ void commit(unsigned long long *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   e32::smem_addr(bar))
               : "memory");
}

// Tensor-memory allocation by one whole warp; the address is written to *slot (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(e32::smem_addr(slot)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Generic-proxy shared-memory writes -> visible to the tensor cores (async proxy).
__device__ __forceinline__ void fence_smem_to_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 16 consecutive FP32 columns of this thread's lane (shape 32x32b: the warp reads its 32 lanes);
// warp-collective.  taddr = base + (lane0 << 16) + column.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Bounded wait for the phase with the given parity (at most e32::kWaitLimit polls and
// e32::kWaitNs nanoseconds).
__device__ __forceinline__ bool mbar_wait_parity(unsigned long long *bar, unsigned parity) {
  const unsigned long long t0 = e32::globaltimer_ns();
  for (unsigned it = 0; it < e32::kWaitLimit; ++it) {
    if (e32::mbar_try_wait(bar, parity)) return true;
    if ((it & 63u) == 63u && e32::globaltimer_ns() - t0 > e32::kWaitNs) break;
  }
  return false;
}

// Sum of v[0..31] over the 32 lanes of the warp by halving exchanges (31 shuffles): lane l returns
// the warp's sum of column l.
__device__ __forceinline__ float warp_column_sums32(float (&v)[32]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 16, L = 32; o >= 1; o >>= 1, L >>= 1) {
    const bool upper = (lane & o) != 0;
#pragma unroll
    for (int i = 0; i < L / 2; ++i) {
      const float send = upper ? v[i] : v[i + L / 2];
      const float keep = upper ? v[i + L / 2] : v[i];
      v[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
    }
  }
  return v[0];
}

}  // namespace tc
}  // namespace eqd
