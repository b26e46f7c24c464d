// Fifth-generation tensor-core helpers (sm_100a / sm_103a): tcgen05 MMA with accumulators in
// tensor memory (TMEM), TMEM allocation and loads, mbarrier waits with an iteration limit, and
// the shared-memory matrix descriptors of the no-swizzle canonical layouts.
//
// Operand layout in shared memory ("core-matrix rows"): a [rows x cols] BF16 matrix is stored
// as 8 x 8 core matrices of 128 contiguous bytes; core (r / 8, c / 8) starts at byte
//   ((r / 8) * (cols / 8) + c / 8) * 128
// and element (r, c) sits at (r % 8) * 16 + (c % 8) * 2 inside it. One such buffer serves both
// as a K-major operand (rows = M or N, cols = K) and as an MN-major operand (rows = K,
// cols = M or N) of tcgen05.mma: in both readings the core matrix is 8 rows of 16 bytes, and
// the descriptor gives the byte distance between neighbouring cores along the M/N dimension
// (stride byte offset, SBO) and along K (leading byte offset, LBO).
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

namespace ffgb {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Byte offset of element (r, c) in a core-matrix-row buffer with `cols` columns.
__host__ __device__ __forceinline__ uint32_t core_off(int r, int c, int cols) {
  return (uint32_t)((((r >> 3) * (cols >> 3) + (c >> 3)) << 7) + ((r & 7) << 4) + ((c & 7) << 1));
}

// Shared-memory descriptor, no swizzle: start address, LBO (K-direction core stride) and SBO
// (M/N-direction core stride) in bytes (multiples of 16), version field 1 (bit 46).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;  // base offset 0, LBO mode 0, swizzle none (bits 61-63 = 0)
}

// Instruction descriptor of tcgen05.mma.kind::f16: A and B both BF16 (bf16 = true) or both FP16,
// FP32 D, M x N, a_mn / b_mn: the operand is MN-major (transposed) instead of K-major.
__host__ __device__ __forceinline__ uint32_t idesc_f16kind(int M, int N, bool a_mn, bool b_mn, bool bf16) {
  const uint32_t ab = bf16 ? 1u : 0u;       // operand format: 0 = F16, 1 = BF16
  return (1u << 4)                          // D format: F32
         | (ab << 7)                        // A format
         | (ab << 10)                       // B format
         | ((a_mn ? 1u : 0u) << 15)         // A major
         | ((b_mn ? 1u : 0u) << 16)         // B major
         | ((uint32_t)(N >> 3) << 17)       // N / 8
         | ((uint32_t)(M >> 4) << 24);      // M / 16
}
__host__ __device__ __forceinline__ uint32_t idesc_bf16(int M, int N, bool a_mn, bool b_mn) {
  return idesc_f16kind(M, N, a_mn, b_mn, true);
}

// D[tmem] (+)= A[smem] * B[smem]^T, one instruction, issued by one thread (kind::f16: BF16 or FP16
// operands as the instruction descriptor says).
__device__ __forceinline__ void mma_f16kind(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate));
}

// Arrive on an mbarrier when every tcgen05.mma issued so far by this thread has completed.
__device__ __forceinline__ void mma_commit(uint32_t mbar_saddr) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar_saddr)
               : "memory");
}

// TMEM allocation by one whole warp: ncols (power of two, 32..512) columns, the base address
// written to shared memory at dst_saddr.
__device__ __forceinline__ void tmem_alloc(uint32_t dst_saddr, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_saddr), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Makes this thread's generic-proxy shared-memory writes visible to the tensor cores (async proxy).
__device__ __forceinline__ void fence_smem_to_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 32 consecutive FP32 columns of this thread's TMEM lane: warp w reads lanes 32 (w % 4) ..
// + 31; taddr = base + (lane0 << 16) + column.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void mbar_init(uint32_t mbar_saddr, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar_saddr), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Waits for the phase with the given parity to complete; gives up after max_polls polls and
// returns false (the caller reports the failure instead of hanging).
__device__ __forceinline__ bool mbar_wait(uint32_t mbar_saddr, uint32_t parity, uint32_t max_polls) {
  for (uint32_t i = 0; i < max_polls; ++i) {
    uint32_t done = 0;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(mbar_saddr), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Two floats -> packed FP16 pair (round to nearest even), low half = a.
__device__ __forceinline__ uint32_t pack2_f16(float a, float b) {
  const __half2 v = __floats2half2_rn(a, b);
  return *reinterpret_cast<const uint32_t*>(&v);
}

// Two floats -> packed BF16 pair (round to nearest even), low half = a.
__device__ __forceinline__ uint32_t pack2_bf16(float a, float b) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t*>(&v);
}

}  // namespace tc
}  // namespace ffgb
