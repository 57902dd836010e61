// Fifth-generation tensor-core primitives (tcgen05, sm_100a / sm_103a) as
// inline PTX: tensor-memory allocation, single-thread MMA issue of
// kind::tf32 products with FP32 accumulation in tensor memory, completion
// through an mbarrier, and tensor-memory loads for the epilogue.
//
// Operands live in shared memory in the canonical K-major layout without
// swizzling: the matrix is cut into "core matrices" of 8 rows x 16 bytes
// (8 rows x 4 TF32 values) stored as 128 contiguous bytes, row r at byte
// 16 r.  Core matrices adjacent along K are LBO bytes apart, groups of 8
// rows SBO bytes apart.  One kind::tf32 MMA consumes K = 8 (two core
// matrices along K).
//
// Exact split products: an FP32 value x >= 0 of a row with exponent e
// (2^e > every entry of the row) is written as three integer digits,
// x = 2^e (x1 2^-9 + x2 2^-18 + x3 2^-27) with x1 in [0, 512] and
// x2, x3 in [-256, 256], all exact in TF32.  A product sum over K <= 24
// taken digit class by digit class -- (1,1); (1,2) + (2,1);
// (1,3) + (2,2) + (3,1) -- adds integers below 2^24 only, which the
// tensor core's FP32 accumulation represents exactly whatever its internal
// alignment and truncation; the three class sums are combined in FP32 with
// round-to-nearest.  (Plain 3xTF32, x = tf32(x) + tf32(x - tf32(x)), leaves
// the truncating accumulation inside the MMA visible as a bias of a few
// 1e-7 relative on sums of positive terms.)
#pragma once

#include <stdint.h>

namespace d4 {
namespace tc {

// Bound of every wait on the tensor cores (nanoseconds of %globaltimer).
constexpr unsigned long long WAIT_LIMIT_NS = 1000000000ull;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Shared-memory matrix descriptor: K-major, no swizzle, relative LBO.
// Bits 0-13 start address >> 4, 16-29 LBO >> 4, 32-45 SBO >> 4, 46-47
// descriptor version (1 for tcgen05), 49-51 base offset (0), 52 LBO mode
// (0), 61-63 swizzle mode (0 = none).
__device__ __forceinline__ uint64_t desc_kmajor(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of kind::tf32: D in FP32 (bits 4-5 = 1), A and B
// TF32 (bits 7-9 and 10-12 = 2), both K-major (bits 15, 16 = 0), dense, no
// negation; N >> 3 in bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

// FP32 -> TF32, round to nearest (ties away); the low 13 bits become 0.
__device__ __forceinline__ float to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// D[tmem] (+)= A[adesc] B[bdesc]^T, issued by one thread.
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Arrive on the mbarrier once every MMA issued so far by this thread is done.
__device__ __forceinline__ void commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   mbar)
               : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(mbar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Wait for the phase with the given parity to complete, at most
// ``limit_ns``; false when the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity,
                                          unsigned long long limit_ns = WAIT_LIMIT_NS) {
  if (mbar_try_wait(mbar, parity)) return true;
  const unsigned long long t0 = global_ns();
  while (!mbar_try_wait(mbar, parity))
    if (global_ns() - t0 > limit_ns) return false;
  return true;
}

// Generic-proxy shared-memory writes -> visible to the tensor core.
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Tensor-memory allocation by one full warp; the base address goes to
// shared memory.  ncols: a power of two >= 32.
__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

// 16 consecutive 32-bit columns of one tensor-memory lane per thread: warp
// w (mod 4) reads lanes 32 (w % 4) .. + 31; taddr carries the lane base in
// bits 16-31 and the first column in bits 0-15.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
        "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr)
      : "memory");
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&v)[8]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7])
      : "r"(taddr)
      : "memory");
}

__device__ __forceinline__ void tmem_ld_wait() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// 16-byte asynchronous copy global -> shared (bypassing L1), completed by
// cp_async_wait; commit groups the copies issued so far by this thread.
__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gmem_src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(smem_dst)),
               "l"(gmem_src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
// Wait until at most N of this thread's committed groups are still in flight.
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// dst[0 .. bytes/4) += src[...] (FP32, element-wise, performed at L2) from
// shared memory, asynchronously; bytes a multiple of 16, both addresses
// 16-byte aligned.  bulk_commit groups the operations issued so far by this
// thread and bulk_wait_read waits until their shared-memory sources have been
// read (the writes to global memory complete before the kernel ends).
__device__ __forceinline__ void bulk_reduce_add_f32(float *gmem_dst, const float *smem_src,
                                                    uint32_t bytes) {
  asm volatile(
      "cp.reduce.async.bulk.global.shared::cta.bulk_group.add.f32 [%0], [%1], %2;" ::"l"(gmem_dst),
      "r"(smem_u32(smem_src)), "r"(bytes)
      : "memory");
}
__device__ __forceinline__ void bulk_commit() {
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
__device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}

}  // namespace tc
}  // namespace d4
