// Blackwell tensor-core building blocks for the mixed-precision DFT form:
// inline PTX for tcgen05 (TMEM allocation, MMA from shared-memory operands,
// commit to an mbarrier, TMEM loads) and the shared-memory matrix layout
// the MMA reads.
//
// Layout (no swizzle, K-major): a matrix of R rows by K tf32 columns is
// stored as 8-row x 4-column "core matrices" of 128 contiguous bytes (row r
// of a core matrix at byte 16*(r%8), column k at 4*(k%4)); core matrices
// adjacent along K are 128 bytes apart (the descriptor's leading-dimension
// offset) and 8-row groups are K/4*128 bytes apart (its stride-dimension
// offset).  One MMA of kind::tf32 consumes K = 8 columns, i.e. two core
// matrices along K, so successive K blocks start 256 bytes apart.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace cdx {
namespace tc {

// byte offset of element (r, k) in an R x K (K a multiple of 4) operand
__host__ __device__ __forceinline__ unsigned op_offset(int r, int k, int K) {
  return (unsigned)(((r >> 3) * (K >> 2) + (k >> 2)) * 128 + (r & 7) * 16 + (k & 3) * 4);
}

__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor (tcgen05 format): start address, leading
// (K-direction) and stride (row-group) byte offsets, descriptor version 1,
// no swizzle.
__device__ __forceinline__ uint64_t make_desc(unsigned saddr, unsigned lbo, unsigned sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo & 0x3FFFFu) >> 4) << 16;
  d |= (uint64_t)((sbo & 0x3FFFFu) >> 4) << 32;
  d |= (uint64_t)1 << 46;  // version
  return d;                // base offset 0, relative LBO, no swizzle
}

// Instruction descriptor of kind::tf32: D in F32, A and B in TF32, both
// K-major, M rows and N columns.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4)                      // D format: F32
         | (2u << 7)                    // A format: TF32
         | (2u << 10)                   // B format: TF32
         | ((uint32_t)(N >> 3) << 17)   // N >> 3
         | ((uint32_t)(M >> 4) << 24);  // M >> 4
}

// ---------------------------------------------------------------- TMEM
// Allocate ncols TMEM columns (a power of two, >= 32); the base address is
// written to *slot (shared memory).  Executed by all threads of one warp.
__device__ __forceinline__ void tmem_alloc(unsigned* slot, unsigned ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_addr(slot)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_free(unsigned taddr, unsigned ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Make this thread's shared-memory writes visible to the tensor core.
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// D[tmem] (+)= A[desc] * B[desc]^T, one MMA of kind::tf32; accumulate when acc.
__device__ __forceinline__ void mma_tf32(unsigned d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         int acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

// Arrive on the mbarrier once all MMAs issued by this thread have completed.
__device__ __forceinline__ void mma_commit(uint64_t* mbar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_addr(mbar))
      : "memory");
}

// ---------------------------------------------------------------- mbarrier
__device__ __forceinline__ void mbar_init(uint64_t* mbar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(mbar)), "r"(count)
               : "memory");
}
// Wait for the completion of phase `parity` for at most max_cycles SM clock
// cycles.  Returns false when the limit was reached.
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, unsigned parity, long long max_cycles) {
  const unsigned a = smem_addr(mbar);
  const long long t0 = clock64();
  while (true) {
    unsigned done;
    // the thread may sleep in the instruction (up to the 20 us hint) until
    // the phase completes, instead of spinning
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity), "r"(20000u)
        : "memory");
    if (done) return true;
    if (clock64() - t0 > max_cycles) return false;
  }
}

// ---------------------------------------------------------------- TMEM loads
// 32 lanes x 32 bits, 16 consecutive columns: thread i of the warp gets lane
// (taddr lane + i), columns col .. col+15.
__device__ __forceinline__ void tmem_ld16(unsigned taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// ---------------------------------------------------------------- tf32 split
// x = hi + lo with hi, lo rounded to tf32 (11 significant bits each); the
// three products hi*hi + lo*hi + hi*lo then carry about 22 bits.
__device__ __forceinline__ float tf32_round(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}
__device__ __forceinline__ void tf32_split(float x, float& hi, float& lo) {
  hi = tf32_round(x);
  lo = tf32_round(__fsub_rn(x, hi));
}

}  // namespace tc
}  // namespace cdx
