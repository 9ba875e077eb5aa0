// Blackwell 5th-generation tensor cores (sm_100a / sm_103a) from inline PTX:
// tcgen05.mma with operands in shared memory and the accumulator in tensor
// memory (TMEM), completion through an mbarrier, results read back with
// tcgen05.ld.  Only what the radiance-cache MLP needs: BF16 x BF16 -> FP32,
// one CTA (cta_group::1), M = 128 rows, K-major operands without swizzling.
//
// Operand layout in shared memory ("K-major, no swizzle" canonical layout):
// the matrix is cut into core matrices of 8 rows x 8 BF16 (16 bytes per row,
// 128 contiguous bytes per core matrix); core (row group g, column group c)
// of a matrix with K columns sits at byte (g * K/8 + c) * 128.  The
// descriptor's leading-dimension byte offset is then the step between core
// matrices along K (128 B) and its stride byte offset the step between row
// groups (K/8 * 128 B).  One MMA consumes K = 16 (two core-matrix columns);
// the next K step starts 256 bytes further.
//
// Every wait is bounded: a wait that gives up sets bit 0 of the caller's
// status word and returns false, so no kernel can spin forever.
#pragma once
#include <cstdint>

namespace b200 {
namespace tc {

__device__ __forceinline__ uint32_t smemAddr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of element (row, col) of a BF16 matrix with `k` columns in the
// K-major no-swizzle layout
__host__ __device__ __forceinline__ uint32_t kmajorOffset(int row, int col, int k) {
  return uint32_t((((row >> 3) * (k >> 3) + (col >> 3)) << 7) + ((row & 7) << 4) + ((col & 7) << 1));
}

// shared-memory matrix descriptor: start address, leading (K) and stride
// (row-group) byte offsets, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t smemDesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return uint64_t((addr >> 4) & 0x3fffu) | (uint64_t((lbo >> 4) & 0x3fffu) << 16) |
         (uint64_t((sbo >> 4) & 0x3fffu) << 32) | (uint64_t(1) << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, shape M x N
__host__ __device__ constexpr uint32_t idescBF16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(N >> 3) << 17) | (uint32_t(M >> 4) << 24);
}

// ---- TMEM allocation (one full warp)
__device__ __forceinline__ void tmemAlloc(uint32_t *dstSmem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smemAddr(dstSmem)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmemDealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// ---- mbarrier
__device__ __forceinline__ void mbarInit(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// waits for the phase with parity `parity` to complete; false after `limit` polls
__device__ __forceinline__ bool mbarWait(uint64_t *bar, uint32_t parity, uint32_t limit = 1u << 22) {
  const uint32_t a = smemAddr(bar);
  for (uint32_t i = 0; i < limit; i++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// ---- MMA (one thread), commit of its completion to an mbarrier
__device__ __forceinline__ void mma(uint32_t dTmem, uint64_t aDesc, uint64_t bDesc, uint32_t idesc, bool accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(dTmem),
      "l"(aDesc), "l"(bDesc), "r"(idesc), "r"(accumulate ? 1u : 0u)
      : "memory");
}
__device__ __forceinline__ void commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smemAddr(bar))
               : "memory");
}

// ---- ordering between threads, the async proxy and the tensor core
__device__ __forceinline__ void fenceProxyAsync() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fenceBeforeSync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fenceAfterSync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// ---- TMEM -> registers: this warp's 32 lanes (rows), 16 consecutive 32-bit columns
__device__ __forceinline__ void tmemLoad16(uint32_t taddr, float *v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 16; k++) v[k] = __uint_as_float(r[k]);
}

// D (TMEM, M = 128 rows, N columns) = A (M x K, smem) x B^T (B: N x K, smem),
// issued by the calling thread as K/16 MMAs; a, b: descriptor bases.
__device__ __forceinline__ void gemmIssue(uint32_t dTmem, uint32_t aAddr, int aK, uint32_t bAddr, int bK, int K,
                                          uint32_t idesc) {
  for (int k = 0; k < K / 16; k++) {
    const uint64_t ad = smemDesc(aAddr + uint32_t(k) * 256u, 128u, uint32_t(aK / 8) * 128u);
    const uint64_t bd = smemDesc(bAddr + uint32_t(k) * 256u, 128u, uint32_t(bK / 8) * 128u);
    mma(dTmem, ad, bd, idesc, k > 0);
  }
}

}  // namespace tc
}  // namespace b200
