// Blackwell tensor-core building blocks (sm_103a): tcgen05.mma with TMEM
// accumulators, shared-memory matrix descriptors, mbarrier completion and TMEM
// loads, written as inline PTX.
//
// Layout convention of every operand tile (K-major, no swizzle): a tile of R rows
// x K 32-bit elements is stored as core matrices of 8 rows x 16 bytes (4
// elements), each 128 contiguous bytes with row i at byte 16 i; core matrix
// (row group g, K group j) starts at g * SBO + j * 128 with SBO = K * 32 bytes,
// so a tile occupies R * K * 4 bytes.  The descriptor of one MMA step of K = 8
// starts at the step's first K group: it reads core matrices at start + g * SBO
// + {0, 128} (the leading-dimension offset LBO = 128 bytes between the two K
// groups of the step), never beyond the tile.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define TC_SPIN_LIMIT (1u << 24)   // mbarrier polls before a wait gives up

__device__ __forceinline__ uint32_t tc_smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor (tcgen05): start address, leading-dimension
// byte offset, stride byte offset (all >> 4), descriptor version 1 (bit 46),
// base offset 0, no swizzle.
__device__ __forceinline__ uint64_t tc_smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::tf32 with FP32 accumulation, both operands
// K-major: D format F32 (bits 4-5 = 1), A and B format TF32 (bits 7-9 and
// 10-12 = 2), N >> 3 at bits 17-22, M >> 4 at bits 24-28.
__host__ __device__ __forceinline__ uint32_t tc_idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ float tc_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// x = hi + mid + lo exactly, each part a TF32 number (11 + 11 + 2 significant
// bits; lo is at most 2^-23 |x|)
__device__ __forceinline__ void tc_split3(float x, float& h, float& m, float& l) {
  h = tc_tf32(x);
  const float r = x - h;
  m = tc_tf32(r);
  l = r - m;
}

__device__ __forceinline__ void tc_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
               :: "r"(tc_smem_addr(slot)), "r"(ncols));
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void tc_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(taddr), "r"(ncols));
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes become visible to the tensor core (async proxy)
__device__ __forceinline__ void tc_fence_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void tc_bar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(tc_smem_addr(bar)), "r"(count));
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// D[tmem] (+)= A[smem] * B[smem]; issued by one thread
__device__ __forceinline__ void tc_mma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                            uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
      :: "r"(dtmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}
// the mbarrier completes one phase when every MMA this thread issued before has finished
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
               :: "r"(tc_smem_addr(bar)) : "memory");
}
// bounded wait for phase `parity`; false when the limit ran out
__device__ __forceinline__ bool tc_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = tc_smem_addr(bar);
  for (uint32_t it = 0; it < TC_SPIN_LIMIT; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done) : "r"(a), "r"(parity) : "memory");
    if (done) return true;
  }
  return false;
}

// 16 consecutive 32-bit TMEM columns of this warp's 32 lanes (lane i of the warp
// reads TMEM lane (warp % 4) * 32 + i)
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// byte offset of element (row, k) in a K-major tile with K (multiple of 8) columns
__host__ __device__ __forceinline__ uint32_t tc_off(int row, int k, int K) {
  return (uint32_t)((row >> 3) * (K * 32) + (k >> 2) * 128 + (row & 7) * 16 + (k & 3) * 4);
}
