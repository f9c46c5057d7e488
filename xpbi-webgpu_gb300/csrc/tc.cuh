// Thin inline-PTX layer over the sm_100-family tensor-core path used by the
// warm-start network: tcgen05 MMA with operands in shared memory and the
// accumulator in tensor memory (TMEM), mbarrier completion, TMEM loads.
//
// Operand layout ("canonical K-major, no swizzle"): a tile of R rows x K
// bf16 columns is stored as 8x8 core matrices of 128 contiguous bytes (8 rows
// of 16 bytes); core matrix (row group g, K chunk c) sits at
// (g * (K / 8) + c) * 128. In the shared-memory descriptor the leading byte
// offset is the distance between K-adjacent core matrices (128) and the
// stride byte offset the distance between row groups ((K / 8) * 128).
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace xpbi {
namespace tc {

__device__ __forceinline__ uint32_t smemAddr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Byte offset of element (r, k) of an R x K tile in the core-matrix layout.
__device__ __forceinline__ uint32_t coreOffset(uint32_t r, uint32_t k, uint32_t K) {
  return ((r >> 3) * (K >> 3) + (k >> 3)) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
}

// Shared-memory matrix descriptor (no swizzle, K-major).
__device__ __forceinline__ uint64_t smemDesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1u << 46;  // descriptor version for the sm_100 family
  // base offset 0, absolute LBO mode 0, layout type 0 (no swizzle)
  return d;
}

// Instruction descriptor for kind::f16 with bf16 A and B, f32 accumulate,
// both operands K-major, M x N tile.
__host__ __device__ constexpr uint32_t idescBf16F32(uint32_t M, uint32_t N) {
  return (1u << 4)            // D format: f32
         | (1u << 7)          // A format: bf16
         | (1u << 10)         // B format: bf16
         | ((N >> 3) << 17)   // N / 8
         | ((M >> 4) << 24);  // M / 16
}

__device__ __forceinline__ void mbarInit(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Bounded wait on phase `parity`; returns false if the bound expired.
__device__ __forceinline__ bool mbarWait(uint64_t* bar, uint32_t parity, uint32_t maxSpins) {
  const uint32_t a = smemAddr(bar);
  for (uint32_t s = 0; s < maxSpins; ++s) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// One warp allocates `ncols` TMEM columns; the base address lands in *dst.
__device__ __forceinline__ void tmemAlloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smemAddr(dst)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmemDealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fenceBeforeSync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fenceAfterSync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Generic-proxy shared-memory writes made visible to the tensor core.
__device__ __forceinline__ void fenceProxyAsync() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// D(tmem) (+)= A(smem) * B(smem)^T, one K = 16 step.
__device__ __forceinline__ void mma(uint32_t dTmem, uint64_t aDesc, uint64_t bDesc, uint32_t idesc,
                                    bool accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.u32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dTmem),
      "l"(aDesc), "l"(bDesc), "r"(idesc), "r"((uint32_t)accumulate)
      : "memory");
}

// Arrive on `bar` once every previously issued MMA of this thread completes.
__device__ __forceinline__ void commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smemAddr(bar))
               : "memory");
}

// 32 lanes x 32 bit, 16 consecutive columns per thread; the wait for the
// load sits in the same asm statement so no use of the registers can be
// scheduled before the data has arrived.
__device__ __forceinline__ void ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc
}  // namespace xpbi
