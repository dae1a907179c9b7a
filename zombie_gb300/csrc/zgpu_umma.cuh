// zgpu_umma.cuh -- thin inline-PTX wrappers for the 5th-generation tensor cores (tcgen05):
// tensor-memory allocation, single-thread MMA issue from shared-memory operand descriptors,
// commit to an mbarrier, and tensor-memory loads.  Used by the neural cache's inference
// kernel (zgpu_cache.cu), whose 128-point tiles are one M = 128 MMA each.
//
// Operands live in shared memory in the canonical K-major layout without swizzling: the
// matrix is cut into "core matrices" of 8 rows x 16 bytes (8 BF16 values of 8 consecutive
// K), each stored as 128 contiguous bytes; core matrices adjacent along K are `lbo` bytes
// apart and core matrices adjacent along M (or N) are `sbo` bytes apart.
#pragma once

#include <cstdint>

namespace zg {
namespace umma {

__device__ __forceinline__ uint32_t smemAddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (row, k) of a BF16 operand in the canonical K-major layout with
// lbo = 128 (core matrices adjacent along K are contiguous) and sbo = 16 * kCols
template <int kCols>
__device__ __forceinline__ uint32_t canonicalOffset(int row, int k) {
    return (uint32_t)((row >> 3) * (16 * kCols) + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// shared-memory matrix descriptor: start address, leading (K) and stride (M/N) byte
// offsets, the fixed descriptor version 0b001 at bits 46-48, no swizzling
__device__ __forceinline__ uint64_t descriptor(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// instruction descriptor of kind::f16: BF16 A and B (both K-major), FP32 accumulator, M x N
__host__ __device__ constexpr uint32_t instrBf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// D[tmem] (+)= A * B^T, issued by one thread
__device__ __forceinline__ void mma(uint32_t tmemD, uint64_t a, uint64_t b, uint32_t idesc, bool accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
        :
        : "r"(tmemD), "l"(a), "l"(b), "r"(idesc), "r"((int)accumulate)
        : "memory");
}

// the mbarrier receives one arrival when every MMA issued so far by this thread completes
__device__ __forceinline__ void commit(uint64_t* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 :
                 : "r"(smemAddr(mbar))
                 : "memory");
}

// initialises an mbarrier and makes the initialisation visible to the tensor cores' arrivals
__device__ __forceinline__ void mbarInit(uint64_t* mbar, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" : : "r"(smemAddr(mbar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// waits for the phase with parity `parity` to complete; false after `limit` polls
__device__ __forceinline__ bool mbarWait(uint64_t* mbar, uint32_t parity, long long limit) {
    const uint32_t a = smemAddr(mbar);
    for (long long i = 0; i < limit; i++) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// tensor-memory allocation by one whole warp: the base address is written to *dst (shared)
__device__ __forceinline__ void alloc(uint32_t* dst, uint32_t columns) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :
                 : "r"(smemAddr(dst)), "r"(columns)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void dealloc(uint32_t base, uint32_t columns) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" : : "r"(base), "r"(columns) : "memory");
}

__device__ __forceinline__ void fenceBeforeSync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fenceAfterSync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// makes this thread's generic-proxy shared-memory writes visible to the tensor cores
__device__ __forceinline__ void fenceProxyAsync() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 consecutive FP32 columns of this thread's tensor-memory lane (32x32b shape: warp w of
// the warpgroup reads lanes 32w .. 32w + 31; taddr carries the lane in its upper 16 bits).
// The wait for the load sits in the same asm statement, so no use of the registers can be
// scheduled before it.
__device__ __forceinline__ void load16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

}  // namespace umma
}  // namespace zg
