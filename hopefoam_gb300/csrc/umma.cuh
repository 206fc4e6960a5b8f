// umma.cuh -- minimal sm_100-family tensor-core (tcgen05) building blocks in
// inline PTX: tensor-memory allocation, shared-memory matrix descriptors
// (no-swizzle K-major canonical layout), the TF32 and BF16 MMAs with FP32
// accumulation in TMEM, commit to an mbarrier, bounded mbarrier waits, and TMEM loads.
//
// Canonical no-swizzle K-major operand layout used throughout: the matrix is
// tiled in "core matrices" of 8 rows x 16 bytes (8 x 4 TF32).  Element
// (row r, k) of an operand whose core matrices are packed K-fastest lives at
//   ((r / 8) * (KP / 4) + k / 4) * 128 + (r % 8) * 16 + (k % 4) * 4  bytes,
// KP = padded K.  Descriptor: LBO = 128 B (next core matrix along K),
// SBO = (KP / 4) * 128 B (next 8-row group).  One K = 8 MMA step consumes two
// core matrices along K, so step s starts at base + s * 256 B.
#pragma once

#include <cstdint>

namespace umma {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of element (r, k) in the canonical layout above (4-byte elements)
__host__ __device__ __forceinline__ uint32_t kmajor_offset(int r, int k, int KP) {
    return (uint32_t)((((r >> 3) * (KP >> 2) + (k >> 2)) << 7) + ((r & 7) << 4) + ((k & 3) << 2));
}

// 64-bit shared-memory matrix descriptor, no swizzle, descriptor version 1
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo_bytes, uint32_t sbo_bytes) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo_bytes >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo_bytes >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;  // version
    // base offset 0, LBO mode 0, swizzle mode 0 (none)
    return d;
}

// 32-bit instruction descriptor for kind::tf32: D = F32, A = B = TF32, both K-major, dense
__host__ __device__ __forceinline__ uint32_t idesc_tf32(int M, int N) {
    uint32_t d = 0;
    d |= 1u << 4;                        // D format F32
    d |= 2u << 7;                        // A format TF32
    d |= 2u << 10;                       // B format TF32
    d |= (uint32_t)((N >> 3) & 0x3F) << 17;
    d |= (uint32_t)((M >> 4) & 0x1F) << 24;
    return d;
}

// byte offset of element (r, k) in the same canonical layout for 2-byte
// elements (core matrices of 8 rows x 8 BF16): one K = 16 MMA step also
// consumes two core matrices along K (base + s * 256 B); SBO = (KP / 8) * 128 B
__host__ __device__ __forceinline__ uint32_t kmajor_offset_b16(int r, int k, int KP) {
    return (uint32_t)((((r >> 3) * (KP >> 3) + (k >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1));
}

// 32-bit instruction descriptor for kind::f16 with BF16 operands: D = F32,
// A = B = BF16, both K-major, dense
__host__ __device__ __forceinline__ uint32_t idesc_bf16(int M, int N) {
    uint32_t d = 0;
    d |= 1u << 4;                        // D format F32
    d |= 1u << 7;                        // A format BF16
    d |= 1u << 10;                       // B format BF16
    d |= (uint32_t)((N >> 3) & 0x3F) << 17;
    d |= (uint32_t)((M >> 4) & 0x1F) << 24;
    return d;
}

// D[tmem] (+)= A[smem] * B[smem]^T, BF16 operands (K = 16 per instruction)
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T  (both K-major), issued by one thread
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}

// arrive on an mbarrier when all prior tcgen05 async ops of this thread complete
__device__ __forceinline__ void commit(uint64_t* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
                 : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* mbar, uint32_t phase) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(smem_u32(mbar)), "r"(phase)
        : "memory");
    return ok != 0;
}

// bounded wait: returns false if the phase did not complete within `limit` polls
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t phase, uint32_t limit) {
    for (uint32_t i = 0; i < limit; i++)
        if (mbar_try_wait(mbar, phase)) return true;
    return false;
}

// arrive once on an mbarrier (release semantics at CTA scope)
__device__ __forceinline__ void mbar_arrive(uint64_t* mbar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(mbar)) : "memory");
}

// arrive once on an mbarrier and add `bytes` to the transaction count its
// current phase waits for
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)), "r"(bytes)
                 : "memory");
}

// untiled bulk copy global -> shared (both 16-byte aligned, bytes a multiple
// of 16); completion is signalled as transactions on `mbar`
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* mbar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(mbar))
        : "memory");
}

// 8-byte asynchronous copy global -> shared (both 8-byte aligned), completed
// by cp_async_wait_all in the issuing thread
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// make generic-proxy shared-memory writes visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// TMEM allocation (whole warp); the base address is written to *dst (shared)
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// 32 lanes x 32-bit, 8 consecutive columns per thread (warp-collective)
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* v) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 8; i++) v[i] = __uint_as_float(r[i]);
}

// 32 lanes x 32-bit, 4 consecutive columns per thread (warp-collective)
__device__ __forceinline__ void tmem_ld4(uint32_t taddr, float* v) {
    uint32_t r[4];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 4; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// TF32 split of an FP32 value: hi keeps the 10 explicit mantissa bits the
// tensor core reads (round to nearest), lo = x - hi is exact in FP32.
__device__ __forceinline__ void split_tf32(float x, float& hi, float& lo) {
    uint32_t h;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
    hi = __uint_as_float(h);
    lo = x - hi;
}

}  // namespace umma
