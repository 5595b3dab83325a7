// Thin inline-PTX wrappers for the sm_100a / sm_103a tensor-core path:
// tensor memory (TMEM) allocation, tcgen05.mma with operands in shared memory
// and the accumulator in TMEM, completion through an mbarrier, TMEM loads,
// and bulk global -> shared copies.
//
// Shared-memory operands use the canonical layouts without swizzle: the
// matrix is cut into core matrices of 8 rows x 16 bytes (8 halves), each
// stored as 128 contiguous bytes (row r at byte 16 r).  K-major: core matrix
// (i, j) (M/N group i, K group j) sits at  base + i * SBO + j * LBO.
// MN-major: the 16-byte rows run along M/N and the 8 rows along K; core
// matrix (i, j) again at  base + i * SBO + j * LBO.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace dl {
namespace tc {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// 64-bit shared-memory matrix descriptor: start address, leading byte offset
// (between core matrices along the product's K), stride byte offset (along
// M or N), descriptor version 1, no swizzle.  Without swizzle the two
// offsets keep these axes for K-major and MN-major operands alike.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo & 0x3FFFFu) >> 4) << 16;
    d |= (uint64_t)((sbo & 0x3FFFFu) >> 4) << 32;
    d |= (uint64_t)1 << 46;  // version
    // base offset 0, lbo mode 0, layout type 0 (no swizzle)
    return d;
}

// 32-bit instruction descriptor of kind::f16: fp16 A and B, fp32
// accumulator, shape M x N; A and B K-major unless `a_mn` / `b_mn`.
__host__ __device__ constexpr uint32_t idesc_f16_f32(int M, int N, bool a_mn = false, bool b_mn = false) {
    return (1u << 4)                         // accumulator format: f32
           | (0u << 7) | (0u << 10)          // A, B: f16
           | ((a_mn ? 1u : 0u) << 15)        // A major-ness
           | ((b_mn ? 1u : 0u) << 16)        // B major-ness
           | ((uint32_t)(N >> 3) << 17)      // N / 8
           | ((uint32_t)(M >> 4) << 24);     // M / 16
}

// One warp allocates `ncols` columns (a power of two >= 32) and writes the
// address to shared memory.
__device__ __forceinline__ void tmem_alloc(uint32_t* smem_result, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n"
                 :: "r"(smem_addr(smem_result)), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" :: "r"(taddr), "r"(ncols) : "memory");
}

// D[taddr] (+)= A x B^T, one instruction; `accumulate` 0 overwrites D.
__device__ __forceinline__ void mma_f16(uint32_t taddr, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
        :: "r"(taddr), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate) : "memory");
}

// The mbarrier arrives once all tcgen05 operations this thread issued
// before have completed.
__device__ __forceinline__ void commit(uint64_t* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n"
                 :: "r"(smem_addr(mbar)) : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}
// Make this thread's ordinary shared-memory stores visible to the tensor core.
__device__ __forceinline__ void fence_smem_to_async() {
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" :: "r"(smem_addr(mbar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
    return t;
}

// Wait for the phase with parity `parity` to complete, for at most `limit_ns`
// nanoseconds (and at most 2^30 polls); returns false when the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, uint64_t limit_ns) {
    const uint32_t a = smem_addr(mbar);
    uint64_t t0 = 0;
    for (uint32_t i = 0; i < (1u << 30); i++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done) : "r"(a), "r"(parity) : "memory");
        if (done) return true;
        if ((i & 63) == 0) {
            const uint64_t t = globaltimer_ns();
            if (i == 0) t0 = t;
            else if (t - t0 > limit_ns) return false;
        }
    }
    return false;
}

// One bulk copy global -> shared (the TMA unit's copy engine), completing on
// `mbar`, which is told to expect `bytes`.  Both addresses 16-byte aligned,
// `bytes` a multiple of 16.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* mbar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" :: "r"(smem_addr(mbar)), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n"
                 :: "r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(mbar)) : "memory");
}

// Bulk copies that share one transaction count: arm the barrier once with
// the total bytes, then issue the copies (each completes its bytes on it).
__device__ __forceinline__ void mbar_expect_tx(uint64_t* mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" :: "r"(smem_addr(mbar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_copy(void* dst, const void* src, uint32_t bytes, uint64_t* mbar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n"
                 :: "r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(mbar)) : "memory");
}

// 32 lanes x 32 consecutive 32-bit columns, load and wait in one statement
// (the registers are valid when it returns): thread l of the warp receives
// TMEM lane (warp's lane base + l), columns [col, col + 32).
__device__ __forceinline__ void ld_32x32b_x32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        "tcgen05.wait::ld.sync.aligned;\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr) : "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// Programmatic dependent launch: let the next kernel of the stream (launched
// with programmatic stream serialization) start its prologue now; and wait
// until the kernels this one depends on have completed and their memory
// writes are visible.
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }

// 32 lanes x 16 consecutive 32-bit columns, load and wait in one statement:
// thread l of the warp receives TMEM lane (warp's lane base + l), columns
// [col, col + 16).
__device__ __forceinline__ void ld_32x32b_x16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        "tcgen05.wait::ld.sync.aligned;\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr) : "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc
}  // namespace dl
