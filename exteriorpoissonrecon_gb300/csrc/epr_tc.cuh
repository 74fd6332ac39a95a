// Blackwell (sm_103a) building blocks for the tensor-core kernels of the learned warm start:
// fifth-generation tensor-core MMA (tcgen05) with accumulators in tensor memory, shared-memory
// matrix descriptors, mbarriers with bounded waits, and 16-byte asynchronous copies.  Inline PTX
// only (ISA 8.6+); device code.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>

namespace epr {
namespace tc {

// error bits a kernel reports through its flag word
constexpr unsigned int kErrWaitTimeout = 1u << 0;
// spin limit of every mbarrier wait (each iteration is one try_wait with the hardware's own
// suspend time hint; a healthy wait ends after a few thousand iterations)
constexpr uint32_t kMaxSpins = 1u << 24;

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// ---- mbarrier ---------------------------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the phase with the given parity to complete; gives up after kMaxSpins tries, sets
// kErrWaitTimeout in *err and returns false.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, unsigned int *err)
{
    for (uint32_t i = 0; i < kMaxSpins; i++)
        if (mbar_try_wait(bar, parity)) return true;
    if (err) atomicOr(err, kErrWaitTimeout);
    return false;
}

// ---- 16-byte asynchronous global -> shared copies (zero-filled when src_bytes == 0) -----------
__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gmem_src, uint32_t src_bytes)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_addr(smem_dst)), "l"(gmem_src), "r"(src_bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// generic-proxy writes to shared memory (st.shared, cp.async) made visible to the tensor core's
// asynchronous proxy, which reads the MMA operands
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// ---- tensor memory -----------------------------------------------------------------------------
// one warp allocates `ncols` columns (a power of two >= 32) and the base address lands in *dst
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// ---- descriptors -------------------------------------------------------------------------------
// Shared-memory matrix descriptor, no swizzle, K-major canonical layout: the operand is stored as
// 8-row x 16-byte core matrices (128 contiguous bytes each, row r of the core at +16 r); `lbo` is
// the byte distance between core matrices adjacent along K, `sbo` between core matrices adjacent
// along M (or N).  Fields: start address >> 4 (bits 0-13), LBO >> 4 (16-29), SBO >> 4 (32-45),
// descriptor version 1 (bits 46-47), base offset 0, layout "no swizzle" 0 (bits 61-63).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16 with BF16 A and B (both K-major), FP32 accumulator, dense:
// D format F32 (bits 4-5 = 1), A format BF16 (bits 7-9 = 1), B format BF16 (bits 10-12 = 1),
// N >> 3 (bits 17-22), M >> 4 (bits 24-28).
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// D (tensor memory) = A B^T (+ D when accumulate): issued by one thread
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate)
{
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "setp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
        "}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// the mbarrier receives one arrival when every MMA this thread issued before has completed
__device__ __forceinline__ void mma_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}

// 16 consecutive 32-bit columns of this warp's 32 tensor-memory lanes (lane i of the warp reads
// lane (taddr >> 16) + i); followed by tmem_wait_ld before the registers are used
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v)
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 16; k++) v[k] = __uint_as_float(r[k]);
}

// byte offset of element (row, k) inside a K-major no-swizzle operand tile whose rows hold
// `kcores` core matrices along K (row-group stride 128 kcores bytes)
__host__ __device__ constexpr uint32_t core_offset(int row, int kcore, int kcores)
{
    return (uint32_t)(((row >> 3) * kcores + kcore) * 128 + (row & 7) * 16);
}

// 8 x 8 transpose of 16-bit elements: in[j] holds row j (8 elements, element 2p in the low half
// of word p); out[r] receives column r
__device__ __forceinline__ void transpose8x8_b16(const uint4 *in, uint4 *out)
{
    const uint32_t *w = reinterpret_cast<const uint32_t *>(in);  // w[4 j + p]
    uint32_t *o = reinterpret_cast<uint32_t *>(out);              // o[4 r + q]
#pragma unroll
    for (int p = 0; p < 4; p++)
#pragma unroll
        for (int q = 0; q < 4; q++)
        {
            const uint32_t a = w[4 * (2 * q) + p], b = w[4 * (2 * q + 1) + p];
            o[4 * (2 * p) + q] = __byte_perm(a, b, 0x5410);
            o[4 * (2 * p + 1) + q] = __byte_perm(a, b, 0x7632);
        }
}

}  // namespace tc
}  // namespace epr
