// tc_sm100.cuh -- fifth-generation tensor core (tcgen05) primitives for
// sm_100-family GPUs (GB300 = sm_103a), as inline PTX: tensor-memory
// allocation, shared-memory matrix descriptors, the BF16 MMA with FP32
// accumulation in tensor memory, completion through an mbarrier, and loads
// of the accumulator back to registers.
//
// Operand layout used by every caller: K-major, no swizzle.  A "core
// matrix" is 8 rows x 16 bytes (8 bf16 along K) stored contiguously (row r at
// r*16 bytes).  An R x K operand tile (R = M for A, N for B) is stored as
// core matrices [R/8][K/8]: core (ri, ki) at ri*SBO + ki*LBO with LBO = 128
// bytes (next 8 K-elements) and SBO = (K/8)*128 bytes (next 8 rows).  One
// MMA consumes K = 16 (two core matrices along K); the next K-slice starts
// 2*LBO = 256 bytes further.
//
// Every wait on an mbarrier is bounded: after `limit` polls the caller gets
// false back, records an error and cleans up instead of hanging.
#pragma once

#include <cuda_bf16.h>

#include "common.cuh"

namespace tc {

__device__ __forceinline__ u32 smem_u32(const void *p) { return (u32)__cvta_generic_to_shared(p); }

// --- tensor memory ---------------------------------------------------------

// Allocate ncols (a power of two >= 32) columns of tensor memory for this
// CTA; executed by one full warp; the base address lands in *dst (smem).
__device__ __forceinline__ void tmem_alloc(u32 *dst, u32 ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(u32 taddr, u32 ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// make this thread's ordinary shared-memory stores visible to the tensor
// core, which reads operands through the async proxy
__device__ __forceinline__ void fence_smem_to_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// --- descriptors -----------------------------------------------------------

// Shared-memory matrix descriptor, no swizzle (layout in the file comment).
__device__ __forceinline__ u64 smem_desc(const void *base, u32 lbo_bytes, u32 sbo_bytes)
{
    const u64 addr = smem_u32(base);
    u64 d = 0;
    d |= (addr & 0x3FFFFull) >> 4;                  // bits 0-13: start address / 16
    d |= (u64)((lbo_bytes >> 4) & 0x3FFF) << 16;    // bits 16-29: leading-dimension byte offset / 16
    d |= (u64)((sbo_bytes >> 4) & 0x3FFF) << 32;    // bits 32-45: stride-dimension byte offset / 16
    d |= 1ull << 46;                                // bits 46-48: fixed 0b001
    // bits 49-51 base offset 0, bit 52 relative LBO, bits 61-63 swizzle 0 (none)
    return d;
}

// Instruction descriptor of tcgen05.mma kind::f16: BF16 A and B, FP32 D,
// both operands K-major, shape M x N.
__host__ __device__ __forceinline__ u32 idesc_bf16_f32(u32 M, u32 N)
{
    u32 d = 0;
    d |= 1u << 4;             // D format: F32
    d |= 1u << 7;             // A format: BF16
    d |= 1u << 10;            // B format: BF16
    // bits 13,14 no negation; bits 15,16 A and B K-major
    d |= (N >> 3) << 17;      // bits 17-22: N / 8
    d |= (M >> 4) << 24;      // bits 24-28: M / 16
    return d;
}

// --- MMA and completion -------------------------------------------------------

// D[tmem] = A*B^T (+ D when accumulate), issued by one thread
__device__ __forceinline__ void mma_bf16(u32 d_tmem, u64 a_desc, u64 b_desc, u32 idesc, u32 accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t"
        "}" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mbar_init(u64 *bar, u32 count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// the mbarrier's phase completes when all MMAs issued so far by this thread are done
__device__ __forceinline__ void mma_commit(u64 *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// Poll the mbarrier for completion of phase `parity`, at most `limit` times.
__device__ __forceinline__ bool mbar_wait(u64 *bar, u32 parity, u32 limit)
{
    const u32 a = smem_u32(bar);
    for (u32 i = 0; i < limit; i++) {
        u32 done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t"
            "}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// --- accumulator to registers ------------------------------------------------

// 32 lanes x 16 columns of 32-bit: thread t of the warp gets row (lane base +
// t), columns col..col+15.  The warp must address its own lane quarter
// (lanes 32*(warp%4) ...).
__device__ __forceinline__ void tmem_ld16(u32 taddr, u32 (&r)[16])
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// byte offset of element (row, k) in a K-major no-swizzle operand tile with
// K columns (bf16)
__host__ __device__ __forceinline__ u32 kmajor_offset(u32 row, u32 k, u32 K)
{
    return (row >> 3) * (K / 8) * 128 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2;
}

}  // namespace tc
