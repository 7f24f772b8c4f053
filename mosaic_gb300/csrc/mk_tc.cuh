// Blackwell tensor-core (tcgen05) building blocks in inline PTX: tensor
// memory (TMEM) allocation, the shared-memory matrix and instruction
// descriptors of tcgen05.mma (kind::f16: FP16 or BF16 operands, FP32
// accumulation in TMEM), completion through an mbarrier, and loads of the
// accumulator back to registers.
//
// Operand layout used throughout: K-major, no swizzle ("interleaved" core
// matrices). A core matrix is 8 rows x 16 bytes (8 x 8 16-bit elements),
// stored as 128 contiguous bytes, row after row. An operand of R rows and K
// columns is stored as [R/8][K/8] core matrices: element (r, k) at byte
// ((r / 8) * (K / 8) + k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2. In the
// descriptor the leading-dimension byte offset (between core matrices
// adjacent along K) is then 128 and the stride-dimension byte offset
// (between 8-row groups) K / 8 * 128; one MMA consumes K = 16 (two core
// matrices along K), so consecutive MMAs advance the start address by 256 B.
#pragma once
#include "mk_common.cuh"

// Byte offset of element (r, k) of an R x K K-major operand (see above).
__host__ __device__ __forceinline__ uint32_t mk_umma_offset(int r, int k, int K)
{
    return (uint32_t)((((r >> 3) * (K >> 3) + (k >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1));
}

// Shared-memory matrix descriptor (64 bit): start address, leading- and
// stride-dimension byte offsets (all >> 4), descriptor version 1 at bits
// 46-47, base offset 0, no swizzle (layout type 0 at bits 61-63).
__device__ __forceinline__ uint64_t mk_umma_sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor of tcgen05.mma kind::f16 (32 bit): FP32 D (bits
// 4-5 = 1), A and B types (bits 7-9, 10-12: 0 FP16, 1 BF16), both operands
// K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t mk_umma_idesc_f16(int M, int N, bool bf16)
{
    return (1u << 4) | ((bf16 ? 1u : 0u) << 7) | ((bf16 ? 1u : 0u) << 10) |
           ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// TMEM: one warp allocates `ncols` columns (a power of two, 32..512) and
// writes the base address to shared memory; the same warp frees them.
__device__ __forceinline__ void mk_tmem_alloc(uint32_t *smem_dst, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     mk_smem_addr(smem_dst)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void mk_tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
                 : "memory");
}

__device__ __forceinline__ void mk_tc_fence_before_sync()
{
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void mk_tc_fence_after_sync()
{
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// D[tmem] (+)= A . B^T for one K = 16 step; issued by one thread.
__device__ __forceinline__ void mk_umma_f16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                            uint32_t idesc, uint32_t accumulate)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Arrive (once) on `bar` when every tcgen05.mma issued so far by this
// thread has completed.
__device__ __forceinline__ void mk_umma_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     mk_smem_addr(bar))
                 : "memory");
}

// 16 consecutive 32-bit accumulator columns of this thread's TMEM lane
// (a warp reads the 32 lanes of its quarter: lane base 32 * (warp % 4)).
__device__ __forceinline__ void mk_tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
        "%11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
