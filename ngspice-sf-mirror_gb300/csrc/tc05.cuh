/*
 * tcgen05 building blocks shared by the network kernels (gnn.cu) and the
 * learned predictor inside the transient kernel (engine.cu): tensor-memory
 * allocation, shared-memory and instruction descriptors for BF16 products
 * with FP32 accumulation (kind::f16, M = 128, K-major operands without
 * swizzle), issue, commit to an mbarrier, bounded completion wait and the
 * 32-lane accumulator load.  Inline PTX, sm_103a.
 */
#ifndef NGSF_TC05_CUH
#define NGSF_TC05_CUH

#include <stdint.h>

#define TC05_BM 128              /* accumulator rows (tensor-memory lanes) */
#define TC05_SPIN (1LL << 26)    /* completion-wait polls before giving up */

__device__ __forceinline__ uint32_t tc05_smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

/* Shared-memory matrix descriptor, no swizzle, K-major: core matrices of
 * 8 rows x 16 bytes; lbo = byte distance between core matrices adjacent
 * in K, sbo = between core matrices adjacent in M/N (8-row groups). */
__device__ __forceinline__ uint64_t tc05_smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;   /* descriptor version for tcgen05 */
    return d;                 /* base offset 0, layout SWIZZLE_NONE */
}

/* Instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both
 * K-major, M = 128, N = n. */
__device__ __forceinline__ uint32_t tc05_instr_desc(int n)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
           ((uint32_t)(TC05_BM >> 4) << 24);
}

__device__ __forceinline__ void tc05_mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

/* bounded wait for the mbarrier phase; false when the limit ran out */
__device__ __forceinline__ bool tc05_mbar_wait(uint32_t bar, uint32_t phase)
{
    for (long long i = 0; i < TC05_SPIN; i++) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(bar), "r"(phase)
            : "memory");
        if (ok)
            return true;
    }
    return false;
}

__device__ __forceinline__ void tc05_tmem_alloc(uint32_t dst_smem, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tc05_tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
                 : "memory");
}

__device__ __forceinline__ void tc05_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc05_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tc05_mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void tc05_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

/* 32 lanes x 16 columns of FP32 from tensor memory, one row per thread */
__device__ __forceinline__ void tc05_ld16(uint32_t taddr, float *v)
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++)
        v[i] = __uint_as_float(r[i]);
}


/* Copy a rows x kt tile (K-major bf16 in global memory, row stride ld
 * elements) into the core-matrix layout: element (r, k) at (r/8)*sbo +
 * (k/8)*128 + (r%8)*16 + (k%8)*2 with sbo = kt/8*128, in 16-byte pieces;
 * rows >= nrows are zero.  All threads of the block take part. */
__device__ __forceinline__ void tc05_stage_tile(unsigned char *dst, const void *src, int ld,
                                                int row0, int nrows, int rows, int k0, int kt)
{
    const int kg = kt / 8, sbo = kg * 128;
    const unsigned short *s16 = (const unsigned short *)src;
    for (int c = threadIdx.x; c < rows * kg; c += blockDim.x) {
        const int r = c / kg, g = c % kg;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (row0 + r < nrows)
            v = *(const uint4 *)(s16 + (size_t)(row0 + r) * ld + k0 + g * 8);
        *(uint4 *)(dst + (r / 8) * sbo + g * 128 + (r % 8) * 16) = v;
    }
}

/* byte offset of element (r, k) of a staged tile with kt columns */
__device__ __forceinline__ int tc05_off(int r, int k, int kt)
{
    return (r / 8) * (kt / 8 * 128) + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2;
}

#endif
