// sm_103a tensor-core building blocks as inline PTX: mbarriers, bulk copies,
// TMEM allocation, tcgen05.mma (kind::f16, BF16 in, FP32 accumulate), commits,
// TMEM loads, and the shared-memory / instruction descriptors.
//
// Operand layouts used here are the no-swizzle ("interleaved") canonical forms:
// a core matrix is 8 rows of 16 contiguous bytes (128 B). For a K-major operand
// a row is 8 consecutive K elements of one M (or N) index; for an MN-major
// operand a row is 8 consecutive M (or N) elements of one K index. The
// descriptor's SBO is the byte distance between core matrices that are adjacent
// along M/N, its LBO the distance between core matrices adjacent along K.
#pragma once

#include <cstdint>

namespace amb
{
namespace tc
{
    constexpr long long kSpinLimit = 1ll << 22;  // bounded mbarrier waits (then the kernel gives up)

    __device__ __forceinline__ uint32_t smem_u32(const void* p)
    {
        return static_cast<uint32_t>(__cvta_generic_to_shared(p));
    }

    // ------------------------------------------------------------ mbarriers
    __device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
    {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    }

    __device__ __forceinline__ void fence_mbar_init()
    {
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }

    __device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
    {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                     : "memory");
    }

    __device__ __forceinline__ void mbar_arrive(uint64_t* bar)
    {
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
    }

    __device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
    {
        uint32_t ok;
        asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
                     : "=r"(ok)
                     : "r"(smem_u32(bar)), "r"(parity)
                     : "memory");
        return ok != 0;
    }

    // Bounded wait for the phase of the given parity; false on timeout or when
    // *abort (if given) becomes non-zero (another role gave up).
    __device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, const volatile int* abort)
    {
        for (long long i = 0; i < kSpinLimit; ++i)
        {
            if (mbar_try_wait(bar, parity)) return true;
            if (abort && (i & 255) == 255 && *abort) return false;
        }
        return false;
    }

    // --------------------------------------------------------- bulk copies
    // Untiled bulk copy global -> shared; both addresses 16-byte aligned, bytes % 16 == 0.
    __device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
    {
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         smem_u32(dst)),
                     "l"(src), "r"(bytes), "r"(smem_u32(bar))
                     : "memory");
    }

    // Makes generic-proxy shared-memory writes visible to the tensor core (async proxy).
    __device__ __forceinline__ void fence_proxy_async()
    {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }

    // ----------------------------------------------------------------- TMEM
    // Warp-wide: allocates ncols (power of two, >= 32) columns; writes the base address to *dst.
    __device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
                     "r"(ncols)
                     : "memory");
    }

    __device__ __forceinline__ void tmem_relinquish()
    {
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }

    __device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
    {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
    }

    __device__ __forceinline__ void tc_fence_before()
    {
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    }

    __device__ __forceinline__ void tc_fence_after()
    {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    }

    // ------------------------------------------------------------------ MMA
    // D[tmem] (+)= A[smem] * B[smem]^T, one elected thread.
    __device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                             uint32_t accumulate)
    {
        asm volatile(
            "{ .reg .pred p; setp.ne.b32 p, %4, 0; tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p; }" ::"r"(
                d_tmem),
            "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
            : "memory");
    }

    // Arrives (once) on *bar when every tcgen05 operation this thread issued so far has completed.
    __device__ __forceinline__ void mma_commit(uint64_t* bar)
    {
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         smem_u32(bar))
                     : "memory");
    }

    // Each thread of the warp reads 32 (or 16) consecutive 32-bit columns of its own
    // TMEM lane; the warp reads lanes [32 (warp % 4), +32).
    __device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32])
    {
        uint32_t r[32];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
            "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
              "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]),
              "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
              "=r"(r[30]), "=r"(r[31])
            : "r"(taddr)
            : "memory");
#pragma unroll
        for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
    }

    __device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[32])
    {
        uint32_t r[16];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
            "%14, %15}, [%16];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
            : "r"(taddr)
            : "memory");
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
#pragma unroll
        for (int i = 16; i < 32; ++i) v[i] = 0.f;
    }

    // Each thread of the warp writes zeros to 16 consecutive columns of its own TMEM lane.
    __device__ __forceinline__ void tmem_st16_zero(uint32_t taddr)
    {
        const uint32_t z = 0u;
        asm volatile(
            "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, "
            "%1, %1};" ::"r"(taddr),
            "r"(z)
            : "memory");
    }

    __device__ __forceinline__ void tmem_wait_st()
    {
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
    }

    __device__ __forceinline__ void tmem_wait_ld()
    {
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    }

    // ---------------------------------------------------------- descriptors
    // Shared-memory matrix descriptor, no swizzle: start address, LBO and SBO in
    // 16-byte units (bits 0-13, 16-29, 32-45), descriptor version 1 (bit 46),
    // base offset 0, swizzle mode 0 (bits 61-63).
    __host__ __device__ constexpr uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
    {
        return uint64_t((addr & 0x3FFFFu) >> 4) | (uint64_t((lbo & 0x3FFFFu) >> 4) << 16) |
               (uint64_t((sbo & 0x3FFFFu) >> 4) << 32) | (uint64_t(1) << 46);
    }

    // Instruction descriptor for kind::f16: D FP32 (bits 4-5 = 1), A and B BF16
    // (bits 7-9 and 10-12 = 1), A / B MN-major flags (bits 15, 16), N >> 3 (bits
    // 17-22), M >> 4 (bits 24-28). Dense, no negation.
    __host__ __device__ constexpr uint32_t idesc_bf16(int m, int n, bool a_mn_major, bool b_mn_major)
    {
        return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(a_mn_major) << 15) | (uint32_t(b_mn_major) << 16) |
               (uint32_t(n >> 3) << 17) | (uint32_t(m >> 4) << 24);
    }
}
}
