// tcgen05 / TMA helpers shared by the tensor-core kernels (inline PTX, sm_103a).
//
// Operands live in shared memory in the K-major, no-swizzle core-matrix layout:
// a core matrix is 8 rows x 16 bytes (4 tf32), and an operand with G = rows/8
// row groups stores core matrix (g, q) (rows 8g.., K elements 4q..) at byte
// (q*G + g)*128.  Descriptors give the byte distance between core matrices
// along K (leading) and along M/N (stride).
#pragma once
#include <cstdint>

namespace pcsf {

constexpr long TC_WAIT_LIMIT = 1L << 22;     // polls of an mbarrier before a wait gives up

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (r, k) of a K-major tf32 operand with G = rows/8 row
// groups: core matrix (g = r/8, q = k/4) at (q*G + g)*128, row r%8 at 16 B.
__device__ __forceinline__ uint32_t core_off(int r, int k, int G)
{
    return (uint32_t)((((k >> 2) * G + (r >> 3)) << 7) + ((r & 7) << 4) + ((k & 3) << 2));
}

// shared-memory matrix descriptor: start, leading (K) and stride (M/N) byte
// offsets between core matrices, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

__device__ __forceinline__ void mma_tf32(uint32_t dt, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc)
{
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                 " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n"
                 :: "r"(dt), "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v)
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; j++) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ void tmem_st16(uint32_t taddr, const float *v)
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};"
                 :: "r"(taddr), "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
                    "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
                    "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])), "r"(__float_as_uint(v[8])),
                    "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),
                    "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])),
                    "r"(__float_as_uint(v[15])));
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Each poll may suspend the thread for up to TC_WAIT_HINT_NS (it resumes as soon as
// the phase completes), so waiting warps do not take issue slots from the co-resident
// CTA; TC_WAIT_LIMIT polls bound the wait (~4 s).
constexpr uint32_t TC_WAIT_HINT_NS = 1000;
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity)
{
    uint32_t done = 0;
    for (long it = 0; it < TC_WAIT_LIMIT && !done; it++) {
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
                     " selp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(done) : "r"(bar), "r"(parity), "r"(TC_WAIT_HINT_NS) : "memory");
    }
    return done != 0;
}

// hi part of the TF32 split x = hi + lo: x rounded to the nearest TF32 value (ties away
// from zero), so lo = x - hi (exact in FP32) takes either sign and the bits of lo the
// MMA drops (it reads 10 mantissa bits) cancel on average instead of always shrinking |x|
__device__ __forceinline__ float tf32_hi(float x) { return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u); }

// one bulk copy global -> shared of `bytes` (a multiple of 16, both addresses
// 16-byte aligned), completing on mbarrier bar, which expects those bytes
__device__ __forceinline__ void bulk_load(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(bar), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(dst), "l"(src), "r"(bytes), "r"(bar) : "memory");
}

}  // namespace pcsf
