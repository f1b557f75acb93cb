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

// the same with the A operand in tensor memory (M = 128 rows on the 128 lanes, one
// tf32 element per 32-bit column, K = 8 columns from address a_t)
__device__ __forceinline__ void mma_tf32_ta(uint32_t dt, uint32_t a_t, uint64_t bd, uint32_t idesc, uint32_t acc)
{
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                 " tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n}\n"
                 :: "r"(dt), "r"(a_t), "l"(bd), "r"(idesc), "r"(acc));
}

// D (=|+=) A_lo B_hi + A_hi B_lo + A_hi B_hi over K = 64 (8 steps each, the small
// products first): A 128 x 64 and B 64 x 64 tf32 in the K-major core-matrix layout,
// hi halves at sA / sB, lo halves a_lo / b_lo bytes further.  The descriptors of step
// k are the step-0 descriptors plus k steps (A 4096 B, B 2048 B, in 16-byte units),
// so the issuing thread only adds: rebuilding them per MMA measured 1.5x slower.
__device__ __forceinline__ void mma3_tf32(uint32_t dt, uint32_t sA, uint32_t a_lo, uint32_t sB, uint32_t b_lo,
                                          uint32_t idesc, bool accumulate)
{
    const uint64_t dAhi = sdesc(sA, 2048, 128), dAlo = sdesc(sA + a_lo, 2048, 128);
    const uint64_t dBhi = sdesc(sB, 1024, 128), dBlo = sdesc(sB + b_lo, 1024, 128);
#pragma unroll
    for (int k = 0; k < 8; k++) {
        mma_tf32(dt, dAlo + 256 * k, dBhi + 128 * k, idesc, (accumulate || k > 0) ? 1u : 0u);
        mma_tf32(dt, dAhi + 256 * k, dBlo + 128 * k, idesc, 1);
    }
#pragma unroll
    for (int k = 0; k < 8; k++) mma_tf32(dt, dAhi + 256 * k, dBhi + 128 * k, idesc, 1);
}

// the same products with A_hi in tensor memory (64 columns from ta_hi, lane r = row r)
// and A_lo in shared memory at sAlo: same MMA order, so the same D
__device__ __forceinline__ void mma3_tf32_ta(uint32_t dt, uint32_t ta_hi, uint32_t sAlo, uint32_t sB, uint32_t b_lo,
                                             uint32_t idesc)
{
    const uint64_t dAlo = sdesc(sAlo, 2048, 128);
    const uint64_t dBhi = sdesc(sB, 1024, 128), dBlo = sdesc(sB + b_lo, 1024, 128);
#pragma unroll
    for (int k = 0; k < 8; k++) {
        mma_tf32(dt, dAlo + 256 * k, dBhi + 128 * k, idesc, k > 0 ? 1u : 0u);
        mma_tf32_ta(dt, ta_hi + 8 * k, dBlo + 128 * k, idesc, 1);
    }
#pragma unroll
    for (int k = 0; k < 8; k++) mma_tf32_ta(dt, ta_hi + 8 * k, dBhi + 128 * k, idesc, 1);
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v)
{
    uint32_t r[16];
    // load and wait in one asm block: no use of the values can be scheduled before the wait
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
                 "tcgen05.wait::ld.sync.aligned;"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr)
                 : "memory");
#pragma unroll
    for (int j = 0; j < 16; j++) v[j] = __uint_as_float(r[j]);
}

// two 16-column loads (each thread: its lane, columns a.. and b..) and one wait, in one
// asm block so that no use of the values can be scheduled before the wait
__device__ __forceinline__ void tmem_ld16x2(uint32_t ta, uint32_t tb, float *va, float *vb)
{
    uint32_t r[32];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%32];\n"
                 "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%33];\n"
                 "tcgen05.wait::ld.sync.aligned;"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
                   "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
                   "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                 : "r"(ta), "r"(tb)
                 : "memory");
#pragma unroll
    for (int j = 0; j < 16; j++) {
        va[j] = __uint_as_float(r[j]);
        vb[j] = __uint_as_float(r[16 + j]);
    }
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

// eight consecutive floats from read-only global memory in one 256-bit load (the address
// 32-byte aligned): a warp gathering 32 rows then reads each 32-byte sector once instead
// of twice with two 128-bit loads
__device__ __forceinline__ void ldg8(const float *p, float *r)
{
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(r[0]), "=f"(r[1]), "=f"(r[2]), "=f"(r[3]), "=f"(r[4]), "=f"(r[5]), "=f"(r[6]), "=f"(r[7])
        : "l"(p));
}

// one bulk copy global -> shared of `bytes` (a multiple of 16, both addresses
// 16-byte aligned), completing on mbarrier bar, which expects those bytes
__device__ __forceinline__ void bulk_load(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(bar), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(dst), "l"(src), "r"(bytes), "r"(bar) : "memory");
}

}  // namespace pcsf
