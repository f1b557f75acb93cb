// Tensor-core (tcgen05 kind::f16, sm_103a) pruning with BF16 split products.
//
// The same contraction as k_prune_tc (tc_kernels.cu),
//   D_c[site][a] = sum_j alpha_c[site][j] E_c[a][j]   (M = 128 sites, N = 64, K = 64),
// with each FP32 operand split into three BF16 parts, x = h + m + l
// (h = bf16(x), m = bf16(x - h), l = bf16(x - h - m); the split is exact: x has 24
// significant bits and each part takes 8), and the products whose terms reach
// FP32 accuracy accumulated in FP32 in tensor memory, the small ones first:
//   D = A_l B_h + A_m B_m + A_h B_l + A_m B_h + A_h B_m + A_h B_h
// (the three dropped products, A_m B_l, A_l B_m, A_l B_l, are below 2^-24 of the
// largest term).  A BF16 MMA with K = 16 does the work of two TF32 MMAs with K = 8,
// so these six products take the tensor-pipe time of the three TF32 products of
// k_prune_tc.  Reference contraction replaced: lib/CamlPaml/PhyloLik.ml:87-92.
//
// Layout: 256 threads, thread t owns tile column (site, TMEM lane) t % 128 and
// states 32*(t/128) .. +31.  Partial slots are 64-column regions of tensor memory;
// a contraction stages alpha_c (three BF16 parts) into shared memory as the A operand
// and E_c (three parts, split here from the FP32 E^T that the P(t) formation wrote)
// as the B operand, and D overwrites the child's slot.  Operands use the K-major,
// no-swizzle core-matrix layout: a core matrix is 8 rows x 16 bytes (8 BF16 values),
// core matrix (g, q) (rows 8g.., K elements 8q..) of an operand with G row groups at
// byte (q*G + g)*128 -- the geometry of the TF32 kernel, so the descriptors' leading
// and stride byte offsets and their per-K-step increments are the same numbers.
// The epilogue adds alpha_c = h + m + l (exact) back: v_c = alpha_c + D_c (E = P - I).
// Leaf children are gathers of E^T rows; the root stage is that of k_prune_tc.
//
// Accuracy: like the TF32 kernel, the FP32 accumulation of the tensor cores rounds
// toward minus infinity, so these values serve the search; returned likelihoods come
// from the compensated FP32 or float-float kernels.
//
// Every mbarrier wait is bounded; on timeout the kernel records an error, waits
// (again bounded) for its outstanding tensor-core work, releases its tensor memory
// and exits.
#include <cuda_bf16.h>

#include <cmath>
#include <cstdint>

#include "pcsf_internal.h"
#include "prune_common.cuh"
#include "tc_common.cuh"

namespace pcsf {

namespace {

constexpr int BF_THREADS = 256;
constexpr int BF_M = 128;
constexpr int BF_MAX_SLOTS = 8;
constexpr int BF_MAX_LEAVES = 160;
constexpr uint32_t BA_PART = BF_M * K * 2;     // one BF16 part of A, 16 KB
constexpr uint32_t BB_PART = K * K * 2;        // one BF16 part of B, 8 KB
constexpr uint32_t SMB_A = 0;                  // [h, m, l] parts of A
constexpr uint32_t SMB_B = 3 * BA_PART;        // [h, m, l] parts of B
constexpr uint32_t SMB_LV = SMB_B + 3 * BB_PART;
constexpr int BF_LVS = BF_M + 4;               // padded leaf-state rows (bank-conflict-free fill)

// byte offset of element (r, k) of a K-major BF16 operand with G = rows/8 row groups
__device__ __forceinline__ uint32_t core_off16(int r, int k, int G)
{
    return (uint32_t)((((k >> 3) * G + (r >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1));
}

__device__ __forceinline__ uint32_t bf_bits(__nv_bfloat16 x) { return (uint32_t)__bfloat16_as_ushort(x); }

// eight consecutive K values of one row, split into three BF16 parts packed as 16 bytes each
__device__ __forceinline__ void split8(const float *x, uint4 &h, uint4 &m, uint4 &l)
{
    uint32_t hw[4], mw[4], lw[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        uint32_t hh[2], mm[2], ll[2];
#pragma unroll
        for (int t = 0; t < 2; t++) {
            const float v = x[2 * q + t];
            const __nv_bfloat16 bh = __float2bfloat16_rn(v);
            const float r1 = v - __bfloat162float(bh);
            const __nv_bfloat16 bm = __float2bfloat16_rn(r1);
            const float r2 = r1 - __bfloat162float(bm);
            const __nv_bfloat16 bl = __float2bfloat16_rn(r2);
            hh[t] = bf_bits(bh);
            mm[t] = bf_bits(bm);
            ll[t] = bf_bits(bl);
        }
        hw[q] = hh[0] | (hh[1] << 16);
        mw[q] = mm[0] | (mm[1] << 16);
        lw[q] = ll[0] | (ll[1] << 16);
    }
    h = make_uint4(hw[0], hw[1], hw[2], hw[3]);
    m = make_uint4(mw[0], mw[1], mw[2], mw[3]);
    l = make_uint4(lw[0], lw[1], lw[2], lw[3]);
}

__device__ __forceinline__ float bf_lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf_hi(uint32_t w) { return __uint_as_float(w & 0xFFFF0000u); }

__device__ __forceinline__ void mma_bf16(uint32_t dt, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc)
{
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                 " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
                 :: "r"(dt), "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
}

__global__ void __launch_bounds__(BF_THREADS, 2) k_prune_bf16(PruneArgs a, uint32_t tmem_cols, int *err)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ uint32_t tbase_s;
    __shared__ __align__(8) uint64_t bar_mma;
    __shared__ float cmax[2][2][BF_M];
    __shared__ double red_l[BF_THREADS / 32], red_e[BF_THREADS / 32];
    __shared__ float prf[K], wlf[K];

    const int tid = threadIdx.x, warp = tid >> 5;
    const int site = tid & (BF_M - 1);
    const int half = tid >> 7;
    const int s0 = 32 * half;
    const int nl = a.nl;
    uint8_t *lvT = sm + SMB_LV;
    SchedNode *sched = reinterpret_cast<SchedNode *>(sm + SMB_LV + ((nl * BF_LVS + 15) & ~15));
    const uint32_t barM = smem_addr(&bar_mma);
    const uint32_t sA = smem_addr(sm + SMB_A), sB = smem_addr(sm + SMB_B);
    // kind::f16: D f32, A and B bf16, both K-major, N = 64, M = 128
    const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_addr(&tbase_s)), "r"(tmem_cols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(barM), "r"(1));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int f = tid; f < a.n_internal; f += BF_THREADS) sched[f] = a.sched[f];
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = tbase_s;
    const uint32_t lane_off = (uint32_t)((warp & 3) * 32) << 16;
    uint32_t ph_mma = 0;
    bool ok = true;
    bool mma_pending = false;   // thread 0: a commit whose completion nobody has waited for

    uint64_t dA[3], dB[3];
#pragma unroll
    for (int p = 0; p < 3; p++) {
        dA[p] = sdesc(sA + p * BA_PART, 2048, 128);
        dB[p] = sdesc(sB + p * BB_PART, 1024, 128);
    }

    // alpha of slot s (this thread's 32 states) -> the three parts of the A operand
    auto stage_a = [&](int s) {
        const uint32_t ts = tbase + lane_off + 64 * s + s0;
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
        float x[32];
        tmem_ld16x2(ts, ts + 16, x, x + 16);
#pragma unroll
        for (int j8 = 0; j8 < 4; j8++) {
            uint4 h, m, l;
            split8(x + 8 * j8, h, m, l);
            const uint32_t o = core_off16(site, s0 + 8 * j8, 16);
            *reinterpret_cast<uint4 *>(sm + SMB_A + o) = h;
            *reinterpret_cast<uint4 *>(sm + SMB_A + BA_PART + o) = m;
            *reinterpret_cast<uint4 *>(sm + SMB_A + 2 * BA_PART + o) = l;
        }
    };
    // E_c (B[a][j] = E_c[a][j] = E^T[j][a]) -> the three parts of the B operand
    auto stage_b = [&](const float *Et) {
        for (int g = tid; g < K * K / 8; g += BF_THREADS) {
            const int aa = g & (K - 1), jg = g >> 6;
            float x[8];
#pragma unroll
            for (int t = 0; t < 8; t++) x[t] = __ldg(Et + (size_t)(8 * jg + t) * K + aa);
            uint4 h, m, l;
            split8(x, h, m, l);
            const uint32_t o = core_off16(aa, 8 * jg, 8);
            *reinterpret_cast<uint4 *>(sm + SMB_B + o) = h;
            *reinterpret_cast<uint4 *>(sm + SMB_B + BB_PART + o) = m;
            *reinterpret_cast<uint4 *>(sm + SMB_B + 2 * BB_PART + o) = l;
        }
    };
    // thread 0: D (over slot s) = the six products, small ones first; 4 K-steps of 16 each
    auto issue_mma = [&](int s) {
        const uint32_t dt = tbase + 64 * s;
        const int pa[6] = {2, 1, 0, 1, 0, 0}, pb[6] = {0, 1, 2, 0, 1, 0};
#pragma unroll
        for (int p = 0; p < 6; p++)
#pragma unroll
            for (int k = 0; k < 4; k++)
                mma_bf16(dt, dA[pa[p]] + 256 * k, dB[pb[p]] + 128 * k, idesc, (p > 0 || k > 0) ? 1u : 0u);
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                     :: "r"(barM) : "memory");
    };
    // v (or v *=) alpha + D for the internal child in slot s, alpha = h + m + l from the A operand
    auto child_value = [&](int s, float *v, bool mul) {
        const uint32_t tD = tbase + lane_off + 64 * s + s0;
#pragma unroll
        for (int q = 0; q < 2; q++) {
            float d[16];
            tmem_ld16(tD + 16 * q, d);
#pragma unroll
            for (int j8 = 0; j8 < 2; j8++) {
                const uint32_t o = core_off16(site, s0 + 16 * q + 8 * j8, 16);
                const uint4 h = *reinterpret_cast<const uint4 *>(sm + SMB_A + o);
                const uint4 m = *reinterpret_cast<const uint4 *>(sm + SMB_A + BA_PART + o);
                const uint4 l = *reinterpret_cast<const uint4 *>(sm + SMB_A + 2 * BA_PART + o);
                const uint32_t hw[4] = {h.x, h.y, h.z, h.w}, mw[4] = {m.x, m.y, m.z, m.w}, lw[4] = {l.x, l.y, l.z, l.w};
#pragma unroll
                for (int t = 0; t < 4; t++) {
                    const float x0 = (bf_lo(hw[t]) + bf_lo(mw[t])) + bf_lo(lw[t]);
                    const float x1 = (bf_hi(hw[t]) + bf_hi(mw[t])) + bf_hi(lw[t]);
                    const int j = 8 * j8 + 2 * t;
                    const float u0 = x0 + d[j], u1 = x1 + d[j + 1];
                    v[16 * q + j] = mul ? v[16 * q + j] * u0 : u0;
                    v[16 * q + j + 1] = mul ? v[16 * q + j + 1] * u1 : u1;
                }
            }
        }
    };
    // leaf child: v (or v *=) P_c[a][s] = E^T[s][a] + (a == s), 1 if marginalised
    auto leaf_value = [&](const float *Pc, int s, float *v, bool mul) {
        const float *row = Pc + (size_t)(s < K ? s : 0) * K + s0;
#pragma unroll
        for (int j8 = 0; j8 < 4; j8++) {
            float x[8];
            ldg8(row + 8 * j8, x);
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const float u = (s < K) ? x[k] + ((s == s0 + 8 * j8 + k) ? 1.0f : 0.0f) : 1.0f;
                v[8 * j8 + k] = mul ? v[8 * j8 + k] * u : u;
            }
        }
    };

    for (int w = blockIdx.x; w < a.nwi && ok; w += gridDim.x) {
        const WorkItem wi = a.wi[w];
        const Request rq = a.req[wi.request];
        const int md = rq.model;
        const float *Pbase = reinterpret_cast<const float *>(a.Pbuf) + (size_t)rq.pset * a.nbr * K2;
        const int ncols = wi.ncols;
        const uint8_t *lg = a.leaves + (size_t)wi.col0 * nl;
        __syncthreads();
        for (int f = tid; f < BF_M * nl; f += BF_THREADS) {
            const int c = f / nl, l = f - c * nl;
            lvT[l * BF_LVS + c] = (c < ncols) ? lg[f] : (uint8_t)K;
        }
        if (tid < K) {
            prf[tid] = (float)a.m.prior[md * K + tid];
            wlf[tid] = (float)a.m.wlog[md * K + tid];
        }
        __syncthreads();
        int escale = 0;
        for (int ni = 0; ni < a.n_internal && ok; ni++) {
            const SchedNode sn = sched[ni];
            float v[32];
            bool have = false, bad = false;
            int nc = 0;
            for (int side = 0; side < 2; side++) {
                const int s = side ? sn.rslot : sn.lslot;
                if (s < 0) continue;
                // the previous contraction's epilogue is finished with the operand buffers
                if (nc++ && __syncthreads_or(bad)) { ok = false; break; }
                stage_a(s);
                stage_b(Pbase + (size_t)(side ? sn.rc : sn.lc) * K2);
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                tc_fence_before();
                if (__syncthreads_or(bad)) { ok = false; break; }
                tc_fence_after();
                if (tid == 0) {
                    issue_mma(s);
                    mma_pending = true;
                }
                // the parity advances only with a completed phase, so that after a timed-out
                // wait the quiesce below waits for the commit still outstanding
                const bool done = mbar_wait(barM, ph_mma);
                tc_fence_after();
                if (!done) {
                    bad = true;
                } else {
                    ph_mma ^= 1u;
                    if (tid == 0) mma_pending = false;
                }
                child_value(s, v, have);
                have = true;
            }
            if (!ok) break;
            for (int side = 0; side < 2; side++) {
                if ((side ? sn.rslot : sn.lslot) >= 0) continue;
                const int c = side ? sn.rc : sn.lc;
                leaf_value(Pbase + (size_t)c * K2, lvT[c * BF_LVS + site], v, have);
                have = true;
            }
            // rescale by an exact power of two and park in the output slot
            float mx = 0.0f;
#pragma unroll
            for (int k = 0; k < 32; k++) mx = fmaxf(mx, v[k]);
            float (*cm)[BF_M] = cmax[ni & 1];
            cm[half][site] = mx;
            if (__syncthreads_or(bad)) { ok = false; break; }
            mx = fmaxf(cm[0][site], cm[1][site]);
            const int e = (mx > 0.0f) ? exp_of(mx) : 0;
            escale += e;
            const uint32_t tO = tbase + lane_off + 64 * sn.oslot + s0;
#pragma unroll
            for (int q = 0; q < 2; q++) {
                float y[16];
#pragma unroll
                for (int j = 0; j < 16; j++) y[j] = scale2(v[16 * q + j], -e);
                tmem_st16(tO + 16 * q, y);
            }
        }
        if (!ok) break;
        // root: z = alpha_root . prior (FP32, compensated) and the elpr term, as k_prune_tc
        float *zpart = reinterpret_cast<float *>(sm + SMB_A);   // [2][2][128]; the A operand is idle here
        __syncthreads();
        {
            const uint32_t tR = tbase + lane_off + 64 * sched[a.n_internal - 1].oslot + s0;
            float z = 0.0f, zc = 0.0f, wz = 0.0f;
            asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
#pragma unroll
            for (int q = 0; q < 2; q++) {
                float x[16];
                tmem_ld16(tR + 16 * q, x);
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    const float y = x[j] * prf[s0 + 16 * q + j] - zc;
                    const float t = z + y;
                    zc = (t - z) - y;
                    z = t;
                    wz = fmaf(x[j], wlf[s0 + 16 * q + j], wz);
                }
            }
            zpart[(half * 2 + 0) * BF_M + site] = z;
            zpart[(half * 2 + 1) * BF_M + site] = wz;
        }
        __syncthreads();
        if (half == 0) {
            double tl = 0.0, te = 0.0;
            if (site < ncols) {
                const float z = zpart[0 * BF_M + site] + zpart[2 * BF_M + site];
                const float wz = zpart[1 * BF_M + site] + zpart[3 * BF_M + site];
                if (z > 0.0f) {
                    int ez;
                    const float mz = frexpf(z, &ez);
                    tl = (double)logf(mz) + (double)(ez + escale) * 0.69314718055994530942;
                    te = (double)(wz / z);
                } else {
                    tl = -INFINITY;
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                tl += __shfl_down_sync(0xffffffffu, tl, o);
                te += __shfl_down_sync(0xffffffffu, te, o);
            }
            if ((tid & 31) == 0) { red_l[warp] = tl; red_e[warp] = te; }
        }
        tc_fence_before();
        __syncthreads();
        if (tid == 0) {
            double sl = 0.0, se = 0.0;
            for (int k = 0; k < BF_M / 32; k++) { sl += red_l[k]; se += red_e[k]; }
            a.partials[2 * (size_t)w] = sl;
            a.partials[2 * (size_t)w + 1] = se;
        }
    }
    if (!ok && tid == 0) atomicExch(err, 1);
    // quiesce: after a timed-out wait the commit may still arrive (bounded wait)
    if (__syncthreads_or(mma_pending)) mbar_wait(barM, ph_mma);
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tbase), "r"(tmem_cols));
}

uint32_t bf16_tmem_cols(int nslots)
{
    uint32_t need = (uint32_t)(64 * (nslots > 0 ? nslots : 1)), c = 64;
    while (c < need) c <<= 1;
    return c;
}

cudaError_t set_bf16_attributes(size_t smem)
{
    cudaError_t e = cudaFuncSetAttribute(k_prune_bf16, cudaFuncAttributePreferredSharedMemoryCarveout,
                                         (int)cudaSharedmemCarveoutMaxShared);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_prune_bf16, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    return e;
}

}  // namespace

size_t prune_bf16_smem_bytes(int nl, int nint)
{
    return SMB_LV + (((size_t)nl * BF_LVS + 15) & ~(size_t)15) + (size_t)nint * sizeof(SchedNode);
}

bool prune_bf16_supported(int nslots, int nl) { return nslots <= BF_MAX_SLOTS && nl <= BF_MAX_LEAVES; }

int prune_bf16_ctas_per_sm(int nslots, int nl, int nint)
{
    const int by_tmem = (int)(512 / bf16_tmem_cols(nslots));
    const size_t smem = prune_bf16_smem_bytes(nl, nint);
    cudaFuncAttributes fa;
    int dev = 0, smem_sm = 0, regs_sm = 0, reserved = 0;
    if (set_bf16_attributes(smem) != cudaSuccess || cudaFuncGetAttributes(&fa, k_prune_bf16) != cudaSuccess ||
        cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    const int by_smem = (int)((size_t)smem_sm / (fa.sharedSizeBytes + smem + (size_t)reserved));
    const int by_regs = regs_sm / (fa.numRegs * BF_THREADS);
    int n = by_tmem;
    if (by_smem < n) n = by_smem;
    if (by_regs < n) n = by_regs;
    return n > 0 ? n : 1;
}

cudaError_t launch_prune_bf16(const PruneArgs &a, int *err, cudaStream_t s, int grid)
{
    if (a.nwi <= 0) return cudaSuccess;
    const size_t smem = prune_bf16_smem_bytes(a.nl, a.n_internal);
    cudaError_t e = set_bf16_attributes(smem);
    if (e != cudaSuccess) return e;
    k_prune_bf16<<<grid, BF_THREADS, smem, s>>>(a, bf16_tmem_cols(a.nslots), err);
    return cudaGetLastError();
}

}  // namespace pcsf
