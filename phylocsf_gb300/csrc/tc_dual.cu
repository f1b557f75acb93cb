// Tensor-core tangent pass: lpr and d lpr / d rho of each request in one sweep
// of the tree (forward-mode differentiation of the pruning recursion), for the
// derivative rule of the reduced-precision rho maximisation.
//
// With every branch scaled by rho, P_c = exp(rho b_c Q) and dP_c / d rho =
// b_c Q P_c (Q.ml:260-275).  Each partial carries its tangent:
//   internal child c:  v_c = alpha_c + E_c alpha_c
//                      u_c = alpha'_c + E_c alpha'_c + b_c Q v_c
//   leaf child c (state s):  v_c = P_c[:, s],  u_c = b_c Q v_c
//   node:              alpha_p = v_l v_r,  alpha'_p = u_l v_r + v_l u_r
// and per column d lpr / d rho = (pi . alpha'_root) / (pi . alpha_root) (a
// common power-of-two rescale of alpha and alpha' cancels).
//
// The three contractions of an internal child and the one of a leaf child run
// on the tensor cores exactly as in k_prune_tc (kind::tf32, TF32 hi / lo split,
// M = 128 columns, N = K = 64): B = E_c (the pre-split operand written by the
// P(t) kernel, bulk-copied) or B = Q of the request's model (both models' Q
// operands staged once per CTA).  Tensor memory holds alpha and alpha' of each
// partial slot (128 columns per slot), so trees with at most four slots fit
// (12flies, 29mammals, 58mammals, 100vertebrates); each MMA writes its D over
// columns whose contents were already read.  One CTA of 512 threads per SM,
// four threads per tile column (16 states each), so that the values and
// tangents of both children stay in registers.
//
// The tangent only steers the search (it values Brent's smallest probes), so
// the tensor cores' directed rounding (see tc_kernels.cu) is acceptable here.
// Every mbarrier wait is bounded, with the same exit protocol as k_prune_tc.
#include <cmath>
#include <cstdint>

#include "pcsf_internal.h"
#include "prune_common.cuh"
#include "tc_common.cuh"

namespace pcsf {

constexpr int TD_THREADS = 512;
constexpr int TD_NS = 16;            // states per thread
constexpr int TD_M = 128;
constexpr int TD_MAX_SLOTS = 4;
constexpr int TD_MAX_LEAVES = 160;

// dynamic shared-memory map (bytes)
constexpr uint32_t TD_A = 0;             // [hi, lo][128 x 64]    2 x 32 KB
constexpr uint32_t TD_BE = 65536;        // [hi, lo][64 x 64]     E_c, 2 x 16 KB
constexpr uint32_t TD_BQ = 98304;        // [model][hi, lo][64 x 64]  Q, 2 x 2 x 16 KB
constexpr uint32_t TD_LV = 163840;       // [nl][128] leaf states, then the schedule
constexpr uint32_t TD_ABYTES = 32768, TD_BBYTES = 16384;
// leaf-state rows padded by 4 bytes (the tile fill writes consecutive leaves from consecutive threads)
constexpr int TD_LVS = TD_M + 4;

__device__ __forceinline__ void td_load_alpha(const unsigned char *sm, int site, int s0, float *x)
{
#pragma unroll
    for (int j4 = 0; j4 < 4; j4++) {
        const uint32_t o = core_off(site, s0 + 4 * j4, 16);
        const float4 h = *reinterpret_cast<const float4 *>(sm + TD_A + o);
        const float4 l = *reinterpret_cast<const float4 *>(sm + TD_A + TD_ABYTES + o);
        x[4 * j4 + 0] = h.x + l.x;
        x[4 * j4 + 1] = h.y + l.y;
        x[4 * j4 + 2] = h.z + l.z;
        x[4 * j4 + 3] = h.w + l.w;
    }
}

// this thread's 16 values as the A operand (TF32 hi / lo)
__device__ __forceinline__ void td_store_a(unsigned char *sm, int site, int s0, const float *x)
{
#pragma unroll
    for (int j4 = 0; j4 < 4; j4++) {
        const float4 hv = make_float4(tf32_hi(x[4 * j4]), tf32_hi(x[4 * j4 + 1]), tf32_hi(x[4 * j4 + 2]),
                                      tf32_hi(x[4 * j4 + 3]));
        const float4 lv = make_float4(x[4 * j4] - hv.x, x[4 * j4 + 1] - hv.y, x[4 * j4 + 2] - hv.z,
                                      x[4 * j4 + 3] - hv.w);
        const uint32_t o = core_off(site, s0 + 4 * j4, 16);
        *reinterpret_cast<float4 *>(sm + TD_A + o) = hv;
        *reinterpret_cast<float4 *>(sm + TD_A + TD_ABYTES + o) = lv;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void td_mma3(uint32_t dt, uint32_t sA, uint32_t sB, uint32_t idesc)
{
    mma3_tf32(dt, sA, TD_ABYTES, sB, TD_BBYTES, idesc, false);
}

__global__ void __launch_bounds__(TD_THREADS, 1) k_prune_tc_dual(PruneArgs a, const float *Qop, const double *branch,
                                                                  double *dpart, int *err)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ uint32_t tbase_s;
    __shared__ __align__(8) uint64_t bar_mma, bar_b, bar_q;
    __shared__ float cmax[2][4][TD_M];
    __shared__ double red[3][TD_THREADS / 32];
    __shared__ int16_t bseq[TD_MAX_LEAVES];
    __shared__ float blen[2 * TD_MAX_LEAVES];     // branch lengths b_c (FP32)
    __shared__ int nbseq_s;
    __shared__ float prf[K], wlf[K];             // this work item's model: prior, prior * log prior (FP32)

    const int tid = threadIdx.x, warp = tid >> 5;
    const int site = tid & (TD_M - 1);
    const int quarter = tid >> 7;                 // states 16*quarter .. +15
    const int s0 = TD_NS * quarter;
    const int nl = a.nl;
    uint8_t *lvT = sm + TD_LV;
    SchedNode *sched = reinterpret_cast<SchedNode *>(sm + TD_LV + ((nl * TD_LVS + 15) & ~15));
    const uint32_t barM = smem_addr(&bar_mma), barB = smem_addr(&bar_b), barQ = smem_addr(&bar_q);
    const uint32_t sA = smem_addr(sm + TD_A), sBE = smem_addr(sm + TD_BE), sBQ = smem_addr(sm + TD_BQ);
    const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);
    const float *Bop = reinterpret_cast<const float *>(a.Bop);
    const uint32_t tmem_cols = 512;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_addr(&tbase_s)), "r"(tmem_cols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(barM), "r"(1));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(barB), "r"(1));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(barQ), "r"(1));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        int k = 0;
        for (int f = 0; f < a.n_internal; f++) {
            const SchedNode sn = a.sched[f];
            if (sn.lslot >= 0) bseq[k++] = sn.lc;
            if (sn.rslot >= 0) bseq[k++] = sn.rc;
        }
        nbseq_s = k;
    }
    for (int f = tid; f < a.n_internal; f += TD_THREADS) sched[f] = a.sched[f];
    for (int f = tid; f < a.nbr; f += TD_THREADS) blen[f] = (float)branch[f];
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = tbase_s;
    const int nbseq = nbseq_s;
    const uint32_t lane_off = (uint32_t)((warp & 3) * 32) << 16;
    uint32_t ph_mma = 0, ph_b = 0;
    int ld_w = blockIdx.x, ld_k = 0, b_inflight = 0;
    bool ok = true, bad = false;

    // both models' Q operands, once
    if (tid == 0) {
        bulk_load(sBQ, Qop, 4 * TD_BBYTES, barQ);
        if (!mbar_wait(barQ, 0)) bad = true;
    }
    auto issue_next_b = [&]() {
        while (ld_w < a.nwi && ld_k >= nbseq) { ld_w += gridDim.x; ld_k = 0; }
        if (ld_w >= a.nwi || nbseq == 0) return;
        const int ps = a.req[a.wi[ld_w].request].pset;
        const int c = bseq[ld_k++];
        bulk_load(sBE, Bop + ((size_t)ps * a.nbop + (c - nl)) * 2 * K2, 2 * TD_BBYTES, barB);
        b_inflight++;
    };
    if (tid == 0 && !bad) issue_next_b();
    if (__syncthreads_or(bad)) ok = false;

    // one MMA group D(cols) = A B and its completion; false on a timed-out wait
    // (A must be staged and fenced by every thread before the call)
    // warms L1 with the next node's leaf rows; set per node (none at the last node)
    const float *pf_a = nullptr, *pf_b = nullptr;
    auto pf_next_impl = [&]() {
        if (pf_a) asm volatile("prefetch.global.L1 [%0];" :: "l"(pf_a));
        if (pf_b) asm volatile("prefetch.global.L1 [%0];" :: "l"(pf_b));
    };
    bool pf_on = false;
    auto pf_next = [&]() { if (pf_on) pf_next_impl(); };
    auto run_mma = [&](uint32_t cols, uint32_t sB, bool need_e) -> bool {
        bool okb = true;
        if (tid == 0 && need_e) {
            okb = mbar_wait(barB, ph_b);
            if (okb) { ph_b ^= 1u; b_inflight--; }
        }
        tc_fence_before();
        if (__syncthreads_or(!okb)) return false;
        tc_fence_after();
        if (tid == 0) {
            td_mma3(tbase + cols, sA, sB, idesc);
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                         :: "r"(barM) : "memory");
        }
        pf_next();                       // while the MMAs run
        const bool done = mbar_wait(barM, ph_mma);
        if (done) ph_mma ^= 1u;   // after a timed-out wait the quiesce waits for this phase
        tc_fence_after();
        return done;
    };
    auto stage_slot = [&](uint32_t cols) {   // TMEM columns -> A operand
        float x[TD_NS];
        tmem_ld16(tbase + lane_off + cols + s0, x);
        td_store_a(sm, site, s0, x);
    };
    // leaf child c: P_c[:, s] for this thread's states (1 for a marginalised leaf)
    auto leaf_col = [&](const float *Pbase, int c, float *v) {
        const int st = lvT[c * TD_LVS + site];
        const float *row = Pbase + (size_t)c * K2 + (size_t)(st < K ? st : 0) * K + s0;
#pragma unroll
        for (int j8 = 0; j8 < TD_NS / 8; j8++) {
            float x[8];
            ldg8(row + 8 * j8, x);
#pragma unroll
            for (int k = 0; k < 8; k++)
                v[8 * j8 + k] = (st < K) ? x[k] + ((st == s0 + 8 * j8 + k) ? 1.0f : 0.0f) : 1.0f;
        }
    };
    // x = A (hi + lo) + D(cols)
    auto add_d = [&](uint32_t cols, float *x) {
        float d[TD_NS], al[TD_NS];
        tmem_ld16(tbase + lane_off + cols + s0, d);
        td_load_alpha(sm, site, s0, al);
#pragma unroll
        for (int j = 0; j < TD_NS; j++) x[j] = al[j] + d[j];
    };
    // u (+)= scale * D(cols)
    auto acc_d = [&](uint32_t cols, float scale, float *u, bool init) {
        float d[TD_NS];
        tmem_ld16(tbase + lane_off + cols + s0, d);
#pragma unroll
        for (int j = 0; j < TD_NS; j++) u[j] = init ? scale * d[j] : u[j] + scale * d[j];
    };

    for (int w = blockIdx.x; w < a.nwi && ok; w += gridDim.x) {
        const WorkItem wi = a.wi[w];
        const Request rq = a.req[wi.request];
        const int md = rq.model;
        const float *Pbase = reinterpret_cast<const float *>(a.Pbuf) + (size_t)rq.pset * a.nbr * K2;
        const uint32_t sQ = sBQ + (uint32_t)md * 2 * TD_BBYTES;
        const int ncols = wi.ncols;
        const uint8_t *lg = a.leaves + (size_t)wi.col0 * nl;
        __syncthreads();
        for (int f = tid; f < TD_M * nl; f += TD_THREADS) {
            int c = f / nl, l = f - c * nl;
            lvT[l * TD_LVS + c] = (c < ncols) ? lg[f] : (uint8_t)K;
        }
        if (tid < K) {
            prf[tid] = (float)a.m.prior[md * K + tid];
            wlf[tid] = (float)a.m.wlog[md * K + tid];
        }
        __syncthreads();
        int escale = 0;

        for (int ni = 0; ni < a.n_internal && ok; ni++) {
            const SchedNode sn = sched[ni];
            // v1 / u1: value and tangent of the first child, then of the node; vt: second child's value.
            // Internal children first; the node's tangent is folded in as the second child's parts
            // arrive (u_p = u_1 v_2 + v_1 u_2), which keeps three 16-value arrays live.
            pf_on = ni + 1 < a.n_internal;
            pf_a = pf_b = nullptr;
            if (pf_on) {
                const SchedNode nx = sched[ni + 1];
                if (nx.lslot < 0) {
                    const int st = lvT[nx.lc * TD_LVS + site];
                    pf_a = Pbase + (size_t)nx.lc * K2 + (size_t)(st < K ? st : 0) * K + s0;
                }
                if (nx.rslot < 0) {
                    const int st = lvT[nx.rc * TD_LVS + site];
                    pf_b = Pbase + (size_t)nx.rc * K2 + (size_t)(st < K ? st : 0) * K + s0;
                }
            }
            float v1[TD_NS], u1[TD_NS], vt[TD_NS];
            const bool int0 = sn.lslot >= 0 || sn.rslot >= 0;        // is the first child internal?
            const int cA = (sn.lslot >= 0 || sn.rslot < 0) ? sn.lc : sn.rc;
            const int cB = (cA == sn.lc) ? sn.rc : sn.lc;
            const int sA_ = (cA == sn.lc) ? sn.lslot : sn.rslot, sB_ = (cA == sn.lc) ? sn.rslot : sn.lslot;
            const uint32_t scratch = int0 ? 128u * (uint32_t)sA_ : 128u * (uint32_t)sn.oslot;
            // ---- first child
            if (int0) {
                const uint32_t ca = 128u * sA_, cd = ca + 64u;
                stage_slot(ca);
                if (!run_mma(ca, sBE, true)) bad = true;
                add_d(ca, v1);                                   // v = alpha + E alpha
                if (__syncthreads_or(bad)) { ok = false; break; }
                stage_slot(cd);
                if (!run_mma(cd, sBE, false)) bad = true;
                if (tid == 0 && !bad) issue_next_b();
                add_d(cd, u1);                                   // alpha' + E alpha'
                if (__syncthreads_or(bad)) { ok = false; break; }
                td_store_a(sm, site, s0, v1);
                if (!run_mma(ca, sQ, false)) bad = true;
                acc_d(ca, blen[cA], u1, false);                  // + b Q v
            } else {
                leaf_col(Pbase, cA, v1);
                td_store_a(sm, site, s0, v1);
                if (!run_mma(scratch, sQ, false)) bad = true;
                acc_d(scratch, blen[cA], u1, true);              // u = b Q v
            }
            if (__syncthreads_or(bad)) { ok = false; break; }    // the A operand is free again
            // ---- second child
            if (sB_ >= 0) {
                const uint32_t ca = 128u * sB_, cd = ca + 64u;
                stage_slot(ca);
                if (!run_mma(ca, sBE, true)) bad = true;
                add_d(ca, vt);
#pragma unroll
                for (int k = 0; k < TD_NS; k++) u1[k] *= vt[k];   // u_1 v_2
                if (__syncthreads_or(bad)) { ok = false; break; }
                stage_slot(cd);
                if (!run_mma(cd, sBE, false)) bad = true;
                if (tid == 0 && !bad) issue_next_b();
                {
                    float w[TD_NS];
                    add_d(cd, w);
#pragma unroll
                    for (int k = 0; k < TD_NS; k++) u1[k] += v1[k] * w[k];   // v_1 (alpha' + E alpha')
                }
                if (__syncthreads_or(bad)) { ok = false; break; }
                td_store_a(sm, site, s0, vt);
                if (!run_mma(ca, sQ, false)) bad = true;
                {
                    float d[TD_NS];
                    tmem_ld16(tbase + lane_off + ca + s0, d);
                    const float bb = blen[cB];
#pragma unroll
                    for (int k = 0; k < TD_NS; k++) u1[k] += v1[k] * (bb * d[k]);   // v_1 b Q v_2
                }
            } else {
                leaf_col(Pbase, cB, vt);
#pragma unroll
                for (int k = 0; k < TD_NS; k++) u1[k] *= vt[k];
                td_store_a(sm, site, s0, vt);
                if (!run_mma(scratch, sQ, false)) bad = true;
                float d[TD_NS];
                tmem_ld16(tbase + lane_off + scratch + s0, d);
                const float bb = blen[cB];
#pragma unroll
                for (int k = 0; k < TD_NS; k++) u1[k] += v1[k] * (bb * d[k]);
            }
            float mx = 0.0f;
#pragma unroll
            for (int k = 0; k < TD_NS; k++) {
                v1[k] *= vt[k];
                mx = fmaxf(mx, v1[k]);
            }
            float (*cm)[TD_M] = cmax[ni & 1];
            cm[quarter][site] = mx;
            if (__syncthreads_or(bad)) { ok = false; break; }
            mx = fmaxf(fmaxf(cm[0][site], cm[1][site]), fmaxf(cm[2][site], cm[3][site]));
            const int e = (mx > 0.0f) ? exp_of(mx) : 0;
            escale += e;
            const uint32_t tO = tbase + lane_off + 128u * sn.oslot + s0;
            {
                float y[TD_NS], z[TD_NS];
#pragma unroll
                for (int j = 0; j < TD_NS; j++) {
                    y[j] = scale2(v1[j], -e);
                    z[j] = scale2(u1[j], -e);
                }
                tmem_st16(tO, y);
                tmem_st16(tO + 64, z);
            }
            asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
        }
        if (!ok) break;
        // ---- root: z = pi . alpha, z' = pi . alpha', elpr term: FP32 compensated dot
        // products, log z = log m + e ln 2 with m in [0.5, 1); FP64 for the per-column
        // log and the sums over the tile only (as in k_prune_tc)
        float *zpart = reinterpret_cast<float *>(sm + TD_A);   // [4][3][128]; the A operand is idle
        __syncthreads();
        {
            const uint32_t tR = tbase + lane_off + 128u * sched[a.n_internal - 1].oslot + s0;
            float z = 0.0f, zc = 0.0f, wz = 0.0f, dz = 0.0f, dzc = 0.0f;
            float x[TD_NS], xd[TD_NS];
            tmem_ld16(tR, x);
            tmem_ld16(tR + 64, xd);
#pragma unroll
            for (int j = 0; j < TD_NS; j++) {
                const float p = prf[s0 + j];
                float y = x[j] * p - zc, t = z + y;
                zc = (t - z) - y;
                z = t;
                y = xd[j] * p - dzc;
                t = dz + y;
                dzc = (t - dz) - y;
                dz = t;
                wz = fmaf(x[j], wlf[s0 + j], wz);
            }
            zpart[(quarter * 3 + 0) * TD_M + site] = z;
            zpart[(quarter * 3 + 1) * TD_M + site] = wz;
            zpart[(quarter * 3 + 2) * TD_M + site] = dz;
        }
        __syncthreads();
        if (quarter == 0) {
            double tl = 0.0, te = 0.0, td = 0.0;
            if (site < ncols) {
                float z = 0.0f, wz = 0.0f, dz = 0.0f;
                for (int qq = 0; qq < 4; qq++) {     // fixed order
                    z += zpart[(qq * 3 + 0) * TD_M + site];
                    wz += zpart[(qq * 3 + 1) * TD_M + site];
                    dz += zpart[(qq * 3 + 2) * TD_M + site];
                }
                if (z > 0.0f) {
                    int ez;
                    const float mz = frexpf(z, &ez);
                    tl = (double)logf(mz) + (double)(ez + escale) * 0.69314718055994530942;
                    te = (double)(wz / z);
                    td = (double)(dz / z);
                } else {
                    tl = -INFINITY;
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                tl += __shfl_down_sync(0xffffffffu, tl, o);
                te += __shfl_down_sync(0xffffffffu, te, o);
                td += __shfl_down_sync(0xffffffffu, td, o);
            }
            if ((tid & 31) == 0) { red[0][warp] = tl; red[1][warp] = te; red[2][warp] = td; }
        }
        tc_fence_before();
        __syncthreads();
        if (tid == 0) {
            double sl = 0.0, se = 0.0, sd = 0.0;
            for (int k = 0; k < TD_M / 32; k++) { sl += red[0][k]; se += red[1][k]; sd += red[2][k]; }
            a.partials[2 * (size_t)w] = sl;
            a.partials[2 * (size_t)w + 1] = se;
            dpart[2 * (size_t)w] = sd;
            dpart[2 * (size_t)w + 1] = 0.0;
        }
    }
    if (!ok && tid == 0) atomicExch(err, 1);
    if (tid == 0) {
        while (b_inflight > 0) {
            if (!mbar_wait(barB, ph_b)) { atomicExch(err, 1); break; }
            ph_b ^= 1u;
            b_inflight--;
        }
    }
    if (!ok) mbar_wait(barM, ph_mma);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tbase), "r"(tmem_cols));
}

size_t prune_tc_dual_smem_bytes(int nl, int nint)
{
    return TD_LV + (((size_t)nl * TD_LVS + 15) & ~(size_t)15) + (size_t)nint * sizeof(SchedNode);
}

bool prune_tc_dual_supported(int nslots, int nl) { return nslots <= TD_MAX_SLOTS && nl <= TD_MAX_LEAVES; }

cudaError_t launch_prune_tc_dual(const PruneArgs &a, const float *Qop, const double *branch, double *dpart, int *err,
                                 cudaStream_t s, int grid)
{
    if (a.nwi <= 0) return cudaSuccess;
    const size_t smem = prune_tc_dual_smem_bytes(a.nl, a.n_internal);
    cudaError_t e = cudaFuncSetAttribute(k_prune_tc_dual, cudaFuncAttributePreferredSharedMemoryCarveout,
                                         (int)cudaSharedmemCarveoutMaxShared);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_prune_tc_dual, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_prune_tc_dual<<<grid, TD_THREADS, smem, s>>>(a, Qop, branch, dpart, err);
    return cudaGetLastError();
}

}  // namespace pcsf
