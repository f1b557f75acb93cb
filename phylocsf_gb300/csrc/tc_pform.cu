// Tensor-core P(t) formation for the search evaluations of the tensor-core
// engines (FP32 grid correction, see k_pform in kernels.cu):
//
//   E(t) = E(t_g) + C,   C[i][j] = sum_m isq_i U_im cf_m U_jm sq_j,
//   cf_m = e^{lam_m t_g} expm1(lam_m (t - t_g)),
//
// where C, at most 0.1 % of E, is the only arithmetic that needs a GEMM.  Two
// branches of one P set form one M = 128 tile (rows 64 b + i): A[row][m] =
// isq_i U_im cf_m (staged per pair, TF32 hi / lo), B[j][m] = U_jm sq_j (fixed
// per model, pre-split on the host and fetched once per CTA by bulk copy), and
// D = A_lo B_hi + A_hi B_lo + A_hi B_hi in tensor memory (kind::tf32, N = 64,
// K = 64).  Thread r owns row r: the epilogue adds E(t_g) (or forms the
// below-grid Taylor E = tQ + t^2 Q^2 / 2), applies the clamp / renormalise row
// rule of Q.ml:226-247 with the diagonal as the compensated sum of the row, and
// writes what the tensor-core pruning kernel reads: E^T for the branches above
// leaves (row gathers) and the pre-split B operand for the branches above
// internal nodes.
//
// One CTA (128 threads) per P set walks its branch pairs.  A_hi sits in tensor
// memory (columns 64..127, lane r = row r) and only A_lo in shared memory, so a CTA
// takes 64 KB of shared memory and 128 tensor-memory columns and three CTAs share an
// SM (the kernel is bound by the latency of its per-pair chain).  mbarrier waits are bounded as in the pruning
// kernel; on timeout the CTA records an error, waits (bounded) for its MMAs,
// frees its tensor memory and stops.
#include <cmath>
#include <cstdint>

#include "pcsf_internal.h"
#include "prune_common.cuh"
#include "tc_common.cuh"

namespace pcsf {

constexpr int PFT_THREADS = 128;
constexpr uint32_t PFT_B = 0;          // [hi, lo][64 x 64]   B = U^T D^1/2, 2 x 16 KB
constexpr uint32_t PFT_A = 32768;      // [128 x 64]  A_lo, 32 KB
constexpr uint32_t PFT_SMEM = 65536;
constexpr uint32_t PFT_TMEM_COLS = 128;   // D in 0..63, A_hi in 64..127
constexpr int PFT_MAX_BRANCHES = 320;

__global__ void __launch_bounds__(PFT_THREADS) k_pform_tc(const PSet *ps, const double *branch, int nbr, int nl,
                                                          DevModels m, const float *Bpf, float *Pbuf, float *Bop,
                                                          int32_t *status_key, int *err)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ uint32_t tbase_s;
    __shared__ __align__(8) uint64_t bar_mma, bar_b;
    __shared__ float cfs[2][K];
    __shared__ double exs[2][K];        // expm1(lam_m t) where w_m != 0 (row-sum check)
    __shared__ int mode_g[PFT_MAX_BRANCHES];      // per branch: grid point << 2 | mode
    __shared__ float t_b[PFT_MAX_BRANCHES];       // t (FP32: the Taylor branch and expm1f only)
    __shared__ float h_b[PFT_MAX_BRANCHES];       // t - t_g, formed in FP64

    const int tid = threadIdx.x;
    const int r = blockIdx.x;           // P set (chunk-local)
    const PSet rq = ps[r];
    const int md = rq.model;
    const uint32_t barM = smem_addr(&bar_mma), barB = smem_addr(&bar_b);
    const uint32_t sA = smem_addr(sm + PFT_A), sB = smem_addr(sm + PFT_B);
    const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);
    const float *Uf = m.Uf + (size_t)md * K2;
    const double *lam = m.lam + md * K;
    const double *wrow = m.wrow + md * K;
    const int i = tid & (K - 1), bsel = tid >> 6;      // this thread's row: branch b0 + bsel, state i

    if ((tid >> 5) == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_addr(&tbase_s)), "r"(PFT_TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(barM), "r"(1));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(barB), "r"(1));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = tbase_s;
    bool ok = true;
    if (tid == 0) {
        bulk_load(sB, Bpf + (size_t)md * 2 * K2, 2 * 16384, barB);
        ok = mbar_wait(barB, 0);
    }
    const uint32_t lane_off = (uint32_t)(((tid >> 5) & 3) * 32) << 16;
    uint32_t ph = 0;
    bool pending = false;               // an MMA group was issued and its completion not seen
    const float isq_i = (float)m.isq[md * K + i];
    // per branch: 0 t = 0, 1 below the grid (Taylor), 2 grid correction at point g
    for (int b = tid; b < nbr; b += PFT_THREADS) {
        const double t = rq.rho * branch[b];
        int mode = 0, g = 0;
        if (t == 0.0) mode = 0;
        else if (t < m.grid_t[0]) mode = 1;
        else {
            mode = 2;
            const double x = log(t / m.grid_t[0]) / m.grid_lr;
            g = (int)floor(x);
            if (g < 0) g = 0;
            if (g > m.grid_n - 1) g = m.grid_n - 1;
            if (g + 1 < m.grid_n && (m.grid_t[g + 1] - t) < (t - m.grid_t[g])) g++;
        }
        mode_g[b] = (g << 2) | mode;
        t_b[b] = (float)t;
        h_b[b] = (mode == 2) ? (float)(t - m.grid_t[g]) : 0.0f;
    }
    // FP32 copies of this thread's eigenvalue and its stationary-direction flag
    // (FP64 runs at a small fraction of the FP32 rate on this part)
    const float lam_i = (float)lam[i];
    bool listed = false;
    {
        const int16_t *wl = m.wlist + md * WLIST;
        if (wl[0] == -2) listed = (wrow[i] != 0.0);
        else
            for (int k = 0; k < WLIST; k++) listed |= (wl[k] == i);
    }
    const float ntol = -(float)m.tol, dtol = (float)(-1.0 - m.tol);

    for (int b0 = 0; b0 < nbr; b0 += 2) {
        const int b = b0 + bsel;                      // this thread's branch
        if (__syncthreads_or(!ok)) break;             // per-branch table ready / previous pair done
        const int mode = (b < nbr) ? (mode_g[b] & 3) : 0, g = (b < nbr) ? (mode_g[b] >> 2) : 0;
        const float t = (b < nbr) ? t_b[b] : 0.0f;
        {
            float cf = 0.0f;
            if (mode == 2) cf = m.grid_eg[((size_t)md * m.grid_n + g) * K + i] * expm1f(lam_i * h_b[b]);
            cfs[bsel][i] = cf;      // thread (bsel, i) supplies coefficient m = i
            exs[bsel][i] = listed ? (double)expm1f(lam_i * t) : 0.0;
        }
        __syncthreads();
        // ---- A operand: row tid = isq_i U_im cf_m, TF32 hi (tensor memory) / lo (shared)
        {
            const float4 *urow = reinterpret_cast<const float4 *>(Uf + (size_t)i * K);
#pragma unroll 1
            for (int c = 0; c < 4; c++) {
                float h[16];
#pragma unroll
                for (int q4 = 0; q4 < 4; q4++) {
                    const int q = 4 * c + q4;
                    const float4 u = __ldg(urow + q);
                    const float x0 = isq_i * u.x * cfs[bsel][4 * q], x1 = isq_i * u.y * cfs[bsel][4 * q + 1];
                    const float x2 = isq_i * u.z * cfs[bsel][4 * q + 2], x3 = isq_i * u.w * cfs[bsel][4 * q + 3];
                    const float4 hv = make_float4(tf32_hi(x0), tf32_hi(x1), tf32_hi(x2), tf32_hi(x3));
                    *reinterpret_cast<float4 *>(sm + PFT_A + core_off(tid, 4 * q, 16)) =
                        make_float4(x0 - hv.x, x1 - hv.y, x2 - hv.z, x3 - hv.w);
                    h[4 * q4] = hv.x; h[4 * q4 + 1] = hv.y; h[4 * q4 + 2] = hv.z; h[4 * q4 + 3] = hv.w;
                }
                tmem_st16(tbase + lane_off + 64 + 16 * c, h);
            }
            asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
            mma3_tf32_ta(tbase, tbase + 64, sA, sB, 16384, idesc);
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                         :: "r"(barM) : "memory");
        }
        // ---- epilogue inputs that do not depend on D, loaded while the MMAs run
        float row[K];
        {
            const float *eg = m.gridT + ((size_t)md * m.grid_n + g) * K2;   // E(t_g)^T
            const float *Qf = m.Qf + (size_t)md * K2 + (size_t)i * K, *Q2f = m.Q2f + (size_t)md * K2 + (size_t)i * K;
            const float tt = t, h2 = 0.5f * t * t;
#pragma unroll
            for (int j = 0; j < K; j++) {
                if (mode == 2) row[j] = __ldg(eg + (size_t)j * K + i);
                else if (mode == 1) row[j] = tt * Qf[j] + h2 * Q2f[j];
                else row[j] = 0.0f;
            }
        }
        pending = true;
        const bool done = mbar_wait(barM, ph);
        ph ^= 1u;
        if (done) pending = false;
        tc_fence_after();
        if (mode == 2) {
#pragma unroll
            for (int c = 0; c < 4; c++) {
                float d[16];
                tmem_ld16(tbase + lane_off + 16 * c, d);
#pragma unroll
                for (int j = 0; j < 16; j++) row[16 * c + j] += d[j];
            }
        }
        tc_fence_before();
        if (b < nbr && done) {
            // branch-free in j: i differs per lane, and a branch on j == i would split the
            // warp into single-lane paths for everything that follows
            bool neg = false;
            float diag = 0.0f, dc = 0.0f;
#pragma unroll
            for (int j = 0; j < K; j++) {
                const bool dj = (j == i);
                const float x0 = row[j];
                neg |= dj ? (x0 < dtol) : (x0 < ntol);
                const float x = fmaxf(x0, 0.0f);          // clamp an off-diagonal negative
                row[j] = dj ? x0 : x;
                const float y = -x - dc;                  // Kahan: diag -= x (off-diagonal only)
                const float s = diag + y;
                const float c = (s - diag) - y;
                diag = dj ? diag : s;
                dc = dj ? dc : c;
            }
#pragma unroll
            for (int j = 0; j < K; j++) row[j] = (j == i) ? diag : row[j];
            const double rs = rowsum_minus_one(m, md, i, exs[bsel]);
            if (neg) status_min(status_key + r, b, i, PCSF_ENEGP);
            else if (fabs(rs) > m.tol) status_min(status_key + r, b, i, PCSF_EROWSUM);
            else if (!(diag > -1.0f)) status_min(status_key + r, b, i, PCSF_EDIAG);
            if (b >= nl) {      // above an internal node: the pruning kernel's B operand
                float *dst = Bop + ((size_t)r * (nbr - nl) + (b - nl)) * 2 * K2;
#pragma unroll
                for (int q = 0; q < K / 4; q++)
                    bop_store(dst, i, q, make_float4(row[4 * q], row[4 * q + 1], row[4 * q + 2], row[4 * q + 3]));
            } else {            // above a leaf: E^T rows for the gathers
                float *out = Pbuf + ((size_t)r * nbr + b) * K2;
#pragma unroll
                for (int j = 0; j < K; j++) out[(size_t)j * K + i] = row[j];
            }
        }
        if (!done) ok = false;      // agreed on at the next pair's first barrier
        tc_fence_after();
    }
    if (__syncthreads_or(!ok)) ok = false;
    if (!ok && tid == 0) atomicExch(err, 1);
    if (pending) mbar_wait(barM, ph ^ 1u);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if ((tid >> 5) == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tbase), "r"(PFT_TMEM_COLS));
}

cudaError_t launch_pform_tc(const PSet *ps, int nps, const double *branch, int nbr, int nl, DevModels m,
                            const float *Bpf, float *Pbuf, float *Bop, int32_t *status_key, int *err, cudaStream_t s)
{
    if (nps <= 0) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(k_pform_tc, cudaFuncAttributePreferredSharedMemoryCarveout,
                                         (int)cudaSharedmemCarveoutMaxShared);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_pform_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)PFT_SMEM);
    if (e != cudaSuccess) return e;
    k_pform_tc<<<nps, PFT_THREADS, PFT_SMEM, s>>>(ps, branch, nbr, nl, m, Bpf, Pbuf, Bop, status_key, err);
    return cudaGetLastError();
}

}  // namespace pcsf
