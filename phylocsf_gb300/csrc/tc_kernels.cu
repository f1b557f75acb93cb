// Tensor-core (tcgen05, sm_103a) pruning kernel.
//
// Same contract as k_prune (kernels.cu) -- one work item is a tile of columns of
// one request's region, walked through the register-minimal schedule -- with the
// internal-branch contractions on the 5th-generation tensor cores:
//
//   D_c[site][a] = sum_j alpha_c[site][j] * E_c[a][j]      (M = 128 sites, N = 64, K = 64)
//
// as kind::tf32 MMAs with FP32 accumulation in tensor memory.  TF32 keeps 10
// mantissa bits, so each operand is split into hi = tf32(x) (the MMA ignores the
// low 13 bits) and lo = x - hi, and D = A_lo B_hi + A_hi B_lo + A_hi B_hi (the
// small products first), which restores ~22 bits.  The epilogue adds the exact
// identity part, v_c = alpha_c + D_c (E = P - I), so rounding in D only touches
// the off-diagonal mass of P.
//
// Layout: 256 threads; thread t owns tile column (site) t % 128, i.e. TMEM lane
// t % 128, and states 32*(t/128) .. +31 (warp w reaches lanes 32*(w%4)..).
// Tensor memory holds the partial slots as regions of 64 columns (at least four:
// 256 columns, so two CTAs share an SM).  A contraction has two forms:
//  - region form (a tensor-memory region holds no live partial): the hi part of
//    alpha_c is written back over the child's own slot and is the MMA's A operand
//    there, the lo part goes to shared memory, and D goes to the free region;
//  - shared form (every region is live, e.g. 6 of the 56 contractions of the
//    58-leaf tree): hi and lo both go to the shared-memory A operand and D is
//    written over the child's own slot.
// The region form moves 80 KB of shared-memory operand reads per contraction
// instead of 144 KB, and 64 KB of thread traffic instead of 128 KB.  Both forms issue
// the same MMAs in the same order on the same values, so their results are
// identical.  The epilogue reads alpha_c = hi + lo back from where the staging put
// them.  What bounds the kernel is the latency of the per-node chain (MMA issue and
// completion, the epilogue, the leaf gathers, the barriers), which the two CTAs on an
// SM overlap: the MMA descriptors are precomputed, the leaf rows are gathered with
// 256-bit loads, and while a node's MMAs run its threads prefetch into L1 the leaf
// rows of the next node.
//
// Shared memory (about 106 KB for 58 leaves, 112 KB for 100, so that two CTAs share an
// SM): one A operand (128 x 64, hi + lo), one B operand (64 x 64, hi + lo), the tile's
// leaf states and the schedule.
// The two children of a node are contracted one after the other through the
// same operand buffers.  B operands are pre-split by the P(t) kernel into this
// exact layout, so one elected thread fetches each with a single 32 KB bulk copy
// (cp.async.bulk, completion on an mbarrier), issued as soon as the previous
// contraction has released the buffer.  Leaf children are gathers of E^T rows
// from L2 while the MMAs run.  The per-column rescale exponent is the maximum
// over the two threads of a column.  The root stage forms z = pi . alpha as an FP32
// compensated dot product and log z = log m + e ln 2 (m in [0.5, 1)), with FP64
// only for the per-column log and the tile sums.
//
// Accuracy: the tensor cores' FP32 accumulation is not round-to-nearest: it
// rounds toward minus infinity (a measured mean of -5.7 ulp of the result over
// one K = 64 product, i.e. 8 accumulation steps, for positive and for negative
// results alike), so these values carry a small systematic error.  The engine
// therefore uses this kernel for the search evaluations of the rho maximisation
// and reports every returned likelihood from the compensated FP32 kernel.
//
// Every mbarrier wait is bounded; on timeout the kernel records an error, waits
// (again bounded) for its outstanding copies and tensor-core work, releases its
// tensor memory and exits.
#include <cmath>
#include <cstdint>

#include "pcsf_internal.h"
#include "prune_common.cuh"
#include "tc_common.cuh"

namespace pcsf {

constexpr int TCP_THREADS = 256;     // two threads per tile column
constexpr int TCP_M = 128;
constexpr int TCP_MAX_SLOTS = 8;     // 8 x 64 = all 512 tensor-memory columns
constexpr int TCP_MAX_LEAVES = 160;

// dynamic shared-memory map (bytes)
constexpr uint32_t SM_A = 0;            // [hi, lo][128 x 64 fp32] = 2 x 32 KB
constexpr uint32_t SM_B = 65536;        // [hi, lo][64 x 64 fp32]  = 2 x 16 KB
constexpr uint32_t SM_LV = 98304;       // [nl][LV_STRIDE] leaf states, then the schedule
constexpr uint32_t A_BYTES = 32768, B_BYTES = 16384;
// leaf-state rows padded by 4 bytes: the tile fill writes one byte per (site, leaf)
// with consecutive threads on consecutive leaves, which would otherwise all hit one bank
constexpr int LV_STRIDE = TCP_M;     // leaf-state rows: [leaf][site] bytes, words XOR-swizzled per row
// byte offset of (leaf l, site c): row l's 4-byte words are permuted by XOR with l mod 32,
// so that the fill (consecutive threads on consecutive leaves of one site) and the reads
// (consecutive threads on consecutive sites of one leaf) are both free of bank conflicts
// without padding the rows (whose bytes decide whether two CTAs fit an SM on 100 leaves)
__device__ __forceinline__ int lv_off(int l, int c) { return l * LV_STRIDE + (c ^ ((l & 31) << 2)); }


// alpha = hi + lo of this thread's 32 states, read back from the A operand
__device__ __forceinline__ void load_alpha(const unsigned char *sm, int site, int s0, int q, float *x)
{
#pragma unroll
    for (int j4 = 0; j4 < 4; j4++) {
        const uint32_t o = core_off(site, s0 + 16 * q + 4 * j4, 16);
        const float4 h = *reinterpret_cast<const float4 *>(sm + SM_A + o);
        const float4 l = *reinterpret_cast<const float4 *>(sm + SM_A + A_BYTES + o);
        x[4 * j4 + 0] = h.x + l.x;
        x[4 * j4 + 1] = h.y + l.y;
        x[4 * j4 + 2] = h.z + l.z;
        x[4 * j4 + 3] = h.w + l.w;
    }
}

// KEEP: each column's partial (alpha) stays in registers from the operand staging to
// the epilogue, which then reads only D (else the epilogue reads alpha back from the
// operands, and the second child's staging waits for a barrier that frees them).  Both
// shapes issue the same MMAs on the same operands and produce identical values; the
// engine's autotuner times them.
template <int NPROD, bool KEEP>
__global__ void __launch_bounds__(TCP_THREADS, 2) k_prune_tc(PruneArgs a, uint32_t tmem_cols, int *err)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ uint32_t tbase_s;
    __shared__ __align__(8) uint64_t bar_mma, bar_b;
    __shared__ float cmax[2][2][TCP_M];
    __shared__ double red_l[TCP_THREADS / 32], red_e[TCP_THREADS / 32];
    __shared__ int nbseq_s;

    const int tid = threadIdx.x, warp = tid >> 5;
    const int site = tid & (TCP_M - 1);          // tile column = TMEM lane
    const int half = tid >> 7;                    // states 32*half .. 32*half+31
    const int s0 = 32 * half;
    const int nl = a.nl;
    uint8_t *lvT = sm + SM_LV;
    SchedNode *sched = reinterpret_cast<SchedNode *>(sm + SM_LV + ((nl * LV_STRIDE + 15) & ~15));
    // per contraction (fewer than n_internal): the internal child, in order, and the free
    // tensor-memory region for D or -1
    int16_t *bseq = reinterpret_cast<int16_t *>(sched + a.n_internal);
    int8_t *dreg = reinterpret_cast<int8_t *>(bseq + a.n_internal);
    const uint32_t barM = smem_addr(&bar_mma), barB = smem_addr(&bar_b);
    const uint32_t sA = smem_addr(sm + SM_A), sB = smem_addr(sm + SM_B);
    // kind::tf32, D f32, A/B tf32, both K-major, N = 64, M = 128
    const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);
    const float *Bop = reinterpret_cast<const float *>(a.Bop);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_addr(&tbase_s)), "r"(tmem_cols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(barM), "r"(1));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(barB), "r"(1));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        // replay the schedule's slot occupancy: a contraction takes the region form
        // when some region holds no live partial (the contracted child's slot stays
        // live until its epilogue has read it)
        const uint32_t all = (tmem_cols >= 512) ? 0xFFu : ((1u << (tmem_cols / 64)) - 1u);
        uint32_t occ = 0;
        int k = 0;
        for (int f = 0; f < a.n_internal; f++) {
            const SchedNode sn = a.sched[f];
            for (int side = 0; side < 2; side++) {
                const int s = side ? sn.rslot : sn.lslot;
                if (s < 0) continue;
                const uint32_t fr = all & ~occ;
                bseq[k] = side ? sn.rc : sn.lc;
                dreg[k++] = fr ? (int8_t)(__ffs(fr) - 1) : (int8_t)-1;
                occ &= ~(1u << s);
            }
            occ |= 1u << sn.oslot;
        }
        nbseq_s = k;
    }
    for (int f = tid; f < a.n_internal; f += TCP_THREADS) sched[f] = a.sched[f];
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = tbase_s;
    const int nbseq = nbseq_s;
    const uint32_t lane_off = (uint32_t)((warp & 3) * 32) << 16;   // warp w reaches lanes 32*(w%4)..
    uint32_t ph_mma = 0, ph_b = 0;      // mbarrier parities (every thread tracks both)
    // B loads: (work item, index into bseq) of the next load to issue; thread 0 only
    int ld_w = blockIdx.x, ld_k = 0;
    int b_inflight = 0;                 // loads issued and not yet waited for (thread 0)
    bool ok = true;

    auto issue_next_b = [&]() {         // thread 0: the buffer is free
        while (ld_w < a.nwi && ld_k >= nbseq) { ld_w += gridDim.x; ld_k = 0; }
        if (ld_w >= a.nwi || nbseq == 0) return;
        const int ps = a.req[a.wi[ld_w].request].pset;
        const int c = bseq[ld_k++];
        bulk_load(sB, Bop + ((size_t)ps * a.nbop + (c - nl)) * 2 * K2, 2 * B_BYTES, barB);
        b_inflight++;
    };
    if (tid == 0) issue_next_b();

    // stage alpha of slot s (this thread's 32 states) as the A operand: lo to shared
    // memory; hi to shared memory (shared form) or back over slot s (region form); with
    // KEEP, alpha itself stays in al for the epilogue
    // (the output stores of earlier nodes are waited for here, before the first read)
    auto stage_a = [&](int s, bool region, float *al) {
        const uint32_t ts = tbase + lane_off + 64 * s + s0;
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
        if constexpr (KEEP) {
            tmem_ld16x2(ts, ts + 16, al, al + 16);
#pragma unroll
            for (int q = 0; q < 2; q++) {
                float h[16];
#pragma unroll
                for (int j4 = 0; j4 < 4; j4++) {
                    const float *y = al + 16 * q + 4 * j4;
                    const float4 hv = make_float4(tf32_hi(y[0]), tf32_hi(y[1]), tf32_hi(y[2]), tf32_hi(y[3]));
                    const float4 lv = make_float4(y[0] - hv.x, y[1] - hv.y, y[2] - hv.z, y[3] - hv.w);
                    const uint32_t o = core_off(site, s0 + 16 * q + 4 * j4, 16);
                    if (!region) *reinterpret_cast<float4 *>(sm + SM_A + o) = hv;
                    *reinterpret_cast<float4 *>(sm + SM_A + A_BYTES + o) = lv;
                    h[4 * j4] = hv.x; h[4 * j4 + 1] = hv.y; h[4 * j4 + 2] = hv.z; h[4 * j4 + 3] = hv.w;
                }
                if (region) tmem_st16(ts + 16 * q, h);
            }
            if (region) asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            return;
        }
        float x[32];
        tmem_ld16x2(ts, ts + 16, x, x + 16);
#pragma unroll
        for (int j4 = 0; j4 < 8; j4++) {
            const float4 hv = make_float4(tf32_hi(x[4 * j4]), tf32_hi(x[4 * j4 + 1]), tf32_hi(x[4 * j4 + 2]),
                                          tf32_hi(x[4 * j4 + 3]));
            const float4 lv = make_float4(x[4 * j4] - hv.x, x[4 * j4 + 1] - hv.y, x[4 * j4 + 2] - hv.z,
                                          x[4 * j4 + 3] - hv.w);
            const uint32_t o = core_off(site, s0 + 4 * j4, 16);
            if (!region) *reinterpret_cast<float4 *>(sm + SM_A + o) = hv;
            *reinterpret_cast<float4 *>(sm + SM_A + A_BYTES + o) = lv;
            x[4 * j4] = hv.x; x[4 * j4 + 1] = hv.y; x[4 * j4 + 2] = hv.z; x[4 * j4 + 3] = hv.w;
        }
        if (region) {
            tmem_st16(ts, x);
            tmem_st16(ts + 16, x + 16);
            asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    };
    // thread 0: wait for the B operand
    auto wait_b = [&]() -> bool {
        if (!mbar_wait(barB, ph_b)) return false;
        ph_b ^= 1u;
        b_inflight--;
        return true;
    };
    // thread 0, after the staging barrier: D = A B into region r (region form: A hi in
    // slot s) or over slot s (shared form, r < 0); the same MMA sequence either way
    // Descriptors of K-step k are the step-0 descriptors plus k times the step in
    // 16-byte units (A 4096 B, B 2048 B), so the issuing loop is adds only.
    const uint64_t dAhi = sdesc(sA, 2048, 128), dAlo = sdesc(sA + A_BYTES, 2048, 128);
    const uint64_t dBhi = sdesc(sB, 1024, 128), dBlo = sdesc(sB + B_BYTES, 1024, 128);
    auto issue_mma = [&](int s, int r) {
        const uint32_t dt = tbase + 64 * (r >= 0 ? r : s);
        const uint32_t ta = tbase + 64 * s;
        if (r >= 0) {
            if (NPROD == 3) {
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    mma_tf32(dt, dAlo + 256 * k, dBhi + 128 * k, idesc, k > 0);
                    mma_tf32_ta(dt, ta + 8 * k, dBlo + 128 * k, idesc, 1);
                }
            }
#pragma unroll
            for (int k = 0; k < 8; k++) mma_tf32_ta(dt, ta + 8 * k, dBhi + 128 * k, idesc, NPROD == 3 || k > 0);
        } else {
            if (NPROD == 3) {
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    mma_tf32(dt, dAlo + 256 * k, dBhi + 128 * k, idesc, k > 0);
                    mma_tf32(dt, dAhi + 256 * k, dBlo + 128 * k, idesc, 1);
                }
            }
#pragma unroll
            for (int k = 0; k < 8; k++) mma_tf32(dt, dAhi + 256 * k, dBhi + 128 * k, idesc, NPROD == 3 || k > 0);
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                     :: "r"(barM) : "memory");
    };
    // v (or v *=) alpha + D for the internal child in slot s, alpha from the registers
    // the staging filled (KEEP) or hi + lo from where the staging put them
    auto child_value = [&](int s, int r, const float *al, float *v, bool mul) {
        const uint32_t tD = tbase + lane_off + 64 * (r >= 0 ? r : s) + s0;
        const uint32_t tH = tbase + lane_off + 64 * s + s0;
#pragma unroll
        for (int q = 0; q < 2; q++) {
            float d[16], x[16];
            if constexpr (KEEP) {
                tmem_ld16(tD + 16 * q, d);
#pragma unroll
                for (int j = 0; j < 16; j++) x[j] = al[16 * q + j];
            } else if (r >= 0) {
                tmem_ld16x2(tD + 16 * q, tH + 16 * q, d, x);
#pragma unroll
                for (int j4 = 0; j4 < 4; j4++) {
                    const float4 l = *reinterpret_cast<const float4 *>(
                        sm + SM_A + A_BYTES + core_off(site, s0 + 16 * q + 4 * j4, 16));
                    x[4 * j4 + 0] += l.x;
                    x[4 * j4 + 1] += l.y;
                    x[4 * j4 + 2] += l.z;
                    x[4 * j4 + 3] += l.w;
                }
            } else {
                tmem_ld16(tD + 16 * q, d);
                load_alpha(sm, site, s0, q, x);
            }
#pragma unroll
            for (int j = 0; j < 16; j++) {
                const float u = x[j] + d[j];
                v[16 * q + j] = mul ? v[16 * q + j] * u : u;
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
    // the leaf beside an internal child in two steps: raw E^T row, then the identity
    // part (or 1 where marginalised)
    auto leaf_load = [&](const float *Pc, int s, float *v) {
        const float *row = Pc + (size_t)(s < K ? s : 0) * K + s0;
#pragma unroll
        for (int j8 = 0; j8 < 4; j8++) ldg8(row + 8 * j8, v + 8 * j8);
    };
    auto leaf_fix = [&](int s, float *v) {
#pragma unroll
        for (int j = 0; j < 32; j++) v[j] = (s < K) ? v[j] + ((s == s0 + j) ? 1.0f : 0.0f) : 1.0f;
    };

    for (int w = blockIdx.x; w < a.nwi && ok; w += gridDim.x) {
        const WorkItem wi = a.wi[w];
        const Request rq = a.req[wi.request];
        const int md = rq.model;
        const float *Pbase = reinterpret_cast<const float *>(a.Pbuf) + (size_t)rq.pset * a.nbr * K2;
        const int ncols = wi.ncols;
        const uint8_t *lg = a.leaves + (size_t)wi.col0 * nl;
        __syncthreads();
        for (int f = tid; f < TCP_M * nl; f += TCP_THREADS) {
            int c = f / nl, l = f - c * nl;
            lvT[lv_off(l, c)] = (c < ncols) ? lg[f] : (uint8_t)K;
        }
        __syncthreads();
        // warm L1 with the leaf rows (one 128-byte line per thread and leaf) of the node
        // after ni, while this node waits for its MMAs or its own gathers
        auto prefetch_next = [&](int ni) {
            if (ni + 1 >= a.n_internal) return;
            const SchedNode nx = sched[ni + 1];
            if (nx.lslot < 0) {
                const int sa = lvT[lv_off(nx.lc, site)];
                asm volatile("prefetch.global.L1 [%0];" :: "l"(Pbase + (size_t)nx.lc * K2 + (size_t)(sa < K ? sa : 0) * K + s0));
            }
            if (nx.rslot < 0) {
                const int sb = lvT[lv_off(nx.rc, site)];
                asm volatile("prefetch.global.L1 [%0];" :: "l"(Pbase + (size_t)nx.rc * K2 + (size_t)(sb < K ? sb : 0) * K + s0));
            }
        };
        int escale = 0;     // this column's sum of rescale exponents
        bool pend_bad = false;   // a timed-out wait seen since the last CTA-wide barrier
        int kc = 0;         // contractions so far (index into bseq / dreg)

        for (int ni = 0; ni < a.n_internal && ok; ni++) {
            const SchedNode sn = sched[ni];
            float v[32];
            // internal children are contracted one after the other (l before r); a
            // leaf child beside an internal one is gathered while the MMAs run, except by
            // warp 0, whose thread 0 issues them (all warps loading before the staging
            // measured slower).  Every barrier also agrees on a timed-out wait (bad), so
            // that all threads leave together.
            const int slotL = sn.lslot, slotR = sn.rslot;
            const int nint = (slotL >= 0) + (slotR >= 0);
            const int lfc = (slotL < 0) ? sn.lc : sn.rc;   // the leaf child when nint == 1
            // warp 0 (whose thread 0 issues the MMAs) loads its leaf rows before the staging
            int ls0 = K;
            if (nint == 1 && warp == 0) {
                ls0 = lvT[lv_off(lfc, site)];
                leaf_load(Pbase + (size_t)lfc * K2, ls0, v);
            }
            bool have = (nint == 1), bad = false;
            int nc = 0;
            for (int side = 0; side < 2; side++) {
                const int s = side ? slotR : slotL;
                if (s < 0) continue;
                // the A operand is free again (with KEEP it is once the MMAs have completed,
                // and the first child's D is read before the staging barrier below)
                if (!KEEP && nc && __syncthreads_or(bad)) { ok = false; break; }
                nc++;
                const int r = dreg[kc++];
                float al[KEEP ? 32 : 1];
                stage_a(s, r >= 0, al);
                if (tid == 0 && !wait_b()) bad = true;
                tc_fence_before();
                if (__syncthreads_or(bad || pend_bad)) { ok = false; break; }
                tc_fence_after();
                if (tid == 0) issue_mma(s, r);
                prefetch_next(ni);      // while the MMAs run
                if (nint == 1) {
                    if (warp != 0) {
                        ls0 = lvT[lv_off(lfc, site)];
                        leaf_load(Pbase + (size_t)lfc * K2, ls0, v);
                    }
                    leaf_fix(ls0, v);
                }
                const bool done = mbar_wait(barM, ph_mma);
                tc_fence_after();
                if (!done) bad = true;
                else ph_mma ^= 1u;   // after a timed-out wait the quiesce waits for this phase
                if (tid == 0 && done) issue_next_b();     // the B operand is free again
                child_value(s, r, al, v, have);
                have = true;
            }
            if (!ok) break;
            if (nint == 0) {
                leaf_value(Pbase + (size_t)sn.lc * K2, lvT[lv_off(sn.lc, site)], v, false);
                leaf_value(Pbase + (size_t)sn.rc * K2, lvT[lv_off(sn.rc, site)], v, true);
            }
            // ---- rescale by an exact power of two and park in the output slot
            float mx = 0.0f;
#pragma unroll
            for (int k = 0; k < 32; k++) mx = fmaxf(mx, v[k]);
            float (*cm)[TCP_M] = cmax[ni & 1];          // double-buffered: no second barrier needed
            cm[half][site] = mx;
            // only warps w and w + 4 share these columns: a named barrier of those 64 threads
            // (barriers 1-4; both warps walk the same schedule, so both always arrive).  A
            // timed-out wait is carried to the next CTA-wide barrier (the next staging, or the
            // root), which every thread reaches before any further MMA is issued.
            asm volatile("bar.sync %0, 64;" :: "r"(1 + (warp & 3)) : "memory");
            pend_bad |= bad;
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
        // ---- root: z = alpha_root . prior (FP32, compensated) and the elpr term per column;
        // log z = log m + e ln 2 with m in [0.5, 1) (logf of m is within ~4e-8 absolute,
        // far below the tensor-core noise of these search values); FP64 only for the
        // per-column log and the sums over the tile (this part's FP64 rate is ~1/64 of FP32)
        // (the A operand is idle here: [2][2][128] partial sums, then the model's prior and
        // prior * log prior in FP32)
        float *zpart = reinterpret_cast<float *>(sm + SM_A);
        float *prf = zpart + 4 * TCP_M, *wlf = prf + K;
        if (__syncthreads_or(pend_bad)) { ok = false; break; }   // every warp is past its last node
        if (tid < K) {
            prf[tid] = (float)a.m.prior[md * K + tid];
            wlf[tid] = (float)a.m.wlog[md * K + tid];
        }
        __syncthreads();
        {
            const uint32_t tR = tbase + lane_off + 64 * sched[a.n_internal - 1].oslot + s0;
            float z = 0.0f, zc = 0.0f, wz = 0.0f;
            asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");   // the root's output store
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
            zpart[(half * 2 + 0) * TCP_M + site] = z;
            zpart[(half * 2 + 1) * TCP_M + site] = wz;
        }
        __syncthreads();
        if (half == 0) {
            double tl = 0.0, te = 0.0;
            if (site < ncols) {
                const float z = zpart[0 * TCP_M + site] + zpart[2 * TCP_M + site];
                const float wz = zpart[1 * TCP_M + site] + zpart[3 * TCP_M + site];
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
            for (int k = 0; k < TCP_M / 32; k++) { sl += red_l[k]; se += red_e[k]; }
            a.partials[2 * (size_t)w] = sl;
            a.partials[2 * (size_t)w + 1] = se;
        }
    }
    if (!ok && tid == 0) atomicExch(err, 1);
    // quiesce: a bulk copy may be outstanding (loads run one ahead), and after a
    // timed-out MMA wait its commit may still arrive; both waits are bounded
    if (tid == 0) {
        while (b_inflight > 0) {
            if (!mbar_wait(barB, ph_b)) { atomicExch(err, 1); break; }
            ph_b ^= 1u;
            b_inflight--;
        }
    }
    if (!ok) mbar_wait(barM, ph_mma);
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tbase), "r"(tmem_cols));
}

static uint32_t tmem_cols_for(int nslots)
{
    // at least four regions, so that most contractions find a free one for D
    uint32_t need = (uint32_t)(64 * (nslots > 0 ? nslots : 1)), c = 256;
    while (c < need) c <<= 1;
    return c;
}

size_t prune_tc_smem_bytes(int nl, int nint)
{
    // operands, leaf states, the schedule, then per contraction the child and the D region
    return SM_LV + (((size_t)nl * LV_STRIDE + 15) & ~(size_t)15) + (size_t)nint * (sizeof(SchedNode) + 3);
}

bool prune_tc_supported(int nslots, int nl) { return nslots <= TCP_MAX_SLOTS && nl <= TCP_MAX_LEAVES; }

bool prune_tc_shape_ok(int shape) { return shape >= 0 && shape < PCSF_TC_SHAPES; }

template <int NPROD, bool KEEP>
static cudaError_t set_tc_attributes(size_t smem)
{
    // the whole unified L1 as shared memory, so that two CTAs of ~115 KB fit
    cudaError_t e = cudaFuncSetAttribute(k_prune_tc<NPROD, KEEP>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                         (int)cudaSharedmemCarveoutMaxShared);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_prune_tc<NPROD, KEEP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    return e;
}

// CTAs per SM: the smaller of what shared memory and registers allow (from the
// kernel's attributes and the device limits) and what tensor memory allows
template <bool KEEP>
static int ctas_per_sm(int nslots, int nl, int nint)
{
    const uint32_t cols = tmem_cols_for(nslots);
    const int by_tmem = (int)(512 / cols);
    const size_t smem = prune_tc_smem_bytes(nl, nint);
    cudaFuncAttributes fa, fa1;
    int dev = 0, smem_sm = 0, regs_sm = 0, reserved = 0;
    if (set_tc_attributes<3, KEEP>(smem) != cudaSuccess || set_tc_attributes<1, KEEP>(smem) != cudaSuccess ||
        cudaFuncGetAttributes(&fa, k_prune_tc<3, KEEP>) != cudaSuccess ||
        cudaFuncGetAttributes(&fa1, k_prune_tc<1, KEEP>) != cudaSuccess || cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev) != cudaSuccess)
        return 1;
    const size_t stat = fa.sharedSizeBytes > fa1.sharedSizeBytes ? fa.sharedSizeBytes : fa1.sharedSizeBytes;
    const int regs = fa.numRegs > fa1.numRegs ? fa.numRegs : fa1.numRegs;
    const int by_smem = (int)((size_t)smem_sm / (stat + smem + (size_t)reserved));
    const int by_regs = regs_sm / (regs * TCP_THREADS);
    int n = by_tmem;
    if (by_smem < n) n = by_smem;
    if (by_regs < n) n = by_regs;
    return n > 0 ? n : 1;
}

// shapes: 0 = alpha kept in registers, 1 = alpha read back from the operands
int prune_tc_ctas_per_sm(int nslots, int nl, int nint, int shape)
{
    return shape == 1 ? ctas_per_sm<false>(nslots, nl, nint) : ctas_per_sm<true>(nslots, nl, nint);
}

template <int NPROD, bool KEEP>
static cudaError_t launch_tc(const PruneArgs &a, int *err, cudaStream_t s, int grid)
{
    const size_t smem = prune_tc_smem_bytes(a.nl, a.n_internal);
    cudaError_t e = set_tc_attributes<NPROD, KEEP>(smem);
    if (e != cudaSuccess) return e;
    k_prune_tc<NPROD, KEEP><<<grid, TCP_THREADS, smem, s>>>(a, tmem_cols_for(a.nslots), err);
    return cudaGetLastError();
}

cudaError_t launch_prune_tc(int nprod, const PruneArgs &a, int *err, cudaStream_t s, int grid)
{
    if (a.nwi <= 0) return cudaSuccess;
    const bool keep = a.tc_shape != 1;
    if (nprod == 3) return keep ? launch_tc<3, true>(a, err, s, grid) : launch_tc<3, false>(a, err, s, grid);
    return keep ? launch_tc<1, true>(a, err, s, grid) : launch_tc<1, false>(a, err, s, grid);
}

}  // namespace pcsf
