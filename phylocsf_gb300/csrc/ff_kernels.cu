// Float-float SIMT pruning: returned likelihoods that agree with the FP64 path
// to about 1e-12 relative, at FP32 instruction rates.
//
// The FP32 kernels round every stored partial and every contraction to 24 bits.
// Over a long region those errors add up partly coherently (columns that share
// sub-patterns repeat them), and the model's P(t) stored in FP32 is itself a fixed
// perturbation that every column sees; together they grow linearly with the
// region's length, past 1e-3 dB at a few thousand codons on trees of ~100 leaves.
// This kernel instead carries every quantity as an unevaluated sum of two floats
// (hi + lo, ~48 bits):
//   - E^T = (P - I)^T comes from the FP64 P(t) formation (the FP64 engine's own
//     matrices, row rule of Q.ml:226-247 applied in FP64), split once per P set into
//     hi / lo floats (k_split_ff) and staged into shared memory asynchronously, one
//     node ahead;
//   - a leaf child's partial P[a][s] = delta_as + E[a][s] is formed from the split
//     entries with an error-free sum (PhyloLik.ml:87-88 with a one-hot leaf);
//   - an internal child's v = alpha + sum_j E[a][j] alpha[j] (PhyloLik.ml:89-92)
//     is a compensated dot product: each hi x hi product is split exactly
//     (TwoProduct by FMA), its hi part is added with TwoSum, and the product
//     errors with the TwoSum errors, and the two hi x lo cross terms, are summed in
//     three separate low accumulators (short dependency chains), added at the end;
//   - node products alpha = v_l * v_r are float-float products;
//   - each column is rescaled by an exact power of two after every node;
//   - the root dot with the prior, the log and the tile sums are FP64.
// The error-free steps use __fadd_rn / __fmul_rn, which the compiler never fuses
// into an FMA (a fused form would break the exactness the transforms rely on).  The
// kernel has no FP64 arithmetic outside the root stage: FP64 runs at 1/64 of the FP32
// rate on this part, and splitting the staged doubles in every tile had cost more
// than the contractions themselves.
#include <algorithm>

#include "pcsf_internal.h"
#include "prune_common.cuh"

namespace pcsf {

namespace {

constexpr int FF_THREADS = 256;
constexpr int FF_TC = 16;            // columns per tile (1 per thread): ~98 KB of shared memory, two CTAs per SM
constexpr int FF_CPT = FF_TC / 16;

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// |a| >= |b| (or a == 0)
__device__ __forceinline__ void fast_two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}

struct FFSmem {
    static size_t bytes(int nslots, int nl, int nint)
    {
        size_t b = sizeof(float) * (4 * (size_t)K2 + 2 * (size_t)nslots * K * FF_TC);   // E^T hi/lo x 2 sides, slots hi/lo
        b += sizeof(int) * 2 * FF_TC;                                                   // column maxima (as int bits)
        b += sizeof(int) * FF_TC;                                                       // column exponents
        b += sizeof(SchedNode) * nint;
        b = (b + 15) & ~size_t(15);
        b += (size_t)nl * FF_TC;
        return (b + 15) & ~size_t(15);
    }
};

// FP64 E^T sets [nmat][K2] -> float-float [nmat][hi K2 | lo K2]: hi = the nearest float,
// lo = the nearest float to the remainder (together ~48 bits).
__global__ void k_split_ff(const double *in, float *out, size_t nmat)
{
    const size_t n = nmat * K2;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double x = in[i];
        const float h = (float)x;
        const size_t m = i / K2, k = i - m * K2;
        out[m * 2 * K2 + k] = h;
        out[m * 2 * K2 + K2 + k] = (float)(x - (double)h);
    }
}

__global__ void __launch_bounds__(FF_THREADS) k_prune_ff(PruneArgs a)
{
    extern __shared__ __align__(16) unsigned char ssm[];
    float *Et = reinterpret_cast<float *>(ssm);              // [2 sides][hi K2 | lo K2]
    float *slH = Et + 4 * K2;                                // [nslots][K][TC]
    float *slL = slH + (size_t)a.nslots * K * FF_TC;         // [nslots][K][TC]
    int *colmax = reinterpret_cast<int *>(slL + (size_t)a.nslots * K * FF_TC);   // [2][TC]
    int *cscale = colmax + 2 * FF_TC;                                            // [TC]
    SchedNode *sched = reinterpret_cast<SchedNode *>(cscale + FF_TC);
    size_t off = (reinterpret_cast<unsigned char *>(sched + a.n_internal) - ssm + 15) & ~size_t(15);
    uint8_t *lvT = ssm + off;                                                     // [nl][TC]

    const int tid = threadIdx.x;
    const int ty = tid / 16, tx = tid % 16;
    const int a0 = 4 * ty, c0 = FF_CPT * tx;
    const int nl = a.nl;
    __shared__ double red_l[FF_THREADS / 32], red_e[FF_THREADS / 32];

    for (int f = tid; f < a.n_internal; f += FF_THREADS) sched[f] = a.sched[f];

    for (int w = blockIdx.x; w < a.nwi; w += gridDim.x) {
        const WorkItem wi = a.wi[w];
        const Request rq = a.req[wi.request];
        const int md = rq.model;
        const float *Pbase = reinterpret_cast<const float *>(a.Pbuf) + (size_t)rq.pset * a.nbr * 2 * K2;
        const int ncols = wi.ncols;
        const uint8_t *lg = a.leaves + (size_t)wi.col0 * nl;
        // the split E^T (hi and lo blocks, 32 KB) of a node's internal children into shared
        // memory, copied asynchronously one node ahead; leaf children read their rows from
        // global memory instead
        auto copy_inner = [&](const SchedNode &nx) {
            constexpr int NV = 2 * K2 * sizeof(float) / 16;
#pragma unroll
            for (int side = 0; side < 2; side++) {
                if ((side ? nx.rslot : nx.lslot) < 0) continue;
                const char *src = reinterpret_cast<const char *>(Pbase + (size_t)(side ? nx.rc : nx.lc) * 2 * K2);
                const uint32_t dst = (uint32_t)__cvta_generic_to_shared(Et + side * 2 * K2);
                for (int f = tid; f < NV; f += FF_THREADS)
                    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" :: "r"(dst + 16 * f), "l"(src + 16 * f)
                                 : "memory");
            }
            asm volatile("cp.async.commit_group;" ::: "memory");
        };
        __syncthreads();   // previous work item finished with shared memory
        for (int f = tid; f < FF_TC * nl; f += FF_THREADS) {
            const int c = f / nl, l = f - c * nl;
            lvT[l * FF_TC + c] = (c < ncols) ? lg[f] : (uint8_t)K;
        }
        for (int f = tid; f < 2 * FF_TC; f += FF_THREADS) colmax[f] = 0;
        for (int f = tid; f < FF_TC; f += FF_THREADS) cscale[f] = 0;

        copy_inner(sched[0]);
        for (int ni = 0; ni < a.n_internal; ni++) {
            const SchedNode sn = sched[ni];
            asm volatile("cp.async.wait_all;" ::: "memory");
            __syncthreads();   // this node's E^T staged, the previous node's slots written
            float vh[2][4][FF_CPT], vl[2][4][FF_CPT];
#pragma unroll
            for (int side = 0; side < 2; side++) {
                const int slot = side ? sn.rslot : sn.lslot;
                const int child = side ? sn.rc : sn.lc;
                if (slot < 0) {
                    // leaf: P[a][s] = delta_as + E[a][s] from the split entries; 1 for a marginalised leaf
                    const float *Eg = Pbase + (size_t)child * 2 * K2;
#pragma unroll
                    for (int cc = 0; cc < FF_CPT; cc++) {
                        const int s = lvT[child * FF_TC + c0 + cc];
                        const int sr = s < K ? s : 0;
                        const float4 h4 = __ldg(reinterpret_cast<const float4 *>(Eg + sr * K + a0));
                        const float4 l4 = __ldg(reinterpret_cast<const float4 *>(Eg + K2 + sr * K + a0));
                        const float hv[4] = {h4.x, h4.y, h4.z, h4.w}, lv[4] = {l4.x, l4.y, l4.z, l4.w};
#pragma unroll
                        for (int i = 0; i < 4; i++) {
                            float h = hv[i], l = lv[i];
                            if (a0 + i == s) {   // 1 + E_ss: exact sum, then the low part folded in
                                float t, e;
                                two_sum(1.0f, h, t, e);
                                fast_two_sum(t, __fadd_rn(e, l), h, l);
                            }
                            vh[side][i][cc] = (s >= K) ? 1.0f : h;
                            vl[side][i][cc] = (s >= K) ? 0.0f : l;
                        }
                    }
                } else {
                    // internal: v = alpha + sum_j E[a][j] alpha[j], compensated
                    const float *Eh = Et + side * 2 * K2, *El = Eh + K2;
                    const float *xH = slH + (size_t)slot * K * FF_TC, *xL = slL + (size_t)slot * K * FF_TC;
                    float sh[4][FF_CPT], sa[4][FF_CPT], sb[4][FF_CPT], se[4][FF_CPT];
#pragma unroll
                    for (int i = 0; i < 4; i++)
#pragma unroll
                        for (int cc = 0; cc < FF_CPT; cc++) sh[i][cc] = sa[i][cc] = sb[i][cc] = se[i][cc] = 0.f;
#pragma unroll 2
                    for (int j = 0; j < K; j++) {
                        const float4 eh = *reinterpret_cast<const float4 *>(Eh + j * K + a0);
                        const float4 el = *reinterpret_cast<const float4 *>(El + j * K + a0);
                        float xhv[FF_CPT], xlv[FF_CPT];
                        if constexpr (FF_CPT == 2) {
                            const float2 xh = *reinterpret_cast<const float2 *>(xH + j * FF_TC + c0);
                            const float2 xl = *reinterpret_cast<const float2 *>(xL + j * FF_TC + c0);
                            xhv[0] = xh.x; xhv[FF_CPT - 1] = xh.y; xlv[0] = xl.x; xlv[FF_CPT - 1] = xl.y;
                        } else {
                            xhv[0] = xH[j * FF_TC + c0];
                            xlv[0] = xL[j * FF_TC + c0];
                        }
                        const float ehv[4] = {eh.x, eh.y, eh.z, eh.w}, elv[4] = {el.x, el.y, el.z, el.w};
#pragma unroll
                        for (int i = 0; i < 4; i++)
#pragma unroll
                            for (int cc = 0; cc < FF_CPT; cc++) {
                                const float p = __fmul_rn(ehv[i], xhv[cc]);
                                const float pe = fmaf(ehv[i], xhv[cc], -p);   // exact product error
                                float s, e;
                                two_sum(sh[i][cc], p, s, e);
                                sh[i][cc] = s;
                                sa[i][cc] = fmaf(ehv[i], xlv[cc], sa[i][cc]);
                                sb[i][cc] = fmaf(elv[i], xhv[cc], sb[i][cc]);
                                se[i][cc] = se[i][cc] + (pe + e);
                            }
                    }
#pragma unroll
                    for (int i = 0; i < 4; i++)
#pragma unroll
                        for (int cc = 0; cc < FF_CPT; cc++) {
                            const float ah = xH[(a0 + i) * FF_TC + c0 + cc], al = xL[(a0 + i) * FF_TC + c0 + cc];
                            float s, e;
                            two_sum(ah, sh[i][cc], s, e);
                            const float lo = __fadd_rn(__fadd_rn(al, (sa[i][cc] + sb[i][cc]) + se[i][cc]), e);
                            fast_two_sum(s, lo, vh[side][i][cc], vl[side][i][cc]);
                        }
                }
            }
            __syncthreads();   // every thread is past its reads of the E^T buffers and the child slots
            if (ni + 1 < a.n_internal) copy_inner(sched[ni + 1]);   // E^T buffers are free again
            // alpha = v_l * v_r (float-float product), column maxima of the hi parts
            int *cm = colmax + (ni & 1) * FF_TC;
            int *cm_next = colmax + ((ni + 1) & 1) * FF_TC;
            if (tid < FF_TC) cm_next[tid] = 0;
#pragma unroll
            for (int cc = 0; cc < FF_CPT; cc++) {
                float mx = 0.f;
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const float xh = vh[0][i][cc], xl = vl[0][i][cc], yh = vh[1][i][cc], yl = vl[1][i][cc];
                    const float p = __fmul_rn(xh, yh);
                    float lo = fmaf(xh, yh, -p);
                    lo = fmaf(xh, yl, lo);
                    lo = fmaf(xl, yh, lo);
                    float h, l;
                    fast_two_sum(p, lo, h, l);
                    vh[0][i][cc] = h;
                    vl[0][i][cc] = l;
                    mx = h > mx ? h : mx;
                }
                atomicMax(cm + c0 + cc, __float_as_int(mx));   // non-negative floats order as ints
            }
            __syncthreads();   // column maxima complete
            float *oH = slH + (size_t)sn.oslot * K * FF_TC, *oL = slL + (size_t)sn.oslot * K * FF_TC;
            int ecol[FF_CPT];
#pragma unroll
            for (int cc = 0; cc < FF_CPT; cc++) {
                const float mx = __int_as_float(cm[c0 + cc]);
                ecol[cc] = (mx > 0.f) ? exp_of(mx) : 0;
                if (ty == 0) cscale[c0 + cc] += ecol[cc];
            }
#pragma unroll
            for (int i = 0; i < 4; i++) {
                float yh[FF_CPT], yl[FF_CPT];
#pragma unroll
                for (int cc = 0; cc < FF_CPT; cc++) {
                    yh[cc] = scale2(vh[0][i][cc], -ecol[cc]);
                    yl[cc] = scale2(vl[0][i][cc], -ecol[cc]);
                }
                ColStore<float, FF_CPT>::store(oH + (a0 + i) * FF_TC + c0, yh);
                ColStore<float, FF_CPT>::store(oL + (a0 + i) * FF_TC + c0, yl);
            }
        }
        __syncthreads();   // the root's slot written
        // root: z = alpha_root . prior ; elpr term = (alpha_root . prior*log prior) / z, in FP64
        double tl = 0.0, te = 0.0;
        if (tid < FF_TC && tid < ncols) {
            const int os = sched[a.n_internal - 1].oslot;
            const float *rH = slH + (size_t)os * K * FF_TC, *rL = slL + (size_t)os * K * FF_TC;
            const double *pr = a.m.prior + md * K;
            const double *wl = a.m.wlog + md * K;
            double z = 0.0, wz = 0.0;
            for (int s = 0; s < K; s++) {
                const double x = (double)rH[s * FF_TC + tid] + (double)rL[s * FF_TC + tid];
                z += x * pr[s];
                wz += x * wl[s];
            }
            if (z > 0.0) {
                tl = log(z) + (double)cscale[tid] * 0.69314718055994530942;
                te = wz / z;
            } else {
                tl = -INFINITY;
                te = 0.0;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            tl += __shfl_down_sync(0xffffffffu, tl, o);
            te += __shfl_down_sync(0xffffffffu, te, o);
        }
        if ((tid & 31) == 0) {
            red_l[tid >> 5] = tl;
            red_e[tid >> 5] = te;
        }
        __syncthreads();
        if (tid == 0) {
            double sl = 0.0, se = 0.0;
            for (int k = 0; k < (FF_TC + 31) / 32; k++) {
                sl += red_l[k];
                se += red_e[k];
            }
            a.partials[2 * (size_t)w] = sl;
            a.partials[2 * (size_t)w + 1] = se;
        }
    }
}

}  // namespace

int ff_tile_cols() { return FF_TC; }

cudaError_t launch_split_ff(const double *in, float *out, size_t nmat, cudaStream_t s)
{
    if (nmat == 0) return cudaSuccess;
    const size_t n = nmat * K2;
    const unsigned blocks = (unsigned)std::min<size_t>((n + 255) / 256, 4096);
    k_split_ff<<<blocks, 256, 0, s>>>(in, out, nmat);
    return cudaGetLastError();
}

size_t prune_ff_smem_bytes(int nslots, int nl, int nint) { return FFSmem::bytes(nslots, nl, nint); }

int prune_ff_ctas_per_sm(int nslots, int nl, int nint)
{
    const size_t smem = FFSmem::bytes(nslots, nl, nint);
    int n = 0;
    if (cudaFuncSetAttribute(k_prune_ff, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_prune_ff, FF_THREADS, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

cudaError_t launch_prune_ff(const PruneArgs &a, cudaStream_t s, int grid)
{
    if (a.nwi <= 0) return cudaSuccess;
    const size_t smem = FFSmem::bytes(a.nslots, a.nl, a.n_internal);
    cudaError_t e = cudaFuncSetAttribute(k_prune_ff, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_prune_ff<<<grid, FF_THREADS, smem, s>>>(a);
    return cudaGetLastError();
}

}  // namespace pcsf
