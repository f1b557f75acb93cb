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
//     matrices, row rule of Q.ml:226-247 applied in FP64) and is split into hi / lo
//     floats while it is staged into shared memory;
//   - a leaf child's partial P[a][s] = delta_as + E[a][s] is formed in FP64 and
//     split (PhyloLik.ml:87-88 with a one-hot leaf);
//   - an internal child's v = alpha + sum_j E[a][j] alpha[j] (PhyloLik.ml:89-92)
//     is a compensated dot product: each hi x hi product is split exactly
//     (TwoProduct by FMA), its hi part is added with TwoSum, and the product
//     errors, the TwoSum errors and the hi x lo cross terms are summed in the lo word;
//   - node products alpha = v_l * v_r are float-float products;
//   - each column is rescaled by an exact power of two after every node;
//   - the root dot with the prior, the log and the tile sums are FP64.
// The error-free steps use __fadd_rn / __fmul_rn, which the compiler never fuses
// into an FMA (a fused form would break the exactness the transforms rely on).
#include "pcsf_internal.h"
#include "prune_common.cuh"

namespace pcsf {

namespace {

constexpr int FF_THREADS = 256;
constexpr int FF_TC = 32;            // columns per tile (2 per thread)
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
        size_t b = sizeof(float) * (4 * (size_t)K2 + 2 * (size_t)nslots * K * FF_TC);   // E^T hi/lo x 2, slots hi/lo
        b += sizeof(int) * 2 * FF_TC;                                                   // column maxima (as int bits)
        b += sizeof(int) * FF_TC;                                                       // column exponents
        b += sizeof(SchedNode) * nint;
        b = (b + 15) & ~size_t(15);
        b += (size_t)nl * FF_TC;
        return (b + 15) & ~size_t(15);
    }
};

__global__ void __launch_bounds__(FF_THREADS) k_prune_ff(PruneArgs a)
{
    extern __shared__ __align__(16) unsigned char ssm[];
    float *EtH = reinterpret_cast<float *>(ssm);            // [2][K][K]
    float *EtL = EtH + 2 * K2;                               // [2][K][K]
    float *slH = EtL + 2 * K2;                               // [nslots][K][TC]
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
        const double *Pbase = reinterpret_cast<const double *>(a.Pbuf) + (size_t)rq.pset * a.nbr * K2;
        const int ncols = wi.ncols;
        const uint8_t *lg = a.leaves + (size_t)wi.col0 * nl;
        __syncthreads();   // previous work item finished with shared memory
        for (int f = tid; f < FF_TC * nl; f += FF_THREADS) {
            const int c = f / nl, l = f - c * nl;
            lvT[l * FF_TC + c] = (c < ncols) ? lg[f] : (uint8_t)K;
        }
        for (int f = tid; f < 2 * FF_TC; f += FF_THREADS) colmax[f] = 0;
        for (int f = tid; f < FF_TC; f += FF_THREADS) cscale[f] = 0;

        for (int ni = 0; ni < a.n_internal; ni++) {
            const SchedNode sn = sched[ni];
            // E^T of the internal children, split into hi / lo floats
            for (int side = 0; side < 2; side++) {
                if ((side ? sn.rslot : sn.lslot) < 0) continue;
                const double2 *src = reinterpret_cast<const double2 *>(Pbase + (size_t)(side ? sn.rc : sn.lc) * K2);
                float2 *dh = reinterpret_cast<float2 *>(EtH + side * K2);
                float2 *dl = reinterpret_cast<float2 *>(EtL + side * K2);
                for (int f = tid; f < K2 / 2; f += FF_THREADS) {
                    const double2 x = __ldg(src + f);
                    const float hx = (float)x.x, hy = (float)x.y;
                    dh[f] = make_float2(hx, hy);
                    dl[f] = make_float2((float)(x.x - (double)hx), (float)(x.y - (double)hy));
                }
            }
            __syncthreads();
            float vh[2][4][FF_CPT], vl[2][4][FF_CPT];
#pragma unroll
            for (int side = 0; side < 2; side++) {
                const int slot = side ? sn.rslot : sn.lslot;
                const int child = side ? sn.rc : sn.lc;
                if (slot < 0) {
                    // leaf: P[a][s] = delta_as + E[a][s] in FP64, split; 1 for a marginalised leaf
                    const double *Et = Pbase + (size_t)child * K2;
#pragma unroll
                    for (int cc = 0; cc < FF_CPT; cc++) {
                        const int s = lvT[child * FF_TC + c0 + cc];
                        const double *row = Et + (size_t)(s < K ? s : 0) * K + a0;
                        const double2 r01 = __ldg(reinterpret_cast<const double2 *>(row));
                        const double2 r23 = __ldg(reinterpret_cast<const double2 *>(row + 2));
                        const double e4[4] = {r01.x, r01.y, r23.x, r23.y};
#pragma unroll
                        for (int i = 0; i < 4; i++) {
                            const double x = (s >= K) ? 1.0 : e4[i] + (a0 + i == s ? 1.0 : 0.0);
                            const float h = (float)x;
                            vh[side][i][cc] = h;
                            vl[side][i][cc] = (float)(x - (double)h);
                        }
                    }
                } else {
                    // internal: v = alpha + sum_j E[a][j] alpha[j], compensated
                    const float *Eh = EtH + side * K2, *El = EtL + side * K2;
                    const float *xH = slH + (size_t)slot * K * FF_TC, *xL = slL + (size_t)slot * K * FF_TC;
                    float sh[4][FF_CPT], sl[4][FF_CPT];
#pragma unroll
                    for (int i = 0; i < 4; i++)
#pragma unroll
                        for (int cc = 0; cc < FF_CPT; cc++) sh[i][cc] = sl[i][cc] = 0.f;
#pragma unroll 2
                    for (int j = 0; j < K; j++) {
                        const float4 eh = *reinterpret_cast<const float4 *>(Eh + j * K + a0);
                        const float4 el = *reinterpret_cast<const float4 *>(El + j * K + a0);
                        const float2 xh = *reinterpret_cast<const float2 *>(xH + j * FF_TC + c0);
                        const float2 xl = *reinterpret_cast<const float2 *>(xL + j * FF_TC + c0);
                        const float ehv[4] = {eh.x, eh.y, eh.z, eh.w}, elv[4] = {el.x, el.y, el.z, el.w};
                        const float xhv[2] = {xh.x, xh.y}, xlv[2] = {xl.x, xl.y};
#pragma unroll
                        for (int i = 0; i < 4; i++)
#pragma unroll
                            for (int cc = 0; cc < FF_CPT; cc++) {
                                const float p = __fmul_rn(ehv[i], xhv[cc]);
                                const float pe = fmaf(ehv[i], xhv[cc], -p);   // exact product error
                                float s, e;
                                two_sum(sh[i][cc], p, s, e);
                                sh[i][cc] = s;
                                float t = fmaf(ehv[i], xlv[cc], sl[i][cc]);
                                t = fmaf(elv[i], xhv[cc], t);
                                sl[i][cc] = t + (pe + e);
                            }
                    }
#pragma unroll
                    for (int i = 0; i < 4; i++)
#pragma unroll
                        for (int cc = 0; cc < FF_CPT; cc++) {
                            const float ah = xH[(a0 + i) * FF_TC + c0 + cc], al = xL[(a0 + i) * FF_TC + c0 + cc];
                            float s, e;
                            two_sum(ah, sh[i][cc], s, e);
                            const float lo = __fadd_rn(__fadd_rn(al, sl[i][cc]), e);
                            fast_two_sum(s, lo, vh[side][i][cc], vl[side][i][cc]);
                        }
                }
            }
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
            __syncthreads();   // every thread is past its reads of the E^T buffers and the child slots
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
            __syncthreads();   // slots written before the next node reads them or the E^T buffers are refilled
        }
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
