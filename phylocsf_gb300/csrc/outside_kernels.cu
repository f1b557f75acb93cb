// Outside-pass products beyond the gradient: the expected substitution counts of
// every branch (the sufficient statistics of PhyloEM) and the posterior state
// distribution of selected nodes at every column.
//
// Reference mathematics (paths relative to mlin/PhyloCSF):
//   outside pass             lib/CamlPaml/PhyloLik.ml:96-120    beta_i = P_i^T (beta_p . (P_s alpha_s))
//   node posterior           lib/CamlPaml/PhyloLik.ml:127-138   alpha_i . beta_i / z (a leaf: its own vector)
//   branch posteriors        lib/CamlPaml/PhyloLik.ml:140-174   beta_p[a] (P_s alpha_s)[a] P_i[a][b] alpha_i[b] / z
//   sufficient statistics    lib/CamlPaml/PhyloEM.ml:14-20      the branch posteriors summed over the columns
// With inter_c = beta_p . v_s (v_s = P_s alpha_s the sibling's partial at the parent),
// the counts of branch c are P_c[a][b] M_c[a][b] with M_c = sum_col inter_c alpha_c^T / z:
// per tile a 64 x 64 x (tile columns) product, accumulated over the tiles of a region
// and multiplied by P_c once at the end.
//
// One CTA owns one request (region, model, rho) at a time and walks its column tiles
// in order, so every count is summed in a fixed order (no atomics): the results do
// not depend on the launch configuration.  The inside pass is the one of k_grad and
// stores every child partial, the alpha of every internal node and the per-column
// exponents of the power-of-two rescaling in a per-CTA scratch area; exponent
// bookkeeping per column as in k_grad:
//   alpha_i = alpha~_i 2^{e(i)},  beta_c = beta~_c 2^{f(c)},  z = z~ 2^{e(root)}.
// FP64 on the FP64 engine; FP32 with compensated sums on the others.
#include <cmath>

#include "pcsf_internal.h"
#include "prune_common.cuh"

namespace pcsf {

namespace {

constexpr int OS_THREADS = 256;
constexpr int OS_TC = 32;
constexpr int OS_CPT = OS_TC / 16;

template <typename T>
struct OutLayout {
    static size_t smem(int nslots, int nl, int nint)
    {
        size_t b = sizeof(T) * (2 * (size_t)K2 + (size_t)nslots * K * OS_TC + (size_t)K * OS_TC);   // Mat[2], slots, X
        b += sizeof(typename AtomMax<T>::U) * OS_TC;                                               // column maxima
        b += sizeof(double) * 2 * OS_TC;                                                           // z~, column weights
        b += sizeof(int) * OS_TC;                                                                  // e(root)
        b += sizeof(SchedNode) * nint;
        b = (b + 15) & ~size_t(15);
        b += (size_t)nl * OS_TC;
        return (b + 15) & ~size_t(15);
    }
    static size_t scratch(int nl)
    {
        const int n = 2 * nl - 1;
        size_t b = sizeof(T) * ((size_t)(n - 1) + 2 * (size_t)(nl - 1)) * K * OS_TC;   // V, alpha~ and beta~ of internal nodes
        b += sizeof(int) * 2 * (size_t)n * OS_TC;                                      // e, f
        return (b + 255) & ~size_t(255);
    }
};

template <typename T, int KAHAN>
__global__ void __launch_bounds__(OS_THREADS) k_outside(OutsideArgs a)
{
    constexpr int TC = OS_TC, CPT = OS_CPT;
    typedef typename AtomMax<T>::U MU;
    extern __shared__ __align__(16) unsigned char osm[];
    T *Mat = reinterpret_cast<T *>(osm);                           // [2][K][K]
    T *slots = Mat + 2 * K2;                                        // [nslots][K][TC]
    T *X = slots + (size_t)a.nslots * K * TC;                       // [K][TC]
    MU *colmax = reinterpret_cast<MU *>(X + K * TC);                // [TC]
    double *zt = reinterpret_cast<double *>(colmax + TC);           // [TC]
    double *wcol = zt + TC;                                         // [TC]
    int *eroot = reinterpret_cast<int *>(wcol + TC);                // [TC]
    SchedNode *sched = reinterpret_cast<SchedNode *>(eroot + TC);   // [n_internal]
    size_t off = (reinterpret_cast<unsigned char *>(sched + a.n_internal) - osm + 15) & ~size_t(15);
    uint8_t *lvT = osm + off;                                       // [nl][TC]
    __shared__ double wsum[OS_THREADS / 32];

    const int tid = threadIdx.x;
    const int ty = tid / 16, tx = tid % 16;
    const int a0 = 4 * ty, c0 = CPT * tx;     // contraction tiles: 4 states x 2 columns
    const int b0 = 4 * tx;                     // count blocks: states a0.. (from) x b0.. (to)
    const int nl = a.nl, n = 2 * nl - 1, root = n - 1;
    unsigned char *sbase = reinterpret_cast<unsigned char *>(a.scratch) + (size_t)blockIdx.x * a.scratch_per_cta;
    T *V = reinterpret_cast<T *>(sbase);                             // [n-1][K][TC]
    T *A = V + (size_t)(n - 1) * K * TC;                             // [nl-1][K][TC] alpha~ (internal nodes)
    T *B = A + (size_t)(nl - 1) * K * TC;                            // [nl-1][K][TC] beta~ (internal nodes)
    int *eS = reinterpret_cast<int *>(B + (size_t)(nl - 1) * K * TC);   // [n][TC]
    int *fS = eS + (size_t)n * TC;                                   // [n][TC]
    auto e_of = [&](int node, int col) -> int { return node < nl ? 0 : eS[(size_t)node * TC + col]; };

    for (int f = tid; f < a.n_internal; f += OS_THREADS) sched[f] = a.sched[f];

    for (int r = blockIdx.x; r < a.nreq; r += gridDim.x) {
        const Request rq = a.req[r];
        const int md = rq.model;
        const T *Pbase = reinterpret_cast<const T *>(a.Pbuf) + (size_t)rq.pset * a.nbr * K2;
        const double *pr = a.m.prior + md * K;
        double *cnt = a.counts ? a.counts + (size_t)r * a.nbr * K2 : nullptr;
        double lpr = 0.0;    // thread 0: the request's log-likelihood, summed tile by tile in order

        for (int w = a.wi_begin[r]; w < a.wi_begin[r + 1]; w++) {
            const WorkItem wi = a.wi[w];
            const int ncols = wi.ncols;
            const uint8_t *lg = a.leaves + (size_t)wi.col0 * nl;
            __syncthreads();   // the previous tile is finished with shared memory
            for (int f = tid; f < TC * nl; f += OS_THREADS) {
                const int c = f / nl, l = f - c * nl;
                lvT[l * TC + c] = (c < ncols) ? lg[f] : (uint8_t)K;
            }
            for (int f = tid; f < TC; f += OS_THREADS) colmax[f] = 0;

            // ---------------- inside pass, storing the child partials and the node alphas
            for (int ni = 0; ni < a.n_internal; ni++) {
                const SchedNode sn = sched[ni];
                {
                    const float4 *gl = reinterpret_cast<const float4 *>(Pbase + (size_t)sn.lc * K2);
                    const float4 *gr = reinterpret_cast<const float4 *>(Pbase + (size_t)sn.rc * K2);
                    float4 *sl = reinterpret_cast<float4 *>(Mat);
                    float4 *sr = reinterpret_cast<float4 *>(Mat + K2);
                    constexpr int NV = K2 * sizeof(T) / 16;
                    for (int f = tid; f < NV; f += OS_THREADS) {
                        sl[f] = __ldg(gl + f);
                        sr[f] = __ldg(gr + f);
                    }
                }
                __syncthreads();
                T vl[4][CPT], vr[4][CPT];
                child_partial<T, TC, KAHAN>(Mat, slots, sn.lslot, sn.lc, lvT, a0, c0, vl);
                child_partial<T, TC, KAHAN>(Mat + K2, slots, sn.rslot, sn.rc, lvT, a0, c0, vr);
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int cc = 0; cc < CPT; cc++) {
                        V[((size_t)sn.lc * K + a0 + i) * TC + c0 + cc] = vl[i][cc];
                        V[((size_t)sn.rc * K + a0 + i) * TC + c0 + cc] = vr[i][cc];
                    }
                __syncthreads();   // Mat and slot reads done
#pragma unroll
                for (int cc = 0; cc < CPT; cc++) {
                    T mx = (T)0;
#pragma unroll
                    for (int i = 0; i < 4; i++) {
                        vl[i][cc] *= vr[i][cc];
                        mx = vl[i][cc] > mx ? vl[i][cc] : mx;
                    }
                    AtomMax<T>::upd(colmax + c0 + cc, mx);
                }
                __syncthreads();
                T *out = slots + (size_t)sn.oslot * K * TC;
                T *Ai = A + (size_t)(sn.node - nl) * K * TC;
#pragma unroll
                for (int cc = 0; cc < CPT; cc++) {
                    const T mx = AtomMax<T>::get(colmax + c0 + cc);
                    const int e = (mx > (T)0) ? exp_of(mx) : 0;
#pragma unroll
                    for (int i = 0; i < 4; i++) {
                        const T y = scale2(vl[i][cc], -e);
                        out[(a0 + i) * TC + c0 + cc] = y;
                        Ai[(size_t)(a0 + i) * TC + c0 + cc] = y;
                    }
                    if (ty == 0) {
                        const int col = c0 + cc;
                        eS[(size_t)sn.node * TC + col] = e_of(sn.lc, col) + e_of(sn.rc, col) + e;
                    }
                }
                __syncthreads();   // colmax reads done
                for (int f = tid; f < TC; f += OS_THREADS) colmax[f] = 0;
            }
            __syncthreads();
            // ---------------- root: z~ and the column log-likelihoods
            double tl = 0.0;
            if (tid < TC) {
                const T *ar = A + (size_t)(root - nl) * K * TC;
                double z = 0.0;
                for (int s = 0; s < K; s++) z += (double)ar[s * TC + tid] * pr[s];
                zt[tid] = z;
                eroot[tid] = eS[(size_t)root * TC + tid];
                if (tid < ncols) tl = (z > 0.0) ? log(z) + (double)eroot[tid] * 0.69314718055994530942 : -INFINITY;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) tl += __shfl_down_sync(0xffffffffu, tl, o);
            if ((tid & 31) == 0) wsum[tid >> 5] = tl;
            {   // beta~_root = prior, f(root) = 0
                T *Br = B + (size_t)(root - nl) * K * TC;
                for (int f = tid; f < K * TC; f += OS_THREADS) Br[f] = (T)pr[f / TC];
                for (int f = tid; f < TC; f += OS_THREADS) fS[(size_t)root * TC + f] = 0;
            }
            __syncthreads();
            if (tid == 0)
                for (int k = 0; k < (TC + 31) / 32; k++) lpr += wsum[k];
            // posteriors of the selected root and leaves (node_posterior: zeros where z = 0)
            if (a.sel) {
                const int kr = a.sel[root];
                if (kr >= 0) {
                    const T *ar = A + (size_t)(root - nl) * K * TC;
                    for (int f = tid; f < K * TC; f += OS_THREADS) {
                        const int x = f / TC, col = f % TC;
                        if (col >= ncols) continue;
                        const double z = zt[col];
                        a.post[((size_t)kr * a.total_cols + wi.col0 + col) * K + x] =
                            (z > 0.0) ? (double)ar[x * TC + col] * pr[x] / z : 0.0;
                    }
                }
                for (int l = 0; l < nl; l++) {
                    const int kl = a.sel[l];
                    if (kl < 0) continue;
                    for (int f = tid; f < K * TC; f += OS_THREADS) {
                        const int x = f / TC, col = f % TC;
                        if (col >= ncols) continue;
                        const int s = lvT[l * TC + col];
                        a.post[((size_t)kl * a.total_cols + wi.col0 + col) * K + x] =
                            (zt[col] > 0.0) ? ((s >= K || s == x) ? 1.0 : 0.0) : 0.0;
                    }
                }
            }

            // ---------------- outside pass, parents before children
            for (int ni = a.n_internal - 1; ni >= 0; ni--) {
                const SchedNode sn = sched[ni];
                const int p = sn.node;
                const T *Bp = B + (size_t)(p - nl) * K * TC;
                for (int side = 0; side < 2; side++) {
                    const int c = side ? sn.rc : sn.lc;
                    const int s = side ? sn.lc : sn.rc;
                    const bool internal = c >= nl;
                    __syncthreads();   // the previous side is finished with X, Mat[0], colmax, wcol
                    if (internal) {
                        // E_c in row-major order (the buffer holds E_c^T)
                        const T *g = Pbase + (size_t)c * K2;
                        for (int f = tid; f < K2; f += OS_THREADS) Mat[(f % K) * K + f / K] = g[f];
                    }
                    for (int f = tid; f < TC; f += OS_THREADS) colmax[f] = 0;
                    const T *Vs = V + (size_t)s * K * TC;
                    for (int f = tid; f < K * TC; f += OS_THREADS) X[f] = Bp[f] * Vs[f];    // inter~
                    if (tid < TC) {   // weight of column tid in the counts: 2^{f(p) + e(s) + e(c) - e(root)} / z~
                        const double z = zt[tid];
                        wcol[tid] = (tid < ncols && z > 0.0)
                                        ? ldexp(1.0, fS[(size_t)p * TC + tid] + e_of(s, tid) + e_of(c, tid) - eroot[tid]) / z
                                        : 0.0;
                    }
                    __syncthreads();
                    if (internal) {
                        // beta~_c = P_c^T inter~ = inter~ + E_c^T inter~, rescaled per column
                        T bt[4][CPT];
                        contract<T, TC, KAHAN>(Mat, X, a0, c0, bt);
#pragma unroll
                        for (int cc = 0; cc < CPT; cc++) {
                            T mx = (T)0;
#pragma unroll
                            for (int i = 0; i < 4; i++) {
                                bt[i][cc] += X[(a0 + i) * TC + c0 + cc];
                                mx = bt[i][cc] > mx ? bt[i][cc] : mx;
                            }
                            AtomMax<T>::upd(colmax + c0 + cc, mx);
                        }
                        __syncthreads();
                        T *Bc = B + (size_t)(c - nl) * K * TC;
                        const T *Ac = A + (size_t)(c - nl) * K * TC;
                        const int kc = a.sel ? a.sel[c] : -1;
#pragma unroll
                        for (int cc = 0; cc < CPT; cc++) {
                            const int col = c0 + cc;
                            const T mx = AtomMax<T>::get(colmax + col);
                            const int e = (mx > (T)0) ? exp_of(mx) : 0;
                            const int fc = fS[(size_t)p * TC + col] + e_of(s, col) + e;
#pragma unroll
                            for (int i = 0; i < 4; i++) {
                                const T y = scale2(bt[i][cc], -e);
                                Bc[(size_t)(a0 + i) * TC + col] = y;
                                if (kc >= 0 && col < ncols) {
                                    const double z = zt[col];
                                    a.post[((size_t)kc * a.total_cols + wi.col0 + col) * K + a0 + i] =
                                        (z > 0.0) ? ldexp((double)Ac[(size_t)(a0 + i) * TC + col] * (double)y,
                                                          e_of(c, col) + fc - eroot[col]) / z
                                                  : 0.0;
                                }
                            }
                            if (ty == 0) fS[(size_t)c * TC + col] = fc;
                        }
                    }
                    if (cnt) {
                        __syncthreads();   // the beta contraction is finished with X
                        for (int f = tid; f < K * TC; f += OS_THREADS) X[f] = (T)((double)X[f] * wcol[f % TC]);
                        __syncthreads();
                        // M_c[a][b] += sum_col inter~[a] w alpha~_c[b] for this thread's 4 x 4 block
                        double m4[4][4];
                        T acc[4][4];
#pragma unroll
                        for (int i = 0; i < 4; i++)
#pragma unroll
                            for (int j = 0; j < 4; j++) acc[i][j] = (T)0;
                        if (internal) {
                            const T *Ac = A + (size_t)(c - nl) * K * TC;
                            for (int col = 0; col < TC; col++) {
                                T xa[4], yb[4];
#pragma unroll
                                for (int i = 0; i < 4; i++) xa[i] = X[(a0 + i) * TC + col];
#pragma unroll
                                for (int j = 0; j < 4; j++) yb[j] = Ac[(size_t)(b0 + j) * TC + col];
#pragma unroll
                                for (int i = 0; i < 4; i++)
#pragma unroll
                                    for (int j = 0; j < 4; j++) acc[i][j] += xa[i] * yb[j];
                            }
                        } else {
                            for (int col = 0; col < TC; col++) {
                                const int sl = lvT[c * TC + col];
#pragma unroll
                                for (int i = 0; i < 4; i++) {
                                    const T xa = X[(a0 + i) * TC + col];
#pragma unroll
                                    for (int j = 0; j < 4; j++)
                                        if (sl >= K || sl == b0 + j) acc[i][j] += xa;
                                }
                            }
                        }
                        double *cc4 = cnt + (size_t)c * K2;
#pragma unroll
                        for (int i = 0; i < 4; i++)
#pragma unroll
                            for (int j = 0; j < 4; j++) {
                                m4[i][j] = cc4[(a0 + i) * K + b0 + j] + (double)acc[i][j];
                                cc4[(a0 + i) * K + b0 + j] = m4[i][j];
                            }
                    }
                }
            }
        }
        // counts = P_c o M_c (each thread its own entries, as accumulated)
        if (cnt) {
            for (int c = 0; c < a.nbr; c++) {
                const T *Et = Pbase + (size_t)c * K2;
                double *cc4 = cnt + (size_t)c * K2;
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        const int aa = a0 + i, bb = b0 + j;
                        const double pab = (double)Et[bb * K + aa] + (aa == bb ? 1.0 : 0.0);
                        cc4[aa * K + bb] *= pab;
                    }
            }
        }
        if (tid == 0) a.lpr[r] = lpr;
        __syncthreads();
    }
}

template <typename T, int KAHAN>
cudaError_t launch_outside_t(const OutsideArgs &a, cudaStream_t s, int grid)
{
    const size_t smem = OutLayout<T>::smem(a.nslots, a.nl, a.n_internal);
    cudaError_t e = cudaFuncSetAttribute(k_outside<T, KAHAN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_outside<T, KAHAN><<<grid, OS_THREADS, smem, s>>>(a);
    return cudaGetLastError();
}

}  // namespace

int outside_tile_cols() { return OS_TC; }

size_t outside_smem_bytes(bool fp64, int nslots, int nl, int nint)
{
    return fp64 ? OutLayout<double>::smem(nslots, nl, nint) : OutLayout<float>::smem(nslots, nl, nint);
}

size_t outside_scratch_per_cta(bool fp64, int nl)
{
    return fp64 ? OutLayout<double>::scratch(nl) : OutLayout<float>::scratch(nl);
}

cudaError_t launch_outside(bool fp64, int comp, const OutsideArgs &a, cudaStream_t s, int grid)
{
    if (a.nreq <= 0) return cudaSuccess;
    if (fp64) return launch_outside_t<double, 0>(a, s, grid);
    if (comp == 2) return launch_outside_t<float, 2>(a, s, grid);
    return launch_outside_t<float, 1>(a, s, grid);
}

}  // namespace pcsf
