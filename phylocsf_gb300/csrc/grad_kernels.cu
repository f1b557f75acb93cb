// Adjoint (outside-pass) gradient of the log-likelihood with respect to every
// branch length, for a batch of (region, model, rho) requests.
//
// Reference mathematics (paths relative to mlin/PhyloCSF):
//   outside pass          lib/CamlPaml/PhyloLik.ml:96-120   beta_i = P_i^T (beta_p . (P_s alpha_s))
//   branch posteriors     lib/CamlPaml/PhyloLik.ml:140-174
//   dP/dt                 lib/CamlPaml/Q.ml:260-275          dP/dt = Q P(t)
//   d ELL / d branch      lib/CamlPaml/PhyloEM.ml:140-171    (Fisher identity: = d logL / d t)
// Per column, with v_c = P_c alpha_c the partial of child c at its parent p and
// s its sibling:
//   inter_c = beta_p . v_s,   d log z / d t_c = inter_c^T Q v_c / z,   beta_c = P_c^T inter_c.
//
// One CTA (256 threads) owns a tile of TC columns.  The inside pass is the one of
// k_prune but also stores the partial v_c of every internal child and the per-column
// exponents of the power-of-two rescaling in a per-CTA global scratch area; the
// outside pass then walks the schedule in reverse.  A leaf child's partial is one
// gathered row of E^T plus the identity (P_c[a][s]); with RECOMP the outside pass
// recomputes it from the leaf state instead of storing it (the scratch then holds
// nl - 1 partials and nl - 1 betas instead of 2 nl - 2 and nl - 1: a third less, the
// same values, ~5 % more time for the scattered re-reads of E^T rows).  Exponent bookkeeping per column:
// alpha_i = alpha~_i 2^{e(i)} with e(i) = e(l) + e(r) + s_i, beta_c = beta~_c 2^{f(c)}
// with f(c) = f(p) + e(s) + t_c, and the gradient term carries
// 2^{f(p) + e(s) + e(c) - e(root)} against the scaled z~.
#include <cmath>

#include "pcsf_internal.h"
#include "prune_common.cuh"

namespace pcsf {

constexpr int GR_THREADS = 256;

template <typename T, int TC, bool RECOMP>
struct GradLayout {
    __host__ __device__ static size_t base(int nslots, int nl, int nint)
    {
        size_t b = sizeof(T) * (3 * (size_t)K2 + (size_t)nslots * K * TC + (size_t)K * TC + 16 * TC);
        b += sizeof(typename AtomMax<T>::U) * TC;
        b += sizeof(double) * TC + sizeof(int) * 2 * TC;
        b += sizeof(SchedNode) * nint;
        b = (b + 15) & ~size_t(15);
        b += (size_t)nl * TC;
        return (b + 15) & ~size_t(15);
    }
    // parameter derivatives need U (appended) and two [K][TC] tiles, kept in the partial
    // slots (idle during the outside pass) when there are at least two, else appended
    // too; H_x^T uses Mat[1], which the outside pass does not touch
    static size_t extra(int nslots, int npar)
    {
        if (!npar) return 0;
        return sizeof(T) * ((size_t)K2 + (nslots >= 2 ? 0 : 2 * (size_t)K * TC));
    }
    static size_t smem(int nslots, int nl, int nint, int npar) { return base(nslots, nl, nint) + extra(nslots, npar); }
    // stored child partials: every child's (n - 1), or with RECOMP the internal children's
    __host__ __device__ static size_t nv(int nl) { return RECOMP ? (size_t)(nl - 1) : (size_t)(2 * nl - 2); }
    static size_t scratch(int nl, int npar)
    {
        const int n = 2 * nl - 1;
        size_t b = sizeof(T) * (nv(nl) + (nl - 1)) * K * TC;        // child partials, betas
        b += sizeof(int) * 2 * (size_t)n * TC;
        b = (b + 255) & ~size_t(255);
        if (npar) b += (sizeof(T) * (size_t)(nl - 1) * K * TC + 255) & ~size_t(255);   // alpha of internal nodes
        return b;
    }
};

template <typename T, int TC, int KAHAN, bool RECOMP>
__global__ void __launch_bounds__(GR_THREADS) k_grad(GradArgs a)
{
    typedef GradLayout<T, TC, RECOMP> Layout;
    constexpr int CPT = TC / 16;
    typedef typename AtomMax<T>::U MU;
    extern __shared__ __align__(16) unsigned char gsm[];
    T *Mat = reinterpret_cast<T *>(gsm);                          // [3][K][K]
    T *slots = Mat + 3 * K2;                                       // [nslots][K][TC]
    T *X = slots + (size_t)a.nslots * K * TC;                      // [K][TC]
    T *red = X + K * TC;                                           // [16][TC]
    MU *colmax = reinterpret_cast<MU *>(red + 16 * TC);            // [TC]
    double *zt = reinterpret_cast<double *>(colmax + TC);          // [TC]
    int *eroot = reinterpret_cast<int *>(zt + TC);                 // [TC]
    int *sexp = eroot + TC;                                        // [TC]
    SchedNode *sched = reinterpret_cast<SchedNode *>(sexp + TC);   // [n_internal]
    size_t off = (reinterpret_cast<unsigned char *>(sched + a.n_internal) - gsm + 15) & ~size_t(15);
    uint8_t *lvT = gsm + off;                                      // [nl][TC]
    // parameter derivatives (outside pass only): U and the eigenbasis images of inter and
    // alpha_c over the slots (continuing past them into the extra space at the end of the
    // layout when the slots are fewer), H_x^T in Mat[1]
    T *Ubuf = reinterpret_cast<T *>(gsm + Layout::base(a.nslots, a.nl, a.n_internal));   // [K][K]
    T *Pt = (a.nslots >= 2) ? slots : Ubuf + K2;                   // [K][TC]
    T *Qt = Pt + K * TC;                                           // [K][TC]
    T *Hbuf = Mat + K2;                                            // [K][K]
    __shared__ double wsum_l[GR_THREADS / 32], wsum_e[GR_THREADS / 32];

    const int tid = threadIdx.x;
    const int ty = tid / 16, tx = tid % 16;
    const int a0 = 4 * ty, c0 = CPT * tx;
    const int nl = a.nl, n = 2 * nl - 1;
    unsigned char *sbase = reinterpret_cast<unsigned char *>(a.scratch) + (size_t)blockIdx.x * a.scratch_per_cta;
    T *V = reinterpret_cast<T *>(sbase);                             // [nv][K][TC] child partials (vslot)
    T *B = V + Layout::nv(nl) * K * TC;                              // [nl-1][K][TC] (internal nodes)
    int *eS = reinterpret_cast<int *>(B + (size_t)(nl - 1) * K * TC);  // [n][TC]
    int *fS = eS + (size_t)n * TC;                                   // [n][TC]
    T *Ascr = reinterpret_cast<T *>(sbase + ((sizeof(T) * (Layout::nv(nl) + (nl - 1)) * K * TC +
                                              sizeof(int) * 2 * (size_t)n * TC + 255) & ~size_t(255)));   // [nl-1][K][TC]
    // a child's slab among the stored partials (RECOMP: internal children only)
    auto vslot = [&](int c) -> size_t { return RECOMP ? (size_t)(c - nl) : (size_t)c; };
    const int gstride = a.nbr + a.npar;
    auto e_of = [&](int node, int col) -> int { return node < nl ? 0 : eS[(size_t)node * TC + col]; };
    // partial of child c at its parent, state st, tile column col: stored, or (RECOMP, a
    // leaf) recomputed exactly as the inside pass formed it (child_partial: E^T[s][st] +
    // delta, in one rounding; 1 for a marginalised leaf)
    auto vpart = [&](const T *Pbase, int c, int st, int col) -> T {
        if (!RECOMP || c >= nl) return V[(vslot(c) * K + st) * TC + col];
        const int sl = lvT[c * TC + col];
        if (sl >= K) return (T)1;
        return fma(Pbase[(size_t)c * K2 + (size_t)sl * K + st], (T)1, sl == st ? (T)1 : (T)0);
    };

    for (int f = tid; f < a.n_internal; f += GR_THREADS) sched[f] = a.sched[f];

    for (int w = blockIdx.x; w < a.nwi; w += gridDim.x) {
        const WorkItem wi = a.wi[w];
        const Request rq = a.req[wi.request];
        const int md = rq.model;
        const T *Pbase = reinterpret_cast<const T *>(a.Pbuf) + (size_t)rq.pset * a.nbr * K2;
        const int ncols = wi.ncols;
        const uint8_t *lg = a.leaves + (size_t)wi.col0 * nl;
        __syncthreads();
        for (int f = tid; f < TC * nl; f += GR_THREADS) {
            int c = f / nl, l = f - c * nl;
            lvT[l * TC + c] = (c < ncols) ? lg[f] : (uint8_t)K;
        }
        for (int f = tid; f < TC; f += GR_THREADS) colmax[f] = 0;
        {
            const T *Qg = reinterpret_cast<const T *>(a.Qrow) + (size_t)md * K2;
            for (int f = tid; f < K2; f += GR_THREADS) Mat[2 * K2 + f] = Qg[f];
            if (a.npar) {
                const T *Ug = reinterpret_cast<const T *>(a.Umat) + (size_t)md * K2;
                for (int f = tid; f < K2; f += GR_THREADS) Ubuf[f] = Ug[f];
            }
        }
        double pacc[2] = {0.0, 0.0};      // this work item's parameter derivatives (thread 0)

        // ---------------- inside pass, storing the child partials
        for (int ni = 0; ni < a.n_internal; ni++) {
            const SchedNode sn = sched[ni];
            {
                const float4 *gl = reinterpret_cast<const float4 *>(Pbase + (size_t)sn.lc * K2);
                const float4 *gr = reinterpret_cast<const float4 *>(Pbase + (size_t)sn.rc * K2);
                float4 *sl = reinterpret_cast<float4 *>(Mat);
                float4 *sr = reinterpret_cast<float4 *>(Mat + K2);
                constexpr int NV = K2 * sizeof(T) / 16;
                for (int f = tid; f < NV; f += GR_THREADS) {
                    sl[f] = __ldg(gl + f);
                    sr[f] = __ldg(gr + f);
                }
            }
            __syncthreads();
            T vl[4][CPT], vr[4][CPT];
            child_partial<T, TC, KAHAN>(Mat, slots, sn.lslot, sn.lc, lvT, a0, c0, vl);
            child_partial<T, TC, KAHAN>(Mat + K2, slots, sn.rslot, sn.rc, lvT, a0, c0, vr);
            T mxc[CPT];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int cc = 0; cc < CPT; cc++) {
                    if (!RECOMP || sn.lc >= nl) V[(vslot(sn.lc) * K + a0 + i) * TC + c0 + cc] = vl[i][cc];
                    if (!RECOMP || sn.rc >= nl) V[(vslot(sn.rc) * K + a0 + i) * TC + c0 + cc] = vr[i][cc];
                }
            __syncthreads();   // Mat and slots reads done; colmax zeroed
#pragma unroll
            for (int cc = 0; cc < CPT; cc++) {
                T mx = (T)0;
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    vl[i][cc] *= vr[i][cc];
                    mx = vl[i][cc] > mx ? vl[i][cc] : mx;
                }
                mxc[cc] = mx;
                AtomMax<T>::upd(colmax + c0 + cc, mx);
            }
            __syncthreads();
            T *out = slots + (size_t)sn.oslot * K * TC;
#pragma unroll
            for (int cc = 0; cc < CPT; cc++) {
                T mx = AtomMax<T>::get(colmax + c0 + cc);
                int e = (mx > (T)0) ? exp_of(mx) : 0;
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const T x = scale2(vl[i][cc], -e);
                    out[(a0 + i) * TC + c0 + cc] = x;
                    if (a.npar) Ascr[((size_t)(sn.node - nl) * K + a0 + i) * TC + c0 + cc] = x;
                }
                if (ty == 0) {
                    const int col = c0 + cc;
                    eS[(size_t)sn.node * TC + col] = e_of(sn.lc, col) + e_of(sn.rc, col) + e;
                }
            }
            (void)mxc;
            __syncthreads();   // colmax reads done
            for (int f = tid; f < TC; f += GR_THREADS) colmax[f] = 0;
        }
        __syncthreads();
        // ---------------- root: z~, lpr and elpr terms
        const int root = n - 1;
        double tl = 0.0, te = 0.0;
        if (tid < TC) {
            const T *ar = slots + (size_t)sched[a.n_internal - 1].oslot * K * TC;
            const double *pr = a.m.prior + md * K;
            const double *wl = a.m.wlog + md * K;
            double z = 0.0, wz = 0.0;
            for (int s = 0; s < K; s++) {
                double x = (double)ar[s * TC + tid];
                z += x * pr[s];
                wz += x * wl[s];
            }
            zt[tid] = z;
            eroot[tid] = eS[(size_t)root * TC + tid];
            if (tid < ncols) {
                if (z > 0.0) {
                    tl = log(z) + (double)eroot[tid] * 0.69314718055994530942;
                    te = wz / z;
                } else {
                    tl = -INFINITY;
                }
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            tl += __shfl_down_sync(0xffffffffu, tl, o);
            te += __shfl_down_sync(0xffffffffu, te, o);
        }
        if ((tid & 31) == 0) { wsum_l[tid >> 5] = tl; wsum_e[tid >> 5] = te; }
        // beta~_root = prior, f(root) = 0
        {
            T *Br = B + (size_t)(root - nl) * K * TC;
            const double *pr = a.m.prior + md * K;
            for (int f = tid; f < K * TC; f += GR_THREADS) Br[f] = (T)pr[f / TC];
            for (int f = tid; f < TC; f += GR_THREADS) fS[(size_t)root * TC + f] = 0;
        }
        __syncthreads();
        if (tid == 0) {
            double sl = 0.0, se = 0.0;
            for (int k = 0; k < (TC + 31) / 32; k++) { sl += wsum_l[k]; se += wsum_e[k]; }
            a.partials[2 * (size_t)w] = sl;
            a.partials[2 * (size_t)w + 1] = se;
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
                __syncthreads();   // previous side finished with X, Mat[0], red, colmax, wsum
                if (internal) {
                    // E_c in row-major order (the buffer holds E_c^T)
                    const T *g = Pbase + (size_t)c * K2;
                    for (int f = tid; f < K2; f += GR_THREADS) {
                        int b = f / K, aa = f % K;
                        Mat[aa * K + b] = g[f];
                    }
                }
                for (int f = tid; f < TC; f += GR_THREADS) colmax[f] = 0;
                for (int f = tid; f < K * TC; f += GR_THREADS) X[f] = Bp[f] * vpart(Pbase, s, f / TC, f % TC);
                __syncthreads();
                // gradient: (Q^T inter) . v_c per column, summed over this thread's 4 states
                T wq[4][CPT];
                contract<T, TC, KAHAN>(Mat + 2 * K2, X, a0, c0, wq);
#pragma unroll
                for (int cc = 0; cc < CPT; cc++) {
                    T acc = (T)0;
#pragma unroll
                    for (int i = 0; i < 4; i++) acc += wq[i][cc] * vpart(Pbase, c, a0 + i, c0 + cc);
                    red[ty * TC + c0 + cc] = acc;
                }
                T bt[4][CPT];
                if (internal) {
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
                }
                __syncthreads();
                if (internal) {
                    T *Bc = B + (size_t)(c - nl) * K * TC;
#pragma unroll
                    for (int cc = 0; cc < CPT; cc++) {
                        const int col = c0 + cc;
                        T mx = AtomMax<T>::get(colmax + col);
                        int e = (mx > (T)0) ? exp_of(mx) : 0;
#pragma unroll
                        for (int i = 0; i < 4; i++) Bc[(size_t)(a0 + i) * TC + col] = scale2(bt[i][cc], -e);
                        if (ty == 0) fS[(size_t)c * TC + col] = fS[(size_t)p * TC + col] + e_of(s, col) + e;
                    }
                }
                double gl = 0.0;
                if (tid < TC && tid < ncols && zt[tid] > 0.0) {
                    double sum = 0.0;
                    for (int k = 0; k < 16; k++) sum += (double)red[k * TC + tid];
                    const int ex = fS[(size_t)p * TC + tid] + e_of(s, tid) + e_of(c, tid) - eroot[tid];
                    gl = ldexp(sum, ex) / zt[tid];
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) gl += __shfl_down_sync(0xffffffffu, gl, o);
                if ((tid & 31) == 0) wsum_l[tid >> 5] = gl;
                __syncthreads();
                if (tid == 0) {
                    double g = 0.0;
                    for (int k = 0; k < (TC + 31) / 32; k++) g += wsum_l[k];
                    a.gpart[(size_t)w * gstride + c] = g;
                }
                if (a.npar) {
                    // inter^T (dP_c / dx) alpha_c = p^T H_x q with p = U^T D^-1/2 inter, q = U^T D^1/2 alpha_c
                    const double *sqd = a.m.sq + md * K, *isqd = a.m.isq + md * K;
                    __syncthreads();   // wsum_l, red read; X still holds inter
                    for (int f = tid; f < K * TC; f += GR_THREADS) Qt[f] = X[f] * (T)isqd[f / TC];
                    __syncthreads();
                    T pv[4][CPT];
                    contract<T, TC, KAHAN>(Ubuf, Qt, a0, c0, pv);
                    __syncthreads();
                    if (internal) {
                        const T *Ac = Ascr + (size_t)(c - nl) * K * TC;
                        for (int f = tid; f < K * TC; f += GR_THREADS) Qt[f] = Ac[f] * (T)sqd[f / TC];
                    } else {
                        for (int f = tid; f < K * TC; f += GR_THREADS) {
                            const int st = f / TC, col = f % TC;
                            const int sl = lvT[c * TC + col];
                            Qt[f] = (sl >= K) ? (T)sqd[st] : (sl == st ? (T)sqd[st] : (T)0);
                        }
                    }
                    __syncthreads();
                    {
                        T qv[4][CPT];
                        contract<T, TC, KAHAN>(Ubuf, Qt, a0, c0, qv);
#pragma unroll
                        for (int i = 0; i < 4; i++)
#pragma unroll
                            for (int cc = 0; cc < CPT; cc++) Pt[(a0 + i) * TC + c0 + cc] = qv[i][cc];
                    }
                    for (int x = 0; x < a.npar; x++) {
                        const T *Hg = reinterpret_cast<const T *>(a.Hmat) +
                                      (((size_t)rq.pset * a.nbr + c) * a.npar + x) * K2;
                        for (int f = tid; f < K2; f += GR_THREADS) Hbuf[f] = Hg[f];
                        __syncthreads();   // Hbuf and the q tile (Pt) ready
                        T rv[4][CPT];
                        contract<T, TC, KAHAN>(Hbuf, Pt, a0, c0, rv);
#pragma unroll
                        for (int cc = 0; cc < CPT; cc++) {
                            T acc = (T)0;
#pragma unroll
                            for (int i = 0; i < 4; i++) acc += pv[i][cc] * rv[i][cc];
                            red[ty * TC + c0 + cc] = acc;
                        }
                        __syncthreads();
                        double gx = 0.0;
                        if (tid < TC && tid < ncols && zt[tid] > 0.0) {
                            double sum = 0.0;
                            for (int k = 0; k < 16; k++) sum += (double)red[k * TC + tid];
                            const int ex = fS[(size_t)p * TC + tid] + e_of(s, tid) + e_of(c, tid) - eroot[tid];
                            gx = ldexp(sum, ex) / zt[tid];
                        }
#pragma unroll
                        for (int o = 16; o > 0; o >>= 1) gx += __shfl_down_sync(0xffffffffu, gx, o);
                        if ((tid & 31) == 0) wsum_l[tid >> 5] = gx;
                        __syncthreads();
                        if (tid == 0)
                            for (int k = 0; k < (TC + 31) / 32; k++) pacc[x] += wsum_l[k];
                        __syncthreads();   // Hbuf, red, wsum_l free
                    }
                }
            }
        }
        if (a.npar && tid == 0)
            for (int x = 0; x < a.npar; x++) a.gpart[(size_t)w * gstride + a.nbr + x] = pacc[x];
    }
}

size_t grad_scratch_per_cta(int prec, int nl, int npar, bool recompute_leaves)
{
    if (prec == PCSF_PREC_FP64)
        return recompute_leaves ? GradLayout<double, 32, true>::scratch(nl, npar) : GradLayout<double, 32, false>::scratch(nl, npar);
    return recompute_leaves ? GradLayout<float, 64, true>::scratch(nl, npar) : GradLayout<float, 64, false>::scratch(nl, npar);
}

size_t grad_smem_bytes(int prec, int nslots, int nl, int nint, int npar)
{
    if (prec == PCSF_PREC_FP64) return GradLayout<double, 32, false>::smem(nslots, nl, nint, npar);
    return GradLayout<float, 64, false>::smem(nslots, nl, nint, npar);
}

template <typename T, int TC, int KAHAN, bool RECOMP>
static cudaError_t launch_grad_r(const GradArgs &a, cudaStream_t s, int grid)
{
    size_t smem = GradLayout<T, TC, RECOMP>::smem(a.nslots, a.nl, a.n_internal, a.npar);
    cudaError_t e = cudaFuncSetAttribute(k_grad<T, TC, KAHAN, RECOMP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_grad<T, TC, KAHAN, RECOMP><<<grid, GR_THREADS, smem, s>>>(a);
    return cudaGetLastError();
}

template <typename T, int TC, int KAHAN>
static cudaError_t launch_grad_t(const GradArgs &a, cudaStream_t s, int grid)
{
    return a.recompute_leaves ? launch_grad_r<T, TC, KAHAN, true>(a, s, grid) : launch_grad_r<T, TC, KAHAN, false>(a, s, grid);
}

cudaError_t launch_grad(int prec, int comp, const GradArgs &a, cudaStream_t s, int grid)
{
    if (a.nwi <= 0) return cudaSuccess;
    if (prec == PCSF_PREC_FP64) return launch_grad_t<double, 32, 0>(a, s, grid);
    if (comp == 1) return launch_grad_t<float, 64, 1>(a, s, grid);
    if (comp == 2) return launch_grad_t<float, 64, 2>(a, s, grid);
    return launch_grad_t<float, 64, 0>(a, s, grid);
}

// H_x^T = (F(t) o Bdot_x)^T per (P set, branch, parameter).  F_ij = (e^{lam_i t} -
// e^{lam_j t}) / (lam_i - lam_j), written as e^{lam_j t} (e^{d t} - 1) / d with
// d = lam_i - lam_j and a Taylor series in d t when |d t| < 1e-2 (no cancellation).
template <typename T>
__global__ void __launch_bounds__(256) k_hform(const PSet *ps, const double *branch, int nbr, const double *lam,
                                               const T *Bdot, T *H)
{
    __shared__ double el[K];
    const int b = blockIdx.x, r = blockIdx.y, tid = threadIdx.x;
    const PSet rq = ps[r];
    const int md = rq.model;
    const double t = rq.rho * branch[b];
    const double *lm = lam + (size_t)md * K;
    if (tid < K) el[tid] = exp(lm[tid] * t);
    __syncthreads();
    for (int f = tid; f < K2; f += 256) {
        const int i = f / K, j = f % K;
        const double d = lm[i] - lm[j], dt = d * t;
        double F;
        if (fabs(dt) < 1e-2) F = t * el[j] * (1.0 + dt * (0.5 + dt * (1.0 / 6.0 + dt * (1.0 / 24.0 + dt / 120.0))));
        else F = (el[i] - el[j]) / d;
        for (int x = 0; x < 2; x++)
            H[(((size_t)r * nbr + b) * 2 + x) * K2 + (size_t)j * K + i] = (T)(F * (double)Bdot[((size_t)md * 2 + x) * K2 + f]);
    }
}

cudaError_t launch_hform(bool fp64, const PSet *ps, int nps, const double *branch, int nbr, const double *lam,
                         const void *Bdot, void *H, cudaStream_t s)
{
    if (nps <= 0) return cudaSuccess;
    dim3 grid(nbr, nps);
    if (fp64) k_hform<double><<<grid, 256, 0, s>>>(ps, branch, nbr, lam, (const double *)Bdot, (double *)H);
    else k_hform<float><<<grid, 256, 0, s>>>(ps, branch, nbr, lam, (const float *)Bdot, (float *)H);
    return cudaGetLastError();
}

// grad[r][c] = sum of gpart over request r's work items (fixed order)
__global__ void k_reduce_grad(const double *gpart, const int32_t *wi_begin, int nreq, int nbr, double *grad)
{
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nreq * nbr) return;
    int r = idx / nbr, c = idx % nbr;
    double g = 0.0;
    for (int w = wi_begin[r]; w < wi_begin[r + 1]; w++) g += gpart[(size_t)w * nbr + c];
    grad[idx] = g;
}

cudaError_t launch_reduce_grad(const double *gpart, const int32_t *wi_begin, int nreq, int nbr, double *grad,
                               cudaStream_t s)
{
    if (nreq <= 0) return cudaSuccess;
    int tot = nreq * nbr;
    k_reduce_grad<<<(tot + 255) / 256, 256, 0, s>>>(gpart, wi_begin, nreq, nbr, grad);
    return cudaGetLastError();
}

}  // namespace pcsf
