// SIMT kernels of the likelihood engine: FP64 eigensolver, P(t) formation,
// Felsenstein pruning (FP64 and FP32) and the per-request reduction.
//
// Reference behaviour restated here (paths relative to mlin/PhyloCSF):
//   eigendecomposition  lib/CamlPaml/Q.ml:124-141 (GSL nonsymmv + complex LU in the
//                       reference; a parallel cyclic Jacobi on D^1/2 Q D^-1/2 here)
//   P(t) + row rule     lib/CamlPaml/Q.ml:211-249
//   inside pass         lib/CamlPaml/PhyloLik.ml:73-93
//   root posterior      lib/CamlPaml/PhyloLik.ml:127-138, src/PhyloCSFModel.ml:67-82
#include <cfloat>
#include <cmath>
#include <cstdio>

#include "pcsf_internal.h"
#include "prune_common.cuh"

namespace pcsf {

// ---------------------------------------------------------------------------
// Eigensolver: one CTA per symmetric 64x64 matrix, 256 threads.  Each Jacobi
// sweep visits all 2016 pairs as 63 rounds of 32 disjoint rotations (round-robin
// "circle" ordering), which are applied simultaneously.

constexpr int JAC_THREADS = 256;
constexpr int JAC_LD = K + 1;

__device__ inline void jac_pair(int r, int i, int &p, int &q)
{
    int a, b;
    if (i == 0) { a = K - 1; b = r; }
    else { a = (r + i) % (K - 1); b = (r - i + (K - 1)) % (K - 1); }
    p = a < b ? a : b;
    q = a < b ? b : a;
}

__global__ void __launch_bounds__(JAC_THREADS) k_jacobi(const double *A_in, double *U_out, double *lam_out,
                                                         int *status)
{
    extern __shared__ __align__(16) unsigned char jsm[];
    double *A = reinterpret_cast<double *>(jsm);      // [K][JAC_LD]
    double *V = A + K * JAC_LD;                        // [K][JAC_LD]
    double *red = V + K * JAC_LD;                      // [JAC_THREADS]
    double *cs = red + JAC_THREADS;                    // [32]
    double *sn = cs + 32;                              // [32]
    int *pp = reinterpret_cast<int *>(sn + 32);        // [32]
    int *qq = pp + 32;                                 // [32]
    const int tid = threadIdx.x;
    const double *Ain = A_in + (size_t)blockIdx.x * K2;

    for (int f = tid; f < K2; f += JAC_THREADS) {
        int i = f / K, j = f % K;
        A[i * JAC_LD + j] = Ain[f];
        V[i * JAC_LD + j] = (i == j) ? 1.0 : 0.0;
    }
    __syncthreads();
    // ||A||_F^2 (fixed-order tree reduction)
    double part = 0.0;
    for (int f = tid; f < K2; f += JAC_THREADS) {
        double x = A[(f / K) * JAC_LD + f % K];
        part += x * x;
    }
    red[tid] = part;
    __syncthreads();
    for (int w = JAC_THREADS / 2; w > 0; w >>= 1) {
        if (tid < w) red[tid] += red[tid + w];
        __syncthreads();
    }
    const double norm2 = red[0];
    __syncthreads();

    int converged = 0;
    for (int sweep = 0; sweep < 60; sweep++) {
        part = 0.0;
        for (int f = tid; f < K2; f += JAC_THREADS) {
            int i = f / K, j = f % K;
            if (i < j) { double x = A[i * JAC_LD + j]; part += x * x; }
        }
        red[tid] = part;
        __syncthreads();
        for (int w = JAC_THREADS / 2; w > 0; w >>= 1) {
            if (tid < w) red[tid] += red[tid + w];
            __syncthreads();
        }
        double off = red[0];
        __syncthreads();
        if (off <= 1e-32 * norm2) { converged = 1; break; }
        for (int r = 0; r < K - 1; r++) {
            if (tid < 32) {
                int p, q;
                jac_pair(r, tid, p, q);
                double apq = A[p * JAC_LD + q];
                double c = 1.0, s = 0.0;
                if (apq != 0.0) {
                    double theta = (A[q * JAC_LD + q] - A[p * JAC_LD + p]) / (2.0 * apq);
                    double t = (fabs(theta) > 1e150) ? 0.5 / theta
                               : (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                    c = 1.0 / sqrt(t * t + 1.0);
                    s = t * c;
                }
                cs[tid] = c; sn[tid] = s; pp[tid] = p; qq[tid] = q;
            }
            __syncthreads();
            for (int f = tid; f < K * 32; f += JAC_THREADS) {       // columns: A <- A J, V <- V J
                int row = f >> 5, k = f & 31;
                int p = pp[k], q = qq[k];
                double c = cs[k], s = sn[k];
                double a = A[row * JAC_LD + p], b = A[row * JAC_LD + q];
                A[row * JAC_LD + p] = c * a - s * b;
                A[row * JAC_LD + q] = s * a + c * b;
                double va = V[row * JAC_LD + p], vb = V[row * JAC_LD + q];
                V[row * JAC_LD + p] = c * va - s * vb;
                V[row * JAC_LD + q] = s * va + c * vb;
            }
            __syncthreads();
            for (int f = tid; f < K * 32; f += JAC_THREADS) {       // rows: A <- J^T A
                int col = f >> 5, k = f & 31;
                int p = pp[k], q = qq[k];
                double c = cs[k], s = sn[k];
                double a = A[p * JAC_LD + col], b = A[q * JAC_LD + col];
                A[p * JAC_LD + col] = c * a - s * b;
                A[q * JAC_LD + col] = s * a + c * b;
            }
            __syncthreads();
            if (tid < 32) {
                A[pp[tid] * JAC_LD + qq[tid]] = 0.0;
                A[qq[tid] * JAC_LD + pp[tid]] = 0.0;
            }
            __syncthreads();
        }
    }
    double *Uo = U_out + (size_t)blockIdx.x * K2;
    for (int f = tid; f < K2; f += JAC_THREADS) Uo[f] = V[(f / K) * JAC_LD + f % K];
    if (tid < K) lam_out[(size_t)blockIdx.x * K + tid] = A[tid * JAC_LD + tid];
    if (tid == 0) status[blockIdx.x] = converged ? 0 : 1;
}

cudaError_t launch_jacobi(const double *A, double *U, double *lam, int *status, int nmat, cudaStream_t s)
{
    size_t smem = sizeof(double) * (2 * K * JAC_LD + JAC_THREADS + 64) + sizeof(int) * 64;
    cudaError_t err = cudaFuncSetAttribute(k_jacobi, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    k_jacobi<<<nmat, JAC_THREADS, smem, s>>>(A, U, lam, status);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// P(t) formation.  For branch b of request r at t = rho_r * b_b:
//   E = P(t) - I = D^-1/2 U diag(expm1(lam t)) U^T D^1/2
// (expm1 in FP64; the 64^3 product in the storage precision T), then the row
// rule of Q.ml:226-247 on P = I + E:
//   - the raw row sum must be within tol of 1 (evaluated in FP64 through the
//     eigensystem identity sum_j E_ij = isq_i sum_m U_im expm1(lam_m t) w_m);
//   - off-diagonal negatives within tol are set to 0, below -tol are an error;
//   - the diagonal becomes 1 - sum of the off-diagonal entries, and must lie in
//     (0,1].
// Output is E^T: Pbuf[(r*nbr + b)*K2 + j*K + i] = E[i][j].

constexpr int PF_THREADS = 256;
constexpr int PF_BRANCHES = 4;   // branches per CTA (the eigenvectors are staged once)

template <typename T>
__global__ void __launch_bounds__(PF_THREADS) k_pform(const PSet *ps, const double *branch, int nbr,
                                                       DevModels m, T *Pbuf, int32_t *status_key, int raw,
                                                       float *Bop, int bop_nl, float *dlo)
{
    extern __shared__ __align__(16) unsigned char psm[];
    T *UT = reinterpret_cast<T *>(psm);     // [K][K]   UT[m][j] = U[j][m]
    T *UeT = UT + K2;                         // [K][K]   UeT[m][i] = U[i][m] * coef_m
    T *Es = UeT + K2;                         // [K][K+1] E[i][j]
    T *sqT = Es + K * (K + 1);                // [K]
    T *isqT = sqT + K;                        // [K]
    double *ex = reinterpret_cast<double *>(isqT + K);   // [K] expm1(lam t): row-sum identity
    double *cf = ex + K;                                 // [K] GEMM coefficients
    __shared__ T cfT[K];                                 // the same in the storage type
    __shared__ int mode_s[PF_BRANCHES], grid_s[PF_BRANCHES];
    const int tid = threadIdx.x;
    const int r = blockIdx.y;
    const PSet rq = ps[r];
    const int md = rq.model;
    const double *U = m.U + (size_t)md * K2;
    const float *Uf = m.Uf + (size_t)md * K2;
    const double *lam = m.lam + md * K;
    const double *isq = m.isq + md * K;
    const double *wrow = m.wrow + md * K;
    const bool fp32 = sizeof(T) == 4;

    for (int f = tid; f < K2; f += PF_THREADS) {
        int j = f / K, mm = f % K;   // U[j][mm]
        UT[mm * K + j] = fp32 ? (T)Uf[f] : (T)U[f];
    }
    if (tid < K) {
        sqT[tid] = (T)m.sq[md * K + tid];
        isqT[tid] = (T)isq[tid];
    }
    const int ty = tid / 16, tx = tid % 16;
    // per branch of this CTA, in parallel (one thread each; FP64 is a narrow pipe here):
    // 0: direct eigen formula (FP64);  1: t == 0;  2: Taylor below the grid;  3: grid correction
    if (tid < PF_BRANCHES) {
        const int b = blockIdx.x * PF_BRANCHES + tid;
        int mode = 0, g = 0;
        if (b < nbr && fp32 && m.grid_n > 0) {
            const double t = rq.rho * branch[b];
            if (t == 0.0) mode = 1;
            else if (t < m.grid_t[0]) mode = 2;
            else {
                mode = 3;
                double x = log(t / m.grid_t[0]) / m.grid_lr;
                g = (int)floor(x);
                if (g < 0) g = 0;
                if (g > m.grid_n - 1) g = m.grid_n - 1;
                if (g + 1 < m.grid_n && (m.grid_t[g + 1] - t) < (t - m.grid_t[g])) g++;
            }
        }
        mode_s[tid] = mode;
        grid_s[tid] = g;
    }
    for (int bi = 0; bi < PF_BRANCHES; bi++) {
        const int b = blockIdx.x * PF_BRANCHES + bi;
        if (b >= nbr) break;                       // uniform across the block
        const double t = rq.rho * branch[b];
        __syncthreads();                           // UT and the branch table ready / previous branch done with smem
        const int mode = mode_s[bi];
        if (tid < K) {
            // ex feeds the row-sum check, which needs it only where w_m != 0
            // (the stationary direction); the FP32 modes therefore spend one
            // FP64 expm1 per branch instead of 64 (FP64 is a narrow pipe here).
            if (mode == 0) {
                ex[tid] = expm1(lam[tid] * t);
                cf[tid] = ex[tid];
                cfT[tid] = (T)cf[tid];
            } else {
                ex[tid] = (wrow[tid] != 0.0) ? (double)expm1f((float)(lam[tid] * t)) : 0.0;   // row-sum check only
                if (mode == 3) {
                    // e^{lam t_g} (tabulated) * expm1(lam (t - t_g)) in FP32: the
                    // coefficient is rounded to FP32 for the GEMM in any case
                    const double h = t - m.grid_t[grid_s[bi]];
                    const float eg = m.grid_eg[((size_t)md * m.grid_n + grid_s[bi]) * K + tid];
                    cf[tid] = (double)(eg * expm1f((float)(lam[tid] * h)));
                    cfT[tid] = (T)cf[tid];
                }
            }
        }
        __syncthreads();
        if (mode == 0 || mode == 3) {
            for (int f = tid; f < K2; f += PF_THREADS) {
                int mm = f / K;
                UeT[f] = UT[f] * cfT[mm];
            }
            __syncthreads();
            // E(t_g) (stored transposed) for this thread's 4 x 4 block, loaded before the
            // GEMM: one 16-byte load per column jj (rows 4 ty .. 4 ty + 3)
            float gb[4][4];
            if (mode == 3) {
                const float *base = m.gridT + ((size_t)md * m.grid_n + grid_s[bi]) * K2;
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const float4 q = __ldg(reinterpret_cast<const float4 *>(base + (size_t)(4 * tx + j) * K + 4 * ty));
                    gb[j][0] = q.x; gb[j][1] = q.y; gb[j][2] = q.z; gb[j][3] = q.w;
                }
            }
            T acc[4][4];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] = (T)0;
            for (int mm = 0; mm < K; mm++) {
                T a[4], bb[4];
                Vec4<T>::load(UeT + mm * K + 4 * ty, a);
                Vec4<T>::load(UT + mm * K + 4 * tx, bb);
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int j = 0; j < 4; j++) acc[i][j] += a[i] * bb[j];
            }
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    int ii = 4 * ty + i, jj = 4 * tx + j;
                    T v = acc[i][j] * sqT[jj] * isqT[ii];
                    if (mode == 3) v += (T)gb[j][i];
                    Es[ii * (K + 1) + jj] = v;
                }
        } else {
            const float *Qf = m.Qf + (size_t)md * K2, *Q2f = m.Q2f + (size_t)md * K2;
            const T tt = (T)t, h = (T)(0.5 * t * t);
            for (int f = tid; f < K2; f += PF_THREADS) {
                int i = f / K, j = f % K;
                Es[i * (K + 1) + j] = (mode == 1) ? (T)0 : tt * (T)Qf[f] + h * (T)Q2f[f];
            }
        }
        __syncthreads();
        if (tid < K && !raw) {
            const int i = tid;
            // raw row sum - 1, in FP64 through the eigensystem
            const double rs = rowsum_minus_one(m, md, i, ex);
            // the diagonal is the compensated sum of the stored (rounded)
            // off-diagonal entries, so every stored row of P = I + E sums to 1
            // to within one rounding of the diagonal; a plain FP32 sum here
            // biases lpr by ~1e-4 nats per 3000 codons at rho = 1.  Branch-free in
            // j: i differs per lane, and a branch on j == i would split the warp.
            bool neg = false;
            T diag = (T)0, dc = (T)0;
            const T ntol = (T)(-m.tol), dtol = (T)(-1.0 - m.tol);
            for (int j = 0; j < K; j++) {
                const bool dj = (j == i);
                const T x0 = Es[i * (K + 1) + j];
                neg |= dj ? (x0 < dtol) : (x0 < ntol);   // diagonal: x + 1 < -tol
                const T x = (x0 < (T)0) ? (T)0 : x0;      // an off-diagonal negative within tol becomes 0
                if (!dj && x != x0) Es[i * (K + 1) + j] = x;
                if (fp32) {           // Kahan: diag -= x
                    const T y = -x - dc;
                    const T tt = diag + y;
                    const T c = (tt - diag) - y;
                    diag = dj ? diag : tt;
                    dc = dj ? dc : c;
                } else {
                    diag = dj ? diag : diag - x;
                }
            }
            if (neg) status_min(status_key + r, b, i, PCSF_ENEGP);
            else if (fabs(rs) > m.tol) status_min(status_key + r, b, i, PCSF_EROWSUM);
            else if (!(diag > (T)-1)) status_min(status_key + r, b, i, PCSF_EDIAG);
            // the sum is diag - dc to second order: its low part for the pruning kernel
            if (fp32 && dlo) dlo[((size_t)r * nbr + b) * K + i] = (float)(-dc);
            Es[i * (K + 1) + i] = diag;
        }
        __syncthreads();
        T *out = Pbuf + ((size_t)r * nbr + b) * K2;
        for (int f = tid; f < K2; f += PF_THREADS) {
            int j = f / K, i = f % K;
            out[f] = Es[i * (K + 1) + j];
        }
        if (fp32 && Bop && b >= bop_nl) {      // branch above an internal node: tensor-core operand too
            float *dst = Bop + ((size_t)r * (nbr - bop_nl) + (b - bop_nl)) * 2 * K2;
            for (int f = tid; f < K2 / 4; f += PF_THREADS) {
                const int a = f & (K - 1), q = f >> 6;
                const T *row = Es + a * (K + 1) + 4 * q;
                bop_store(dst, a, q, make_float4((float)row[0], (float)row[1], (float)row[2], (float)row[3]));
            }
        }
    }
}

cudaError_t launch_pform(bool fp64, const PSet *req, int nreq, const double *branch, int nbr, DevModels m,
                         void *Pbuf, int32_t *status_key, cudaStream_t s, bool raw, float *bop, int bop_nl, float *dlo)
{
    if (nreq <= 0) return cudaSuccess;
    dim3 grid((nbr + PF_BRANCHES - 1) / PF_BRANCHES, nreq);
    if (fp64) {
        size_t smem = sizeof(double) * (2 * K2 + K * (K + 1) + 4 * K);
        cudaError_t e = cudaFuncSetAttribute(k_pform<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k_pform<double><<<grid, PF_THREADS, smem, s>>>(req, branch, nbr, m, (double *)Pbuf, status_key, raw ? 1 : 0,
                                                       nullptr, 0, nullptr);
    } else {
        size_t smem = sizeof(float) * (2 * K2 + K * (K + 1) + 2 * K);
        smem = (smem + 15) & ~size_t(15);
        smem += sizeof(double) * 2 * K;
        cudaError_t e = cudaFuncSetAttribute(k_pform<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k_pform<float><<<grid, PF_THREADS, smem, s>>>(req, branch, nbr, m, (float *)Pbuf, status_key, raw ? 1 : 0,
                                                      bop, bop_nl, raw ? nullptr : dlo);
    }
    return cudaGetLastError();
}

__global__ void k_d2f(const double *in, float *out, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = (float)in[i];
}

cudaError_t launch_d2f(const double *in, float *out, size_t n, cudaStream_t s)
{
    k_d2f<<<264, 256, 0, s>>>(in, out, n);
    return cudaGetLastError();
}

// FP64 -> FP32 for E^T matrices that already obey the row rule: off-diagonal
// entries are rounded and each diagonal is re-formed as the FP64 sum of its
// row's rounded entries (storage E^T: element (i, j) of E at [j*K + i]).
// Matrices are [set][nbr]; with bop, the branches b >= bop_nl also get their
// tensor-core B operand (see bop_store).
__global__ void __launch_bounds__(256) k_d2f_rows(const double *in, float *out, size_t nmat, int nbr, float *bop,
                                                  int bop_nl, float *dlo)
{
    const size_t mat = blockIdx.x * (size_t)4 + threadIdx.x / K;
    const int i = threadIdx.x % K;
    if (mat >= nmat) return;
    const double *src = in + mat * K2;
    float *dst = out + mat * K2;
    double d = 0.0;
    for (int j = 0; j < K; j++) {
        if (j == i) continue;
        const float x = (float)src[j * K + i];
        dst[j * K + i] = x;
        d -= (double)x;
    }
    dst[i * K + i] = (float)d;
    if (dlo) dlo[mat * K + i] = (float)(d - (double)(float)d);   // low part of the diagonal
    const int b = (int)(mat % (size_t)nbr);
    if (bop && b >= bop_nl) {
        float *bd = bop + ((mat / nbr) * (size_t)(nbr - bop_nl) + (b - bop_nl)) * 2 * K2;
        for (int q = 0; q < K / 4; q++)
            bop_store(bd, i, q, make_float4(dst[(4 * q) * K + i], dst[(4 * q + 1) * K + i], dst[(4 * q + 2) * K + i],
                                            dst[(4 * q + 3) * K + i]));
    }
}

// any byte of w above 64: (b & 0x7F) + 63 reaches bit 7 exactly when b & 0x7F > 64
// (no carry between bytes: at most 190), and b's own bit 7 covers b >= 128
__device__ __forceinline__ bool bytes_above_64(uint32_t w)
{
    return ((((w & 0x7F7F7F7Fu) + 0x3F3F3F3Fu) | w) & 0x80808080u) != 0u;
}

__global__ void k_check_codes(const uint8_t *codes, size_t n, unsigned long long *first_bad)
{
    const size_t t0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (size_t)gridDim.x * blockDim.x;
    const size_t nv = n / 16;
    for (size_t v = t0; v < nv; v += stride) {
        const uint4 x = reinterpret_cast<const uint4 *>(codes)[v];
        if (bytes_above_64(x.x) || bytes_above_64(x.y) || bytes_above_64(x.z) || bytes_above_64(x.w))
            for (int j = 0; j < 16; j++)
                if (codes[16 * v + j] > 64) {
                    atomicMin(first_bad, (unsigned long long)(16 * v + j));
                    break;
                }
    }
    for (size_t i = 16 * nv + t0; i < n; i += stride)
        if (codes[i] > 64) atomicMin(first_bad, (unsigned long long)i);
}

cudaError_t launch_check_codes(const uint8_t *codes, size_t n, unsigned long long *first_bad, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    size_t blocks = (n / 16 + 255) / 256;
    if (blocks < 1) blocks = 1;
    if (blocks > 4096) blocks = 4096;
    k_check_codes<<<(unsigned)blocks, 256, 0, s>>>(codes, n, first_bad);
    return cudaGetLastError();
}

cudaError_t launch_d2f_rows(const double *in, float *out, size_t nmat, int nbr, float *bop, int bop_nl, cudaStream_t s,
                            float *dlo)
{
    if (nmat == 0) return cudaSuccess;
    k_d2f_rows<<<(unsigned)((nmat + 3) / 4), 256, 0, s>>>(in, out, nmat, nbr, bop, bop_nl, dlo);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Pruning (inside pass).  One CTA (256 threads) owns a tile of TC columns of
// one request's region and walks the internal nodes in the register-minimal
// (Sethi-Ullman) schedule computed on the host; partials live in shared
// memory slots [K][TC].  Thread (ty,tx) owns states 4ty..4ty+3 and columns
// tx*CPT..tx*CPT+CPT-1.
//
// For a child c of node i:   v_c[a] = alpha_c[a] + sum_j E_c[a][j] alpha_c[j]
// (internal child; E = P - I keeps the large diagonal exact; the sum is formed
// first, optionally with compensated summation, and alpha_c[a] added last), or the gather
// v_c[a] = P_c[a][s] for a leaf in state s (1 for a marginalised leaf: P rows
// sum to 1 after the row rule).  Then alpha_i = v_l * v_r, and each column is
// rescaled by an exact power of two so its maximum lies in [0.5,1); the
// exponents are summed per column and added back as e*ln2 in FP64 at the root.

constexpr int PR_THREADS = 256;

template <typename T, int TC>
struct PruneSmem {
    static constexpr int CPT = TC / 16;
    static size_t bytes(int nslots, int nl, int nint)
    {
        size_t b = sizeof(T) * (2 * K2 + (size_t)nslots * K * TC);
        b += sizeof(typename AtomMax<T>::U) * 2 * TC;
        b += sizeof(int) * TC;
        b += sizeof(SchedNode) * nint;
        b = (b + 15) & ~size_t(15);
        b += (size_t)nl * TC;
        return (b + 15) & ~size_t(15);
    }
};

template <typename T, int TC, int KAHAN>
__global__ void __launch_bounds__(PR_THREADS) k_prune(PruneArgs a)
{
    constexpr int CPT = TC / 16;
    typedef typename AtomMax<T>::U MU;
    extern __shared__ __align__(16) unsigned char ssm[];
    T *Et = reinterpret_cast<T *>(ssm);                 // [2][K][K]
    T *slots = Et + 2 * K2;                              // [nslots][K][TC]
    MU *colmax = reinterpret_cast<MU *>(slots + (size_t)a.nslots * K * TC);   // [2][TC]
    int *cscale = reinterpret_cast<int *>(colmax + 2 * TC);                   // [TC]
    SchedNode *sched = reinterpret_cast<SchedNode *>(cscale + TC);            // [n_internal]
    size_t off = (reinterpret_cast<unsigned char *>(sched + a.n_internal) - ssm + 15) & ~size_t(15);
    uint8_t *lvT = ssm + off;                                                  // [nl][TC]

    const int tid = threadIdx.x;
    const int ty = tid / 16, tx = tid % 16;
    const int a0 = 4 * ty, c0 = CPT * tx;
    const int nl = a.nl;
    __shared__ double red_l[PR_THREADS / 32], red_e[PR_THREADS / 32];
    __shared__ double ltab[256];           // log(1 + k/256), the dither factors' logs
    __shared__ double dsum[TC];            // per column: sum over leaves of log c
    const bool dith = a.dither && sizeof(T) == 4;

    for (int f = tid; f < a.n_internal; f += PR_THREADS) sched[f] = a.sched[f];
    if (dith)
        for (int f = tid; f < 256; f += PR_THREADS) ltab[f] = log1p((double)f / 256.0);

    for (int w = blockIdx.x; w < a.nwi; w += gridDim.x) {
        const WorkItem wi = a.wi[w];
        const Request rq = a.req[wi.request];
        const int md = rq.model;
        const T *Pbase = reinterpret_cast<const T *>(a.Pbuf) + (size_t)rq.pset * a.nbr * K2;
        // low parts of diag(E) of this P set (FP32 only)
        const float *dlo = (sizeof(T) == 4 && a.dlo) ? a.dlo + (size_t)rq.pset * a.nbr * K : nullptr;
        const int ncols = wi.ncols;
        const uint8_t *lg = a.leaves + (size_t)wi.col0 * nl;
        // E^T of a node's internal children into shared memory, copied asynchronously one
        // node ahead (issued once the previous node's contraction has released the
        // buffers); leaf children read their rows from global memory instead
        auto copy_inner = [&](const SchedNode &nx) {
            constexpr int NV = K2 * sizeof(T) / 16;
#pragma unroll
            for (int side = 0; side < 2; side++) {
                if ((side ? nx.rslot : nx.lslot) < 0) continue;
                const char *src = reinterpret_cast<const char *>(Pbase + (size_t)(side ? nx.rc : nx.lc) * K2);
                const uint32_t dst = (uint32_t)__cvta_generic_to_shared(Et + side * K2);
                for (int f = tid; f < NV; f += PR_THREADS)
                    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" :: "r"(dst + 16 * f), "l"(src + 16 * f)
                                 : "memory");
            }
            asm volatile("cp.async.commit_group;" ::: "memory");
        };
        __syncthreads();   // previous work item finished with shared memory
        for (int f = tid; f < TC * nl; f += PR_THREADS) {
            int c = f / nl, l = f - c * nl;
            lvT[l * TC + c] = (c < ncols) ? lg[f] : (uint8_t)K;
        }
        for (int f = tid; f < 2 * TC; f += PR_THREADS) colmax[f] = 0;
        for (int f = tid; f < TC; f += PR_THREADS) cscale[f] = 0;
        // dither keys are the column's position within its region, so that results
        // do not depend on where a region sits in the batch
        const int64_t dcol0 = dith ? (int64_t)(uint32_t)((uint32_t)wi.col0 - rq.start) : -1;
        if (dith) {
            __syncthreads();   // ltab ready
            for (int c = tid; c < TC; c += PR_THREADS) {
                double sd = 0.0;
                for (int l = 0; l < nl; l++) sd += ltab[dither_k(dcol0 + c, l)];
                dsum[c] = sd;
            }
        }

        copy_inner(sched[0]);
        for (int ni = 0; ni < a.n_internal; ni++) {
            const SchedNode sn = sched[ni];
            asm volatile("cp.async.wait_all;" ::: "memory");
            __syncthreads();
            T vl[4][CPT], vr[4][CPT];
            child_partial<T, TC, KAHAN>(Et, slots, sn.lslot, sn.lc, lvT, a0, c0, vl, dcol0, Pbase + (size_t)sn.lc * K2,
                                        dlo ? dlo + (size_t)sn.lc * K : nullptr);
            child_partial<T, TC, KAHAN>(Et + K2, slots, sn.rslot, sn.rc, lvT, a0, c0, vr, dcol0,
                                        Pbase + (size_t)sn.rc * K2, dlo ? dlo + (size_t)sn.rc * K : nullptr);
            __syncthreads();
            if (ni + 1 < a.n_internal) copy_inner(sched[ni + 1]);   // E^T buffers are free again
            MU *cm = colmax + (ni & 1) * TC;
            MU *cm_next = colmax + ((ni + 1) & 1) * TC;
            if (tid < TC) cm_next[tid] = 0;
#pragma unroll
            for (int cc = 0; cc < CPT; cc++) {
                T mx = (T)0;
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    vl[i][cc] *= vr[i][cc];
                    mx = vl[i][cc] > mx ? vl[i][cc] : mx;
                }
                AtomMax<T>::upd(cm + c0 + cc, mx);
            }
            __syncthreads();
            T *out = slots + (size_t)sn.oslot * K * TC;
            int ecol[CPT];
#pragma unroll
            for (int cc = 0; cc < CPT; cc++) {
                const T mx = AtomMax<T>::get(cm + c0 + cc);
                ecol[cc] = (mx > (T)0) ? exp_of(mx) : 0;
                if (ty == 0) cscale[c0 + cc] += ecol[cc];
            }
            // one vector store per state row (CPT consecutive columns): scalar stores
            // here were 4-way bank-conflicted
#pragma unroll
            for (int i = 0; i < 4; i++) {
                T y[CPT];
#pragma unroll
                for (int cc = 0; cc < CPT; cc++) y[cc] = scale2(vl[i][cc], -ecol[cc]);
                ColStore<T, CPT>::store(out + (a0 + i) * TC + c0, y);
            }
        }
        __syncthreads();
        // root: z = alpha_root . prior ; elpr term = (alpha_root . prior*log prior) / z
        double tl = 0.0, te = 0.0;
        if (tid < TC && tid < ncols) {
            const T *ar = slots + (size_t)sched[a.n_internal - 1].oslot * K * TC;
            const double *pr = a.m.prior + md * K;
            const double *wl = a.m.wlog + md * K;
            double z = 0.0, wz = 0.0;
            for (int s = 0; s < K; s++) {
                double x = (double)ar[s * TC + tid];
                z += x * pr[s];
                wz += x * wl[s];
            }
            if (z > 0.0) {
                tl = log(z) + (double)cscale[tid] * 0.69314718055994530942 - (dith ? dsum[tid] : 0.0);
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
        if ((tid & 31) == 0) { red_l[tid >> 5] = tl; red_e[tid >> 5] = te; }
        __syncthreads();
        if (tid == 0) {
            double sl = 0.0, se = 0.0;
            for (int k = 0; k < (TC + 31) / 32; k++) { sl += red_l[k]; se += red_e[k]; }
            a.partials[2 * (size_t)w] = sl;
            a.partials[2 * (size_t)w + 1] = se;
        }
    }
}

int prune_tile_cols(int prec)
{
    if (prec == PCSF_PREC_TF32X3 || prec == PCSF_PREC_TF32 || prec == PCSF_PREC_BF16X3) return 128;
    return prec == PCSF_PREC_FP64 ? 32 : 64;
}

// Column tile of the SIMT pruning kernel.  FP32 uses 64 columns, except for trees of
// five or more partial slots (the 120-leaf tree): there 64 columns take ~124 KB of
// shared memory, one CTA per SM, and 32 columns let two CTAs share an SM.
// tile (32 or 64) overrides this rule for the FP32 kernel (the engine's autotuner sets it).
int simt_tile_cols(int prec, int nslots, int tile)
{
    if (prec == PCSF_PREC_FP64) return 32;
    if (tile == 32 || tile == 64) return tile;
    return nslots >= 5 ? 32 : 64;
}

size_t prune_smem_bytes(int prec, int nslots, int nl, int nint, int tile)
{
    if (prec == PCSF_PREC_FP64) return PruneSmem<double, 32>::bytes(nslots, nl, nint);
    if (simt_tile_cols(prec, nslots, tile) == 32) return PruneSmem<float, 32>::bytes(nslots, nl, nint);
    return PruneSmem<float, 64>::bytes(nslots, nl, nint);
}

template <typename T, int TC, int KAHAN>
static cudaError_t launch_prune_t(const PruneArgs &a, cudaStream_t s, int grid)
{
    size_t smem = PruneSmem<T, TC>::bytes(a.nslots, a.nl, a.n_internal);
    cudaError_t e = cudaFuncSetAttribute(k_prune<T, TC, KAHAN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_prune<T, TC, KAHAN><<<grid, PR_THREADS, smem, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_prune(int prec, int comp, const PruneArgs &a, cudaStream_t s, int grid)
{
    if (a.nwi <= 0) return cudaSuccess;
    if (prec == PCSF_PREC_FP64) return launch_prune_t<double, 32, 0>(a, s, grid);
    if (simt_tile_cols(prec, a.nslots, a.tile) == 32) {
        if (comp == 1) return launch_prune_t<float, 32, 1>(a, s, grid);
        if (comp == 2) return launch_prune_t<float, 32, 2>(a, s, grid);
        return launch_prune_t<float, 32, 0>(a, s, grid);
    }
    if (comp == 1) return launch_prune_t<float, 64, 1>(a, s, grid);
    if (comp == 2) return launch_prune_t<float, 64, 2>(a, s, grid);
    return launch_prune_t<float, 64, 0>(a, s, grid);
}

// ---------------------------------------------------------------------------
// Per-request sums of the work-item partials, in work-item order (deterministic).

__global__ void k_reduce(const double *partials, const int32_t *wi_begin, int nreq, double *out_lpr, double *out_elpr,
                         const int32_t *out_index)
{
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nreq) return;
    double sl = 0.0, se = 0.0;
    for (int w = wi_begin[r]; w < wi_begin[r + 1]; w++) {
        sl += partials[2 * (size_t)w];
        se += partials[2 * (size_t)w + 1];
    }
    const int o = out_index ? out_index[r] : r;
    out_lpr[o] = sl;
    out_elpr[o] = se;
}

cudaError_t launch_reduce(const double *partials, const int32_t *wi_begin, int nreq, double *out_lpr,
                          double *out_elpr, cudaStream_t s, const int32_t *out_index)
{
    if (nreq <= 0) return cudaSuccess;
    k_reduce<<<(nreq + 127) / 128, 128, 0, s>>>(partials, wi_begin, nreq, out_lpr, out_elpr, out_index);
    return cudaGetLastError();
}

}  // namespace pcsf
