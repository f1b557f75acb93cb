// Device helpers shared by the pruning and gradient kernels.
#pragma once
#include <cuda_runtime.h>

#include "pcsf_internal.h"

namespace pcsf {

template <typename T> struct Vec4;
template <> struct Vec4<float> {
    static __device__ inline void load(const float *p, float v[4])
    {
        float4 x = *reinterpret_cast<const float4 *>(p);
        v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
    }
};
template <> struct Vec4<double> {
    static __device__ inline void load(const double *p, double v[4])
    {
        double2 x = *reinterpret_cast<const double2 *>(p);
        double2 y = *reinterpret_cast<const double2 *>(p + 2);
        v[0] = x.x; v[1] = x.y; v[2] = y.x; v[3] = y.y;
    }
};

template <typename T> struct AtomMax;
template <> struct AtomMax<float> {
    typedef int U;
    static __device__ inline void upd(U *p, float v) { atomicMax(p, __float_as_int(v)); }
    static __device__ inline float get(const U *p) { return __int_as_float(*p); }
};
template <> struct AtomMax<double> {
    typedef unsigned long long U;
    static __device__ inline void upd(U *p, double v) { atomicMax(p, (unsigned long long)__double_as_longlong(v)); }
    static __device__ inline double get(const U *p) { return __longlong_as_double((long long)*p); }
};

template <typename T, int CPT> struct ColLoad;
template <> struct ColLoad<float, 4> {
    static __device__ inline void load(const float *p, float v[4]) { Vec4<float>::load(p, v); }
};
template <> struct ColLoad<float, 2> {
    static __device__ inline void load(const float *p, float v[2])
    {
        float2 x = *reinterpret_cast<const float2 *>(p);
        v[0] = x.x; v[1] = x.y;
    }
};
template <> struct ColLoad<double, 2> {
    static __device__ inline void load(const double *p, double v[2])
    {
        double2 x = *reinterpret_cast<const double2 *>(p);
        v[0] = x.x; v[1] = x.y;
    }
};
template <> struct ColLoad<double, 4> {
    static __device__ inline void load(const double *p, double v[4]) { Vec4<double>::load(p, v); }
};

template <typename T, int CPT> struct ColStore;
template <> struct ColStore<float, 4> {
    static __device__ inline void store(float *p, const float v[4]) { *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]); }
};
template <> struct ColStore<float, 1> {
    static __device__ inline void store(float *p, const float v[1]) { *p = v[0]; }
};
template <> struct ColStore<float, 2> {
    static __device__ inline void store(float *p, const float v[2]) { *reinterpret_cast<float2 *>(p) = make_float2(v[0], v[1]); }
};
template <> struct ColStore<double, 2> {
    static __device__ inline void store(double *p, const double v[2]) { *reinterpret_cast<double2 *>(p) = make_double2(v[0], v[1]); }
};
template <> struct ColStore<double, 4> {
    static __device__ inline void store(double *p, const double v[4])
    {
        *reinterpret_cast<double2 *>(p) = make_double2(v[0], v[1]);
        *reinterpret_cast<double2 *>(p + 2) = make_double2(v[2], v[3]);
    }
};

// P(t) status keys: first error in (branch, row) order wins
__device__ __forceinline__ void status_min(int32_t *key, int branch, int row, int code)
{
    atomicMin(key, ((branch * K + row) << 4) | code);
}

// Tensor-core B operand of E (rows a, K = j): TF32 hi / lo parts in the K-major
// core-matrix layout of the tensor-core kernel (tc_kernels.cu), 16 KB each:
// element (a, j) at float offset (j/4)*256 + a*4 + j%4 of its part.
__device__ __forceinline__ void bop_store(float *dst, int a, int q, float4 x)
{
    // hi rounded to the nearest TF32 value (as tf32_hi in tc_common.cuh), lo = x - hi exact
    const float4 h = make_float4(__uint_as_float((__float_as_uint(x.x) + 0x1000u) & 0xFFFFE000u),
                                 __uint_as_float((__float_as_uint(x.y) + 0x1000u) & 0xFFFFE000u),
                                 __uint_as_float((__float_as_uint(x.z) + 0x1000u) & 0xFFFFE000u),
                                 __uint_as_float((__float_as_uint(x.w) + 0x1000u) & 0xFFFFE000u));
    const float4 l = make_float4(x.x - h.x, x.y - h.y, x.z - h.z, x.w - h.w);
    *reinterpret_cast<float4 *>(dst + q * 256 + a * 4) = h;
    *reinterpret_cast<float4 *>(dst + K2 + q * 256 + a * 4) = l;
}

// Row sum of the raw P(t) minus one, through the eigensystem: isq_i sum_m U_im
// expm1(lam_m t) w_m, where only the stationary direction(s) have w_m != 0;
// ex[m] = expm1(lam_m t) must be valid for those m.
__device__ __forceinline__ double rowsum_minus_one(const DevModels &m, int md, int i, const double *ex)
{
    const double *U = m.U + (size_t)md * K2 + (size_t)i * K;
    const double *w = m.wrow + md * K;
    const int16_t *wl = m.wlist + md * WLIST;
    double rs = 0.0;
    if (wl[0] == -2) {
        for (int mm = 0; mm < K; mm++)
            if (w[mm] != 0.0) rs += U[mm] * ex[mm] * w[mm];
    } else {
        for (int k = 0; k < WLIST && wl[k] >= 0; k++) rs += U[wl[k]] * ex[wl[k]] * w[wl[k]];
    }
    return rs * m.isq[md * K + i];
}

// Per-column dithering of the leaf partials (SIMT FP32 pruning): each leaf partial
// of column col is scaled by the exact factor c = 1 + k/256, k = dither_k(col, leaf),
// and sum_leaves log c is subtracted from the column's log-likelihood.  The values
// are mathematically unchanged; the FP32 rounding errors of columns that share
// sub-patterns (the same states below a node) stop being identical, so they no
// longer add up linearly over thousands of columns.
__device__ __forceinline__ int dither_k(int64_t col, int leaf)
{
    uint32_t h = (uint32_t)col * 0x9E3779B1u + (uint32_t)((uint64_t)col >> 32) * 0x7FEB352Du + (uint32_t)leaf * 0x85EBCA77u;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    h *= 0x297A2D39u;
    h ^= h >> 15;
    return (int)(h & 255u);
}

// exp_of(x): the e of frexp (x = m 2^e, m in [0.5, 1)) read from the exponent
// field for normal x; frexp itself for zero, subnormals and non-finite x.
__device__ __forceinline__ int exp_of(float x)
{
    const int b = (__float_as_int(x) >> 23) & 0xff;
    if (b != 0 && b != 0xff) return b - 126;
    int e;
    frexpf(x, &e);
    return e;
}
__device__ __forceinline__ int exp_of(double x)
{
    const int b = (int)((__double_as_longlong(x) >> 52) & 0x7ff);
    if (b != 0 && b != 0x7ff) return b - 1022;
    int e;
    frexp(x, &e);
    return e;
}
// scale2(x, e) = x * 2^e as two multiplications by exact powers of two (e split
// in halves of equal sign, so the intermediate lies between x and the result):
// exact, like ldexp, whenever x and the result are normal or zero; |e| <= 252
// (float) / 2044 (double), far beyond the per-node rescales.
__device__ __forceinline__ float scale2(float x, int e)
{
    const int e1 = e >> 1, e2 = e - e1;
    return x * __int_as_float((e1 + 127) << 23) * __int_as_float((e2 + 127) << 23);
}
__device__ __forceinline__ double scale2(double x, int e)
{
    const int e1 = e >> 1, e2 = e - e1;
    return x * __longlong_as_double((long long)(e1 + 1023) << 52) * __longlong_as_double((long long)(e2 + 1023) << 52);
}

// out[i][cc] = sum_j M[j][a0+i] * X[j][c0+cc] for a 64 x TC shared-memory tile
// X ([K][TC]) and a 64 x 64 matrix M ([K][K], row j contiguous).
// COMP selects the summation: 0 plain FP32 (products smaller than half an ulp of
// the running sum are lost, a downward bias), 1 Kahan on every term, 2 blocked:
// eight products summed plainly, then each block folded into the running sum
// with Kahan's correction (about a ninth of the plain bias at 1.5 operations per
// product instead of 5).
template <typename T, int TC, int COMP>
__device__ inline void contract(const T *M, const T *X, int a0, int c0, T out[4][TC / 16])
{
    constexpr int CPT = TC / 16;
    T comp[4][CPT];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int cc = 0; cc < CPT; cc++) {
            out[i][cc] = (T)0;
            comp[i][cc] = (T)0;
        }
    if (COMP == 2) {
        // a block's sum starts from its first product (0 + p rounds as p does), and the
        // first block is the running sum itself (its fold into zeros is exact, with a
        // zero correction): the same values as zero-initialised sums and folds, with
        // fewer instructions in this issue-bound loop
        auto block = [&](int jb, T g[4][CPT]) {
#pragma unroll
            for (int j = jb; j < jb + 8; j++) {
                T e[4], x[CPT];
                Vec4<T>::load(M + j * K + a0, e);
                ColLoad<T, CPT>::load(X + j * TC + c0, x);
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int cc = 0; cc < CPT; cc++) g[i][cc] = (j == jb) ? e[i] * x[cc] : fma(e[i], x[cc], g[i][cc]);
            }
        };
        block(0, out);
#pragma unroll 1
        for (int jb = 8; jb < K; jb += 8) {
            T g[4][CPT];
            block(jb, g);
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int cc = 0; cc < CPT; cc++) {
                    T y = g[i][cc] - comp[i][cc];
                    T t = out[i][cc] + y;
                    comp[i][cc] = (t - out[i][cc]) - y;
                    out[i][cc] = t;
                }
        }
    } else {
#pragma unroll 4
        for (int j = 0; j < K; j++) {
            T e[4], x[CPT];
            Vec4<T>::load(M + j * K + a0, e);
            ColLoad<T, CPT>::load(X + j * TC + c0, x);
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int cc = 0; cc < CPT; cc++) {
                    if (COMP == 1) {
                        // compensated summation: the rounding error of each addition is
                        // carried in comp, so small terms are not lost against a large sum
                        T y = e[i] * x[cc] - comp[i][cc];
                        T t = out[i][cc] + y;
                        comp[i][cc] = (t - out[i][cc]) - y;
                        out[i][cc] = t;
                    } else {
                        out[i][cc] += e[i] * x[cc];
                    }
                }
        }
    }
    if (COMP) {
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int cc = 0; cc < CPT; cc++) out[i][cc] -= comp[i][cc];
    }
}

// Partial of child c at its parent: v[a] = alpha_c[a] + sum_j E_c[a][j] alpha_c[j]
// (internal child, slot >= 0; Et = E_c^T) or the gather v[a] = P_c[a][s] of a
// leaf in state s (1 for a marginalised leaf: P rows sum to 1).
template <typename T, int TC, int KAHAN>
__device__ inline void child_partial(const T *Et, const T *slots, int slot, int leaf, const uint8_t *lvT, int a0,
                                     int c0, T v[4][TC / 16], int64_t dither_col0 = -1, const T *leaf_g = nullptr,
                                     const float *dlo = nullptr)
{
    constexpr int CPT = TC / 16;
    // dlo (may be null): the low parts of this branch's diag(E), added to the diagonal
    // term: FP32 storage of E_ii is the one rounding that every column sharing a state
    // at this node repeats identically, so over a long region it adds up coherently
    // (2-3e-3 dB over 10,000 codons at rho = 3 without it)
    if (slot < 0) {
        if (leaf_g) {   // the leaf's E^T rows straight from global memory (4 states per column)
#pragma unroll
            for (int cc = 0; cc < CPT; cc++) {
                const int s = lvT[leaf * TC + c0 + cc];
                const T c = (dither_col0 >= 0) ? (T)(1.0f + (float)dither_k(dither_col0 + c0 + cc, leaf) * (1.0f / 256.0f))
                                               : (T)1;
                T e[4];
                Vec4<T>::load(leaf_g + (size_t)(s < K ? s : 0) * K + a0, e);
                const T lo_s = dlo ? (T)dlo[s < K ? s : 0] : (T)0;
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const int a = a0 + i;
                    T val = fma(e[i], c, (a == s ? c : (T)0));
                    if (a == s) {       // + c lo_s: the rounding error r of c (1 + E_ss) is recovered (exactly
                                        // when P_ss >= 1/2, where c - val is exact), so that lo_s enters
                                        // the one final rounding instead of vanishing below half an ulp of c
                        const T r = fma(e[i], c, c - val);
                        val = val + fma(lo_s, c, r);
                    }
                    v[i][cc] = (s >= K) ? c : val;
                }
            }
            return;
        }
#pragma unroll
        for (int cc = 0; cc < CPT; cc++) {
            int s = lvT[leaf * TC + c0 + cc];
            // with dithering, c * P[a][s] in one rounding (c exact, see dither_k)
            const T c = (dither_col0 >= 0) ? (T)(1.0f + (float)dither_k(dither_col0 + c0 + cc, leaf) * (1.0f / 256.0f))
                                           : (T)1;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                int a = a0 + i;
                v[i][cc] = (s >= K) ? c : fma(Et[s * K + a], c, (a == s ? c : (T)0));
            }
        }
        return;
    }
    const T *al = slots + (size_t)slot * K * TC;
    contract<T, TC, KAHAN>(Et, al, a0, c0, v);
    T lo[4] = {(T)0, (T)0, (T)0, (T)0};
    if (dlo) {
        const float4 l4 = *reinterpret_cast<const float4 *>(dlo + a0);
        lo[0] = (T)l4.x; lo[1] = (T)l4.y; lo[2] = (T)l4.z; lo[3] = (T)l4.w;
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {
        T x[CPT];
        ColLoad<T, CPT>::load(al + (a0 + i) * TC + c0, x);
#pragma unroll
        for (int cc = 0; cc < CPT; cc++) v[i][cc] = x[cc] + (dlo ? fma(lo[i], x[cc], v[i][cc]) : v[i][cc]);
    }
}

}  // namespace pcsf
