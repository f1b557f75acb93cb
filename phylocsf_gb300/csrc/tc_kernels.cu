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
// TMEM (512 columns x 128 lanes x 32 bit): D_l cols [0,64), D_r [64,128), and
// up to six parked partials alpha (64 columns each) from col 128.  Shared memory
// holds the MMA operands in the K-major no-swizzle core-matrix layout (8 rows x
// 16 bytes per core matrix), written with 16-byte stores so that a warp covers
// one contiguous 512-byte run: A (alpha, 128 x 64) hi/lo for two children and B
// (E row-major, 64 x 64) hi/lo for two children.  Leaf children are gathers of
// E^T rows from L2 while the MMAs run.  The per-column rescale exponent is the
// maximum over the two threads of a column.
//
// Accuracy: the tensor cores' FP32 accumulation is not round-to-nearest: it
// rounds toward minus infinity (a measured mean of -5.7 ulp of the result over
// one K = 64 product, i.e. 8 accumulation steps, for positive and for negative
// results alike), so these values carry a small systematic error.  The engine therefore uses this
// kernel for the search evaluations of the rho maximisation and reports every
// returned likelihood from the compensated FP32 kernel.
//
// Every mbarrier wait is bounded; on timeout the kernel records an error, waits
// (again bounded) for its tensor-core work, releases its tensor memory and exits.
#include <cmath>
#include <cstdint>

#include "pcsf_internal.h"

namespace pcsf {

constexpr int TCP_THREADS = 256;     // two threads per tile column
constexpr int TCP_M = 128;
constexpr int TCP_MAX_SLOTS = 6;
constexpr int TCP_MAX_LEAVES = 160;
constexpr uint32_t TCP_TMEM_COLS = 512;
constexpr long TCP_WAIT_LIMIT = 1L << 22;

// shared-memory map (bytes)
constexpr uint32_t SM_A = 0;            // [2 children][hi,lo][128 x 64 fp32] = 4 x 32 KB
constexpr uint32_t SM_B = 131072;       // [2 children][hi,lo][64 x 64 fp32]  = 4 x 16 KB
constexpr uint32_t SM_LV = 196608;      // [nl][128] leaf states
constexpr uint32_t A_BYTES = 32768, B_BYTES = 16384;

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (r, k) of a K-major tf32 operand with G = rows/8 row
// groups: core matrix (g = r/8, q = k/4) at (q*G + g)*128, row r%8 at 16 B.
__device__ __forceinline__ uint32_t core_off(int r, int k, int G)
{
    return (uint32_t)((((k >> 2) * G + (r >> 3)) << 7) + ((r & 7) << 4) + ((k & 3) << 2));
}

// shared-memory matrix descriptor: start, leading (K) and stride (M/N) byte
// offsets between core matrices, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

__device__ __forceinline__ void mma_tf32(uint32_t dt, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc)
{
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                 " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n"
                 :: "r"(dt), "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v)
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; j++) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ void tmem_st16(uint32_t taddr, const float *v)
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};"
                 :: "r"(taddr), "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
                    "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
                    "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])), "r"(__float_as_uint(v[8])),
                    "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),
                    "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])),
                    "r"(__float_as_uint(v[15])));
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity)
{
    uint32_t done = 0;
    for (long it = 0; it < TCP_WAIT_LIMIT && !done; it++) {
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                     " selp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(done) : "r"(bar), "r"(parity) : "memory");
    }
    return done != 0;
}

__device__ __forceinline__ float tf32_hi(float x) { return __uint_as_float(__float_as_uint(x) & 0xFFFFE000u); }

template <int NPROD>
__global__ void __launch_bounds__(TCP_THREADS, 1) k_prune_tc(PruneArgs a, int *err)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ uint32_t tbase_s;
    __shared__ __align__(8) uint64_t bar;
    __shared__ SchedNode sched[TCP_MAX_LEAVES];
    __shared__ float cmax[2][TCP_M];
    __shared__ double zpart[2][2][TCP_M];
    __shared__ double red_l[TCP_THREADS / 32], red_e[TCP_THREADS / 32];

    const int tid = threadIdx.x, warp = tid >> 5;
    const int site = tid & (TCP_M - 1);          // tile column = TMEM lane
    const int half = tid >> 7;                    // states 32*half .. 32*half+31
    const int s0 = 32 * half;
    const int nl = a.nl;
    uint8_t *lvT = sm + SM_LV;
    const uint32_t barA = smem_addr(&bar);
    // kind::tf32, D f32, A/B tf32, both K-major, N = 64, M = 128
    const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_addr(&tbase_s)), "r"(TCP_TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(barA), "r"(1));
    for (int f = tid; f < a.n_internal; f += TCP_THREADS) sched[f] = a.sched[f];
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = tbase_s;
    const uint32_t lane_off = (uint32_t)((warp & 3) * 32) << 16;   // warp w reaches lanes 32*(w%4)..
    uint32_t phase = 0;
    bool ok = true;

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
            lvT[l * TCP_M + c] = (c < ncols) ? lg[f] : (uint8_t)K;
        }
        int escale = 0;     // this column's sum of rescale exponents

        for (int ni = 0; ni < a.n_internal && ok; ni++) {
            const SchedNode sn = sched[ni];
            const int slot_of[2] = {sn.lslot, sn.rslot};
            const int child[2] = {sn.lc, sn.rc};
            const bool any_mma = slot_of[0] >= 0 || slot_of[1] >= 0;
            // ---- stage B = E_c (row-major E[a][j]) hi / lo for internal children; float4 per (a, 4 j)
#pragma unroll
            for (int side = 0; side < 2; side++) {
                if (slot_of[side] < 0) continue;
                const float *g = Pbase + (size_t)child[side] * K2;   // E^T: g[j*64 + a] = E[a][j]
                unsigned char *bh = sm + SM_B + side * 2 * B_BYTES;
                unsigned char *bl = bh + B_BYTES;
                for (int f = tid; f < 16 * K; f += TCP_THREADS) {
                    const int aa = f & 63, q = f >> 6;
                    float4 x;
                    x.x = __ldg(g + (4 * q + 0) * K + aa);
                    x.y = __ldg(g + (4 * q + 1) * K + aa);
                    x.z = __ldg(g + (4 * q + 2) * K + aa);
                    x.w = __ldg(g + (4 * q + 3) * K + aa);
                    const float4 lo = make_float4(x.x - tf32_hi(x.x), x.y - tf32_hi(x.y), x.z - tf32_hi(x.z), x.w - tf32_hi(x.w));
                    const uint32_t o = core_off(aa, 4 * q, 8);
                    *reinterpret_cast<float4 *>(bh + o) = x;
                    *reinterpret_cast<float4 *>(bl + o) = lo;
                }
            }
            // ---- stage A = alpha_c (site-major) hi / lo from TMEM; this thread's 32 states
#pragma unroll
            for (int side = 0; side < 2; side++) {
                if (slot_of[side] < 0) continue;
                unsigned char *ah = sm + SM_A + side * 2 * A_BYTES;
                unsigned char *al = ah + A_BYTES;
                const uint32_t ts = tbase + lane_off + 128 + 64 * slot_of[side] + s0;
#pragma unroll
                for (int q = 0; q < 2; q++) {
                    float x[16];
                    tmem_ld16(ts + 16 * q, x);
#pragma unroll
                    for (int j4 = 0; j4 < 4; j4++) {
                        const float4 hv = make_float4(x[4 * j4], x[4 * j4 + 1], x[4 * j4 + 2], x[4 * j4 + 3]);
                        const float4 lv = make_float4(hv.x - tf32_hi(hv.x), hv.y - tf32_hi(hv.y), hv.z - tf32_hi(hv.z),
                                                      hv.w - tf32_hi(hv.w));
                        const uint32_t o = core_off(site, s0 + 16 * q + 4 * j4, 16);
                        *reinterpret_cast<float4 *>(ah + o) = hv;
                        *reinterpret_cast<float4 *>(al + o) = lv;
                    }
                }
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            tc_fence_before();
            __syncthreads();
            tc_fence_after();
            if (tid == 0 && any_mma) {
#pragma unroll
                for (int side = 0; side < 2; side++) {
                    if (slot_of[side] < 0) continue;
                    const uint32_t dt = tbase + 64 * side;
                    const uint32_t ah = smem_addr(sm + SM_A + side * 2 * A_BYTES), al = ah + A_BYTES;
                    const uint32_t bh = smem_addr(sm + SM_B + side * 2 * B_BYTES), bl = bh + B_BYTES;
                    uint32_t acc = 0;
                    if (NPROD == 3) {
                        for (int s = 0; s < 8; s++) {
                            mma_tf32(dt, sdesc(al + s * 4096, 2048, 128), sdesc(bh + s * 2048, 1024, 128), idesc, acc);
                            acc = 1;
                            mma_tf32(dt, sdesc(ah + s * 4096, 2048, 128), sdesc(bl + s * 2048, 1024, 128), idesc, 1);
                        }
                    }
                    for (int s = 0; s < 8; s++) {
                        mma_tf32(dt, sdesc(ah + s * 4096, 2048, 128), sdesc(bh + s * 2048, 1024, 128), idesc, acc);
                        acc = 1;
                    }
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                             :: "r"(barA) : "memory");
            }
            // leaf children: gather E^T row s (L2) while the MMAs run
            float v[32];
#pragma unroll
            for (int side = 0; side < 2; side++) {
                if (slot_of[side] >= 0) continue;
                const int s = lvT[child[side] * TCP_M + site];
                const float4 *row = reinterpret_cast<const float4 *>(Pbase + (size_t)child[side] * K2 + (size_t)(s < K ? s : 0) * K + s0);
#pragma unroll
                for (int j4 = 0; j4 < 8; j4++) {
                    float4 x = make_float4(1.f, 1.f, 1.f, 1.f);
                    if (s < K) {
                        x = __ldg(row + j4);
                        const int a0 = s0 + 4 * j4;
                        if (s >= a0 && s < a0 + 4) (&x.x)[s - a0] += 1.0f;
                    }
                    const float u[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
                    for (int k = 0; k < 4; k++) v[4 * j4 + k] = (side && slot_of[0] < 0) ? v[4 * j4 + k] * u[k] : u[k];
                }
            }
            if (any_mma) {
                bool done = mbar_wait(barA, phase);
                phase ^= 1u;
                if (__syncthreads_or(!done)) {
                    if (tid == 0) atomicExch(err, 1);
                    mbar_wait(barA, phase ^ 1u);   // a second bounded wait for the in-flight MMAs
                    ok = false;
                    break;
                }
            }
            tc_fence_after();
            // ---- epilogue: internal children v = alpha + D, product with the other child
#pragma unroll
            for (int side = 0; side < 2; side++) {
                if (slot_of[side] < 0) continue;
                const uint32_t tD = tbase + lane_off + 64 * side + s0;
                const uint32_t tS = tbase + lane_off + 128 + 64 * slot_of[side] + s0;
                // does v already hold the other child's partial?
                const bool have_other = (side == 1) || (slot_of[1] < 0);
#pragma unroll
                for (int q = 0; q < 2; q++) {
                    float d[16], x[16];
                    tmem_ld16(tD + 16 * q, d);
                    tmem_ld16(tS + 16 * q, x);
#pragma unroll
                    for (int j = 0; j < 16; j++) {
                        const float u = x[j] + d[j];
                        v[16 * q + j] = have_other ? v[16 * q + j] * u : u;
                    }
                }
            }
            float mx = 0.0f;
#pragma unroll
            for (int k = 0; k < 32; k++) mx = fmaxf(mx, v[k]);
            cmax[half][site] = mx;
            __syncthreads();
            mx = fmaxf(cmax[0][site], cmax[1][site]);
            int e = 0;
            if (mx > 0.0f) frexpf(mx, &e);
            escale += e;
            const uint32_t tO = tbase + lane_off + 128 + 64 * sn.oslot + s0;
#pragma unroll
            for (int q = 0; q < 2; q++) {
                float y[16];
#pragma unroll
                for (int j = 0; j < 16; j++) y[j] = ldexpf(v[16 * q + j], -e);
                tmem_st16(tO + 16 * q, y);
            }
            asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
            tc_fence_before();
            __syncthreads();
            tc_fence_after();
        }
        if (!ok) break;
        // ---- root: z = alpha_root . prior, elpr term, FP64 sums over the tile
        {
            const uint32_t tR = tbase + lane_off + 128 + 64 * sched[a.n_internal - 1].oslot + s0;
            const double *pr = a.m.prior + md * K + s0;
            const double *wl = a.m.wlog + md * K + s0;
            double z = 0.0, wz = 0.0;
#pragma unroll
            for (int q = 0; q < 2; q++) {
                float x[16];
                tmem_ld16(tR + 16 * q, x);
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    z += (double)x[j] * pr[16 * q + j];
                    wz += (double)x[j] * wl[16 * q + j];
                }
            }
            zpart[half][0][site] = z;
            zpart[half][1][site] = wz;
        }
        __syncthreads();
        double tl = 0.0, te = 0.0;
        if (half == 0 && site < ncols) {
            const double z = zpart[0][0][site] + zpart[1][0][site];
            const double wz = zpart[0][1][site] + zpart[1][1][site];
            if (z > 0.0) {
                tl = log(z) + (double)escale * 0.69314718055994530942;
                te = wz / z;
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
        tc_fence_before();
        __syncthreads();
        if (tid == 0) {
            double sl = 0.0, se = 0.0;
            for (int k = 0; k < TCP_THREADS / 32; k++) { sl += red_l[k]; se += red_e[k]; }
            a.partials[2 * (size_t)w] = sl;
            a.partials[2 * (size_t)w + 1] = se;
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tbase), "r"(TCP_TMEM_COLS));
}

size_t prune_tc_smem_bytes(int nl) { return SM_LV + (size_t)nl * TCP_M; }

bool prune_tc_supported(int nslots, int nl) { return nslots <= TCP_MAX_SLOTS && nl <= TCP_MAX_LEAVES; }

cudaError_t launch_prune_tc(int nprod, const PruneArgs &a, int *err, cudaStream_t s, int grid)
{
    if (a.nwi <= 0) return cudaSuccess;
    size_t smem = prune_tc_smem_bytes(a.nl);
    if (nprod == 3) {
        cudaError_t e = cudaFuncSetAttribute(k_prune_tc<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k_prune_tc<3><<<grid, TCP_THREADS, smem, s>>>(a, err);
    } else {
        cudaError_t e = cudaFuncSetAttribute(k_prune_tc<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k_prune_tc<1><<<grid, TCP_THREADS, smem, s>>>(a, err);
    }
    return cudaGetLastError();
}

}  // namespace pcsf
