// Host runtime of the likelihood engine and its C-ABI (include/phylocsf_engine.h).
//
// Reference behaviour restated here (paths relative to mlin/PhyloCSF):
//   Q assembly / scaling   src/PhyloCSFModel.ml:11-30, lib/CamlPaml/PhyloModel.ml:76-84,94-106
//   lpr_leaves             src/PhyloCSFModel.ml:67-82
//   maximize_lpr           src/PhyloCSFModel.ml:84-99
//   find_init              lib/CamlPaml/Fit.ml:27-48
//   Brent maximiser        lib/CamlPaml/Fit.ml:3-24 (GSL "brent" fminimizer semantics)
//   FixedLik / MaxLik      src/PhyloCSFModel.ml:113-146
//
// Every region's two fits (coding, noncoding) are independent state machines
// that advance in lockstep rounds: each round gathers the tree scales every
// unfinished fit needs, evaluates all of them in one batched device pass
// (P(t) formation for each distinct (model, rho), then pruning over column
// tiles), and feeds the results back.  Evaluations are memoised per fit by
// exact rho, so repeated evaluations at the same point (which the reference
// performs and which give bit-identical results) are not recomputed.
#include <algorithm>
#include <array>
#include <thread>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <unordered_map>
#include <string>
#include <utility>
#include <vector>

#include "pcsf_internal.h"

using namespace pcsf;

namespace {

thread_local std::string g_static_error;

template <typename T> struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    ~DevBuf() { release(); }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    cudaError_t reserve(size_t count)
    {
        if (count <= n) return cudaSuccess;
        release();
        size_t want = std::max<size_t>(count, 1);
        cudaError_t e = cudaMalloc(&p, want * sizeof(T));
        if (e == cudaSuccess) n = want;
        return e;
    }
};

template <typename T> struct HostBuf {
    T *p = nullptr;
    size_t n = 0;
    ~HostBuf() { release(); }
    void release()
    {
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
    }
    cudaError_t reserve(size_t count)
    {
        if (count <= n) return cudaSuccess;
        release();
        size_t want = std::max<size_t>(count, 1);
        cudaError_t e = cudaMallocHost(&p, want * sizeof(T));
        if (e == cudaSuccess) n = want;
        return e;
    }
};

// SplitMix64: the stand-in for OCaml's Random in find_init (seed 0 per fit).
inline uint64_t splitmix64(uint64_t &s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
inline double uniform01(uint64_t &s) { return (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }

constexpr double GOLDEN = 0.3819660;
constexpr double SQRT_DBL_EPS = 1.4901161193847656e-08;

}  // namespace

void pcsf_internal_set_error(const std::string &msg) { g_static_error = msg; }

struct pcsf_engine {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[8] = {};
    int prec = PCSF_PREC_FP32;
    bool compensated = false;
    bool block_comp = false;
    bool tc_direct = false;
    bool pt64 = false;             // FP32 storage of FP64-formed P(t)
    int comp_mode() const { return compensated ? 1 : block_comp ? 2 : 0; }
    int accurate_comp() const { return block_comp ? 2 : 1; }
    bool has_models = false;
    std::string err;

    // tree
    int nl = 0, n = 0, nbr = 0;
    std::vector<int> parent, lch, rch;
    std::vector<double> branch;
    std::vector<SchedNode> sched;
    int nslots = 0;

    // models (host copies)
    double U[2][K2], lam[2][K], sq[2][K], isq[2][K], wrow[2][K], prior[2][K], wlog[2][K];
    int16_t wlist[2][WLIST];
    float Uf[2][K2];
    double tol = 1e-6;

    // device copies
    DevBuf<double> dU, dlam, dsq, disq, dwrow, dprior, dwlog, dbranch;
    DevBuf<int16_t> dwlist;
    DevBuf<float> dUf, dgridT, dgrid_eg, dQf, dQ2f;
    DevBuf<double> dgrid_t;
    DevBuf<SchedNode> dsched;
    DevModels dm{};

    // per-launch work buffers
    DevBuf<unsigned char> Pbuf;
    DevBuf<double> Pbuf64;
    DevBuf<float> Bop;             // tensor-core B operands of the branches above internal nodes
    DevBuf<float> dPfB;            // B operand of the tensor-core P(t) formation, per model
    DevBuf<float> dQop;            // B operand of Q for the tangent pass, per model
    DevBuf<unsigned char> dHmat;   // parameter-derivative matrices per chunk-local P set
    size_t smem_optin = 0;
    DevBuf<double> ddpart, ddrho, ddscr;
    bool dual_ok = false;          // the tangent pass fits this tree
    int tc_grid = 0;
    int tc_shape = 0;              // TF32 tensor-core search kernel's shape (set by pcsf_engine_autotune)
    // d lpr / d rho for the derivative rule of the search: 1 = central difference of two search
    // evaluations (tensor-core engines), 0 = the analytic tangent pass or adjoint
    int deriv_mode = 0;
    double tc_shape_ms[PCSF_TC_SHAPES] = {};   // the autotuner's time per pass of each shape (0: untimed)
    size_t pbuf_psets = 0;
    DevBuf<PSet> dps;
    DevBuf<Request> dreq;
    DevBuf<WorkItem> dwi;
    DevBuf<int32_t> dwib, dstatus;
    DevBuf<double> dpart, dlpr, delpr;
    // gradient path
    DevBuf<unsigned char> gscratch;
    bool grad_recompute = false;   // adjoint: recompute leaf children's partials instead of storing them
    DevBuf<double> dgpart, dgrad;
    DevBuf<float> dQrowf;
    DevBuf<double> dQrowd;
    HostBuf<double> hgrad;
    int grad_grid = 0;
    HostBuf<PSet> hps;
    HostBuf<Request> hreq;
    HostBuf<WorkItem> hwi;
    HostBuf<int32_t> hwib, hstatus;
    HostBuf<double> hlpr, helpr;
    int prune_grid = 0;
    int simt_tile = 0;             // SIMT column tile (0: the default rule; set by pcsf_engine_autotune)
    int smem_sm = 0;               // shared memory per SM, for the grid of a tile
    int ff_grid = 0;               // CTAs of the float-float kernel (0: the tree does not fit it)
    // returned values (and the accurate search decisions) of a region come from the
    // float-float kernel when columns x (n_leaves - 2) reaches this; FP32 and tensor-core
    // engines only (the FP64 engine is exact already)
    int64_t exact_min_units = 150000;
    int sm_count = 0;
    DevBuf<int> derr;     // set by a kernel whose bounded wait timed out
    DevBuf<unsigned long long> dbadcode;   // first invalid leaf code of an uploaded batch
    DevBuf<float> Dlo;    // [chunk P sets][nbr][K] low parts of diag(E) (SIMT FP32 evaluations)

    pcsf_stats stats{};

    int fail(int code, const char *fmt, ...)
    {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        err = buf;
        return code;
    }
    int cuda_fail(cudaError_t e, const char *what)
    {
        return fail(e == cudaErrorMemoryAllocation ? PCSF_ENOMEM : PCSF_ECUDA, "%s: %s", what, cudaGetErrorString(e));
    }
    ~pcsf_engine()
    {
        for (auto &e : ev)
            if (e) cudaEventDestroy(e);
        if (stream) cudaStreamDestroy(stream);
    }
};

// precisions whose search evaluations run on the tensor cores
static inline bool tc_prec(int prec)
{
    return prec == PCSF_PREC_TF32X3 || prec == PCSF_PREC_TF32 || prec == PCSF_PREC_BF16X3;
}

struct pcsf_batch {
    pcsf_engine *e = nullptr;
    int device = 0;       // the engine's device, for destroying the batch after its engine
    int nreg = 0;
    std::vector<int64_t> offs;
    int64_t total_cols = 0;
    DevBuf<uint8_t> dleaves;
};

#define CK(call, what)                                      \
    do {                                                    \
        cudaError_t _e = (call);                            \
        if (_e != cudaSuccess) return e->cuda_fail(_e, what); \
    } while (0)

// ---------------------------------------------------------------------------
// Tree: validation and the register-minimal evaluation schedule.

static int build_tree(pcsf_engine *e, const pcsf_tree *t)
{
    if (!t || !t->parent || !t->branch) return e->fail(PCSF_EINVAL, "tree: null pointer");
    int nl = t->n_leaves;
    if (nl < 2 || nl > MAX_LEAVES) return e->fail(PCSF_EINVAL, "tree: n_leaves=%d out of range [2,%d]", nl, MAX_LEAVES);
    int n = 2 * nl - 1;
    e->nl = nl;
    e->n = n;
    e->nbr = n - 1;
    e->parent.assign(t->parent, t->parent + n);
    e->branch.assign(t->branch, t->branch + n - 1);
    e->lch.assign(n, -1);
    e->rch.assign(n, -1);
    if (e->parent[n - 1] != -1) return e->fail(PCSF_EINVAL, "tree: parent[root] must be -1");
    for (int i = 0; i < n - 1; i++) {
        int p = e->parent[i];
        if (p < nl || p >= n || p <= i)
            return e->fail(PCSF_EINVAL, "tree: node %d has parent %d (T order needs nl <= parent, child < parent)", i, p);
        if (e->lch[p] < 0) e->lch[p] = i;
        else if (e->rch[p] < 0) e->rch[p] = i;
        else return e->fail(PCSF_EINVAL, "tree: node %d has more than two children", p);
        double b = e->branch[i];
        if (!(b >= 0.0) || !std::isfinite(b)) return e->fail(PCSF_EINVAL, "tree: branch %d has length %g", i, b);
    }
    for (int i = nl; i < n; i++)
        if (e->rch[i] < 0) return e->fail(PCSF_EINVAL, "tree: internal node %d is not bifurcating", i);

    // Sethi-Ullman need: leaf 0; internal max(na, nb+1) with na >= nb.
    std::vector<int> need(n, 0);
    for (int i = nl; i < n; i++) {
        int a = need[e->lch[i]], b = need[e->rch[i]];
        if (a < b) std::swap(a, b);
        need[i] = std::max(std::max(a, b + 1), 1);
    }
    e->nslots = need[n - 1];
    // emit post-order with the needier child first; slots from a free stack
    e->sched.clear();
    std::vector<int> slot_of(n, -1), free_slots;
    for (int s = e->nslots - 1; s >= 0; s--) free_slots.push_back(s);
    std::vector<std::pair<int, int>> stack;   // (node, state)
    stack.push_back({n - 1, 0});
    while (!stack.empty()) {
        auto [i, st] = stack.back();
        stack.pop_back();
        if (i < nl) continue;
        int first = e->lch[i], second = e->rch[i];
        if (need[second] > need[first]) std::swap(first, second);
        if (st == 0) {
            stack.push_back({i, 1});
            stack.push_back({second, 0});
            stack.push_back({first, 0});
            continue;
        }
        SchedNode sn{};
        sn.node = (int16_t)i;
        sn.lc = (int16_t)e->lch[i];
        sn.rc = (int16_t)e->rch[i];
        sn.lslot = (int8_t)slot_of[e->lch[i]];
        sn.rslot = (int8_t)slot_of[e->rch[i]];
        int out;
        if (slot_of[first] >= 0) out = slot_of[first];
        else if (slot_of[second] >= 0) out = slot_of[second];
        else {
            if (free_slots.empty()) return e->fail(PCSF_EINVAL, "tree: schedule ran out of slots");
            out = free_slots.back();
            free_slots.pop_back();
        }
        if (slot_of[first] >= 0 && slot_of[first] != out) free_slots.push_back(slot_of[first]);
        if (slot_of[second] >= 0 && slot_of[second] != out) free_slots.push_back(slot_of[second]);
        sn.oslot = (int8_t)out;
        slot_of[i] = out;
        e->sched.push_back(sn);
    }
    if ((int)e->sched.size() != nl - 1 || e->sched.back().node != n - 1)
        return e->fail(PCSF_EINVAL, "tree: schedule construction failed");
    return PCSF_OK;
}

// ---------------------------------------------------------------------------
// Models

// q_ij = s_ij pi_j, q_ii = -sum_{j != i} q_ij (ascending j), scale = -sum_i pi_i q_ii
// (ascending i), Q /= scale -- the evaluation order of the reference's
// expression trees (PhyloCSFModel.ml:11-30, PhyloModel.ml:76-84,94-106).
static int assemble_q(const double *S, const double *pi, double *Q)
{
    for (int i = 0; i < K; i++) {
        double tot = 0.0;
        for (int j = 0; j < K; j++) {
            double q = (i == j) ? 0.0 : S[i * K + j] * pi[j];
            Q[i * K + j] = q;
            if (i != j) tot = q + tot;
        }
        Q[i * K + i] = 0.0 - tot;
    }
    double scale = 0.0;
    for (int i = 0; i < K; i++)
        if (Q[i * K + i] != 0.0) scale = scale - pi[i] * Q[i * K + i];
    if (!(scale > 0.0)) return PCSF_ESCALE;
    for (int i = 0; i < K2; i++) Q[i] = Q[i] / scale;
    return PCSF_OK;
}

// FP32 P(t) formation support: E(t_g) = P(t_g) - I on a geometric grid
// t_g = t0 r^g (t0 = 1e-5, r = 1.002) formed in FP64 and stored in FP32, plus
// Q and Q^2 for t < t0.  A branch then needs only the FP32 correction
// D^-1/2 U diag(e^{lam t} - e^{lam t_g}) U^T D^1/2, whose rounding error is
// proportional to |t - t_g| <= 0.1% of t instead of t itself.  (The eigen-sum
// cancels heavily on the small entries of E; with r = 1.01 the correction's
// rounding still cost ~8e-5 nats per 3000 codons at rho = 0.05.)  About 6,200
// grid points per model for the bundled trees: 0.2 GB of FP32 matrices.
static int build_pt_grid(pcsf_engine *e, const double *Q[2])
{
    const double t0 = 1e-5, ratio = 1.002;
    double bmax = 0.0;
    for (double b : e->branch) bmax = std::max(bmax, b);
    const double tmax = std::max(10.5 * bmax, 1.0);
    const double lr = std::log(ratio);
    const int G = (int)std::ceil(std::log(tmax / t0) / lr) + 1;
    std::vector<double> gt(G);
    for (int g = 0; g < G; g++) gt[g] = t0 * std::exp(g * lr);
    CK(e->dgrid_t.reserve(G), "cudaMalloc");
    CK(e->dgridT.reserve((size_t)2 * G * K2), "cudaMalloc");
    CK(cudaMemcpyAsync(e->dgrid_t.p, gt.data(), sizeof(double) * G, cudaMemcpyHostToDevice, e->stream), "H2D grid");
    DevBuf<double> tmp;
    DevBuf<PSet> dps;
    DevBuf<int32_t> dst;
    CK(tmp.reserve((size_t)G * K2), "cudaMalloc");
    CK(dps.reserve(2), "cudaMalloc");
    CK(dst.reserve(2), "cudaMalloc");
    PSet ps[2] = {{0, 0, 1.0}, {1, 0, 1.0}};
    CK(cudaMemcpyAsync(dps.p, ps, sizeof ps, cudaMemcpyHostToDevice, e->stream), "H2D");
    for (int m = 0; m < 2; m++) {
        CK(launch_pform(true, dps.p + m, 1, e->dgrid_t.p, G, e->dm, tmp.p, dst.p + m, e->stream, true), "grid launch");
        CK(launch_d2f(tmp.p, e->dgridT.p + (size_t)m * G * K2, (size_t)G * K2, e->stream), "grid convert");
        e->stats.kernel_launches += 2;
    }
    std::vector<float> eg((size_t)2 * G * K);
    for (int m = 0; m < 2; m++)
        for (int g = 0; g < G; g++)
            for (int mm = 0; mm < K; mm++) eg[((size_t)m * G + g) * K + mm] = (float)std::exp(e->lam[m][mm] * gt[g]);
    CK(e->dgrid_eg.reserve((size_t)2 * G * K), "cudaMalloc");
    CK(cudaMemcpyAsync(e->dgrid_eg.p, eg.data(), sizeof(float) * eg.size(), cudaMemcpyHostToDevice, e->stream),
       "H2D grid");
    std::vector<float> qf(2 * K2), q2f(2 * K2);
    for (int m = 0; m < 2; m++)
        for (int i = 0; i < K; i++)
            for (int j = 0; j < K; j++) {
                double acc = 0.0;
                for (int k = 0; k < K; k++) acc += Q[m][i * K + k] * Q[m][k * K + j];
                qf[m * K2 + i * K + j] = (float)Q[m][i * K + j];
                q2f[m * K2 + i * K + j] = (float)acc;
            }
    CK(e->dQf.reserve(2 * K2), "cudaMalloc");
    CK(e->dQ2f.reserve(2 * K2), "cudaMalloc");
    CK(cudaMemcpyAsync(e->dQf.p, qf.data(), sizeof(float) * 2 * K2, cudaMemcpyHostToDevice, e->stream), "H2D");
    CK(cudaMemcpyAsync(e->dQ2f.p, q2f.data(), sizeof(float) * 2 * K2, cudaMemcpyHostToDevice, e->stream), "H2D");
    CK(cudaStreamSynchronize(e->stream), "P(t) grid");
    e->dm.gridT = e->dgridT.p;
    e->dm.grid_t = e->dgrid_t.p;
    e->dm.grid_eg = e->dgrid_eg.p;
    e->dm.grid_n = G;
    e->dm.grid_lr = lr;
    e->dm.Qf = e->dQf.p;
    e->dm.Q2f = e->dQ2f.p;
    return PCSF_OK;
}

// The eigen-directions with w_m != 0 (normally the stationary one alone), for
// the row-sum check of the P(t) kernels; wl[0] = -2 when there are more than WLIST.
static void make_wlist(const double *w, int16_t *wl)
{
    int k = 0;
    for (int mm = 0; mm < K; mm++)
        if (w[mm] != 0.0) {
            if (k == WLIST) { wl[0] = -2; return; }
            wl[k++] = (int16_t)mm;
        }
    for (; k < WLIST; k++) wl[k] = -1;
}

static int setup_models(pcsf_engine *e, const double *Q[2], const double *eq[2], const double *prior[2])
{
    // symmetric similarity transforms A = D^1/2 Q D^-1/2, eigendecomposed in FP64 on the device
    std::vector<double> A(2 * K2);
    for (int m = 0; m < 2; m++) {
        for (int i = 0; i < K; i++) {
            if (!(eq[m][i] > 0.0) || !std::isfinite(eq[m][i]))
                return e->fail(PCSF_EINVAL, "model %d: equilibrium frequency %d is %g (must be > 0)", m, i, eq[m][i]);
            if (!(prior[m][i] > 0.0)) return e->fail(PCSF_EINVAL, "model %d: prior %d is %g (must be > 0)", m, i, prior[m][i]);
            e->sq[m][i] = std::sqrt(eq[m][i]);
            e->isq[m][i] = 1.0 / e->sq[m][i];
            e->prior[m][i] = prior[m][i];
            e->wlog[m][i] = prior[m][i] * std::log(prior[m][i]);
        }
        for (int i = 0; i < K; i++)
            for (int j = 0; j < K; j++) {
                double aij = e->sq[m][i] * Q[m][i * K + j] / e->sq[m][j];
                double aji = e->sq[m][j] * Q[m][j * K + i] / e->sq[m][i];
                if (std::fabs(aij - aji) > 1e-8 * (std::fabs(aij) + std::fabs(aji)) + 1e-300)
                    return e->fail(PCSF_EINVAL, "model %d: Q is not reversible with respect to the given equilibrium (%d,%d)", m, i, j);
                A[m * K2 + i * K + j] = 0.5 * (aij + aji);
            }
    }
    DevBuf<double> dA, dUtmp, dl;
    DevBuf<int> dst;
    CK(dA.reserve(2 * K2), "cudaMalloc");
    CK(dUtmp.reserve(2 * K2), "cudaMalloc");
    CK(dl.reserve(2 * K), "cudaMalloc");
    CK(dst.reserve(2), "cudaMalloc");
    CK(cudaMemcpyAsync(dA.p, A.data(), sizeof(double) * 2 * K2, cudaMemcpyHostToDevice, e->stream), "H2D Q");
    CK(launch_jacobi(dA.p, dUtmp.p, dl.p, dst.p, 2, e->stream), "eigensolver launch");
    e->stats.kernel_launches += 1;
    int hst[2];
    CK(cudaMemcpyAsync(e->U, dUtmp.p, sizeof(double) * 2 * K2, cudaMemcpyDeviceToHost, e->stream), "D2H U");
    CK(cudaMemcpyAsync(e->lam, dl.p, sizeof(double) * 2 * K, cudaMemcpyDeviceToHost, e->stream), "D2H lambda");
    CK(cudaMemcpyAsync(hst, dst.p, sizeof(int) * 2, cudaMemcpyDeviceToHost, e->stream), "D2H status");
    CK(cudaStreamSynchronize(e->stream), "eigensolver");
    if (hst[0] || hst[1]) return e->fail(PCSF_EEIG, "eigensolver did not converge");

    for (int m = 0; m < 2; m++) {
        // w_m = sum_j U_jm sqrt(pi_j): nonzero (to rounding) only for the stationary mode
        double nrm = 0.0;
        for (int j = 0; j < K; j++) nrm += eq[m][j];
        nrm = std::sqrt(nrm);
        for (int mm = 0; mm < K; mm++) {
            double w = 0.0;
            for (int j = 0; j < K; j++) w += e->U[m][j * K + mm] * e->sq[m][j];
            e->wrow[m][mm] = (std::fabs(w) > 1e-9 * nrm) ? w : 0.0;
        }
        for (int i = 0; i < K2; i++) e->Uf[m][i] = (float)e->U[m][i];
        make_wlist(e->wrow[m], e->wlist[m]);
    }
    CK(e->dwlist.reserve(2 * WLIST), "cudaMalloc");
    CK(cudaMemcpyAsync(e->dwlist.p, e->wlist, sizeof(int16_t) * 2 * WLIST, cudaMemcpyHostToDevice, e->stream), "H2D");
    CK(e->dU.reserve(2 * K2), "cudaMalloc");
    CK(e->dUf.reserve(2 * K2), "cudaMalloc");
    CK(e->dlam.reserve(2 * K), "cudaMalloc");
    CK(e->dsq.reserve(2 * K), "cudaMalloc");
    CK(e->disq.reserve(2 * K), "cudaMalloc");
    CK(e->dwrow.reserve(2 * K), "cudaMalloc");
    CK(e->dprior.reserve(2 * K), "cudaMalloc");
    CK(e->dwlog.reserve(2 * K), "cudaMalloc");
    CK(cudaMemcpyAsync(e->dU.p, e->U, sizeof(double) * 2 * K2, cudaMemcpyHostToDevice, e->stream), "H2D");
    CK(cudaMemcpyAsync(e->dUf.p, e->Uf, sizeof(float) * 2 * K2, cudaMemcpyHostToDevice, e->stream), "H2D");
    CK(cudaMemcpyAsync(e->dlam.p, e->lam, sizeof(double) * 2 * K, cudaMemcpyHostToDevice, e->stream), "H2D");
    CK(cudaMemcpyAsync(e->dsq.p, e->sq, sizeof(double) * 2 * K, cudaMemcpyHostToDevice, e->stream), "H2D");
    CK(cudaMemcpyAsync(e->disq.p, e->isq, sizeof(double) * 2 * K, cudaMemcpyHostToDevice, e->stream), "H2D");
    CK(cudaMemcpyAsync(e->dwrow.p, e->wrow, sizeof(double) * 2 * K, cudaMemcpyHostToDevice, e->stream), "H2D");
    CK(cudaMemcpyAsync(e->dprior.p, e->prior, sizeof(double) * 2 * K, cudaMemcpyHostToDevice, e->stream), "H2D");
    CK(cudaMemcpyAsync(e->dwlog.p, e->wlog, sizeof(double) * 2 * K, cudaMemcpyHostToDevice, e->stream), "H2D");
    CK(cudaStreamSynchronize(e->stream), "model upload");
    e->dm.U = e->dU.p;
    e->dm.Uf = e->dUf.p;
    e->dm.lam = e->dlam.p;
    e->dm.sq = e->dsq.p;
    e->dm.isq = e->disq.p;
    e->dm.wrow = e->dwrow.p;
    e->dm.wlist = e->dwlist.p;
    e->dm.prior = e->dprior.p;
    e->dm.wlog = e->dwlog.p;
    e->dm.tol = e->tol;
    e->dm.grid_n = 0;
    e->has_models = true;
    if (e->prec == PCSF_PREC_TF32X3 || e->prec == PCSF_PREC_TF32) {
        // B operand of the tensor-core P(t) formation: B[j][m] = U_jm sqrt(pi_j), TF32 hi / lo,
        // K-major core-matrix layout (element (j, m) at float (m/4)*256 + j*4 + m%4 of its part)
        std::vector<float> bpf((size_t)2 * 2 * K2);
        for (int m = 0; m < 2; m++)
            for (int j = 0; j < K; j++)
                for (int mm = 0; mm < K; mm++) {
                    const float x = (float)(e->U[m][j * K + mm] * e->sq[m][j]);
                    uint32_t bits;
                    std::memcpy(&bits, &x, 4);
                    bits = (bits + 0x1000u) & 0xFFFFE000u;   // nearest TF32 value
                    float hi;
                    std::memcpy(&hi, &bits, 4);
                    const size_t o = (size_t)m * 2 * K2 + (mm / 4) * 256 + j * 4 + mm % 4;
                    bpf[o] = hi;
                    bpf[o + K2] = x - hi;
                }
        // B operand of Q for the tangent pass: B[a][j] = Q[a][j], same layout
        std::vector<float> qop((size_t)2 * 2 * K2);
        for (int m = 0; m < 2; m++)
            for (int aa = 0; aa < K; aa++)
                for (int j = 0; j < K; j++) {
                    const float x = (float)Q[m][aa * K + j];
                    uint32_t bits;
                    std::memcpy(&bits, &x, 4);
                    bits = (bits + 0x1000u) & 0xFFFFE000u;   // nearest TF32 value
                    float hi;
                    std::memcpy(&hi, &bits, 4);
                    const size_t o = (size_t)m * 2 * K2 + (j / 4) * 256 + aa * 4 + j % 4;
                    qop[o] = hi;
                    qop[o + K2] = x - hi;
                }
        CK(e->dQop.reserve(qop.size()), "cudaMalloc");
        CK(cudaMemcpyAsync(e->dQop.p, qop.data(), sizeof(float) * qop.size(), cudaMemcpyHostToDevice, e->stream), "H2D");
        e->dual_ok = prune_tc_dual_supported(e->nslots, e->nl);
        CK(e->dPfB.reserve(bpf.size()), "cudaMalloc");
        CK(cudaMemcpyAsync(e->dPfB.p, bpf.data(), sizeof(float) * bpf.size(), cudaMemcpyHostToDevice, e->stream), "H2D");
        CK(cudaStreamSynchronize(e->stream), "model upload");
    }
    {
        // Q row-major in both arithmetic types, for dP/dt = Q P(t) in the gradient
        std::vector<double> qd(2 * K2);
        std::vector<float> qf(2 * K2);
        for (int m = 0; m < 2; m++)
            for (int i = 0; i < K2; i++) {
                qd[m * K2 + i] = Q[m][i];
                qf[m * K2 + i] = (float)Q[m][i];
            }
        CK(e->dQrowd.reserve(2 * K2), "cudaMalloc");
        CK(e->dQrowf.reserve(2 * K2), "cudaMalloc");
        CK(cudaMemcpyAsync(e->dQrowd.p, qd.data(), sizeof(double) * 2 * K2, cudaMemcpyHostToDevice, e->stream), "H2D");
        CK(cudaMemcpyAsync(e->dQrowf.p, qf.data(), sizeof(float) * 2 * K2, cudaMemcpyHostToDevice, e->stream), "H2D");
        CK(cudaStreamSynchronize(e->stream), "Q upload");
    }
    if (e->prec != PCSF_PREC_FP64) {
        int rc = build_pt_grid(e, Q);
        if (rc) return rc;
    }
    return PCSF_OK;
}

// CTAs of the SIMT kernel for a column tile: as many per SM as shared memory allows (<= 8)
static int simt_grid(const pcsf_engine *e, int tile)
{
    const size_t smem = prune_smem_bytes(e->prec, e->nslots, e->nl, (int)e->sched.size(), tile);
    int per_sm = std::max(1, (int)((size_t)e->smem_sm / (smem + 1024)));
    return e->sm_count * std::min(per_sm, 8);
}

static int engine_init_common(pcsf_engine *e, const pcsf_tree *tree, int32_t flags)
{
    int prec = flags & 0xff;
    if (prec != PCSF_PREC_FP64 && prec != PCSF_PREC_FP32 && prec != PCSF_PREC_TF32X3 && prec != PCSF_PREC_TF32 &&
        prec != PCSF_PREC_BF16X3)
        return e->fail(PCSF_EINVAL, "precision mode %d is not available in this build", prec);
    e->prec = prec;
    e->compensated = (flags & PCSF_COMPENSATED) != 0;
    e->block_comp = (flags & PCSF_BLOCK_COMPENSATED) != 0;
    e->tc_direct = (flags & PCSF_TC_DIRECT) != 0;
    e->pt64 = (flags & PCSF_PT_FP64) != 0;
    int ndev = 0;
    cudaError_t ce = cudaGetDeviceCount(&ndev);
    if (ce != cudaSuccess || ndev == 0)
        return e->fail(PCSF_ECUDA, "no CUDA device: %s", ce != cudaSuccess ? cudaGetErrorString(ce) : "count is 0");
    int want = ((flags >> 8) & 0xff) - 1;
    if (want >= ndev) return e->fail(PCSF_EINVAL, "device %d requested, %d present", want, ndev);
    if (want >= 0) CK(cudaSetDevice(want), "cudaSetDevice");
    CK(cudaGetDevice(&e->device), "cudaGetDevice");
    cudaDeviceProp prop;
    CK(cudaGetDeviceProperties(&prop, e->device), "cudaGetDeviceProperties");
    if (!(prop.major == 10 && prop.minor == 3))
        return e->fail(PCSF_ECUDA, "device %d (%s) is sm_%d%d; this library is built for sm_103a only", e->device,
                       prop.name, prop.major, prop.minor);
    CK(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking), "cudaStreamCreate");
    for (auto &v : e->ev) CK(cudaEventCreate(&v), "cudaEventCreate");
    int rc = build_tree(e, tree);
    if (rc) return rc;
    CK(e->dbranch.reserve(e->nbr), "cudaMalloc");
    CK(e->dsched.reserve(e->sched.size()), "cudaMalloc");
    CK(cudaMemcpyAsync(e->dbranch.p, e->branch.data(), sizeof(double) * e->nbr, cudaMemcpyHostToDevice, e->stream), "H2D");
    CK(cudaMemcpyAsync(e->dsched.p, e->sched.data(), sizeof(SchedNode) * e->sched.size(), cudaMemcpyHostToDevice,
                       e->stream), "H2D");
    e->sm_count = prop.multiProcessorCount;
    e->smem_optin = prop.sharedMemPerBlockOptin;
    CK(e->derr.reserve(1), "cudaMalloc");
    CK(cudaMemsetAsync(e->derr.p, 0, sizeof(int), e->stream), "memset");
    const bool tc = e->prec == PCSF_PREC_TF32X3 || e->prec == PCSF_PREC_TF32;
    e->deriv_mode = tc_prec(e->prec) ? 1 : 0;   // tensor-core searches: central differences
    if (e->prec == PCSF_PREC_BF16X3) {
        if (!prune_bf16_supported(e->nslots, e->nl))
            return e->fail(PCSF_EINVAL, "BF16 tensor-core path supports up to 160 leaves and 8 partial slots");
        if (prune_bf16_smem_bytes(e->nl, (int)e->sched.size()) > (size_t)prop.sharedMemPerBlockOptin)
            return e->fail(PCSF_EINVAL, "BF16 tensor-core path needs %zu B shared memory",
                           prune_bf16_smem_bytes(e->nl, (int)e->sched.size()));
        e->tc_grid = prop.multiProcessorCount * prune_bf16_ctas_per_sm(e->nslots, e->nl, (int)e->sched.size());
    }
    if (tc && !prune_tc_supported(e->nslots, e->nl))
        return e->fail(PCSF_EINVAL, "tensor-core path supports up to 160 leaves and 8 partial slots (tree: %d, %d)",
                       e->nl, e->nslots);
    if (tc && prune_tc_smem_bytes(e->nl, (int)e->sched.size()) > (size_t)prop.sharedMemPerBlockOptin)
        return e->fail(PCSF_EINVAL, "tensor-core path needs %zu B shared memory",
                       prune_tc_smem_bytes(e->nl, (int)e->sched.size()));
    if (tc)
        e->tc_grid = prop.multiProcessorCount * prune_tc_ctas_per_sm(e->nslots, e->nl, (int)e->sched.size(), e->tc_shape);
    size_t smem = prune_smem_bytes(e->prec, e->nslots, e->nl, (int)e->sched.size());
    if (smem > (size_t)prop.sharedMemPerBlockOptin)
        return e->fail(PCSF_EINVAL, "tree needs %d partial slots (%zu B shared memory > %zu)", e->nslots, smem,
                       (size_t)prop.sharedMemPerBlockOptin);
    e->smem_sm = (int)prop.sharedMemPerMultiprocessor;
    e->prune_grid = simt_grid(e, 0);
    size_t gsmem = grad_smem_bytes(e->prec, e->nslots, e->nl, (int)e->sched.size(), 0);
    if (gsmem > (size_t)prop.sharedMemPerBlockOptin)
        return e->fail(PCSF_EINVAL, "tree needs %zu B shared memory for the gradient", gsmem);
    int gper = std::max(1, std::min(4, (int)(prop.sharedMemPerMultiprocessor / (gsmem + 1024))));
    e->grad_grid = prop.multiProcessorCount * gper;
    if (e->prec != PCSF_PREC_FP64 &&
        prune_ff_smem_bytes(e->nslots, e->nl, (int)e->sched.size()) <= (size_t)prop.sharedMemPerBlockOptin)
        e->ff_grid = prop.multiProcessorCount * std::max(1, prune_ff_ctas_per_sm(e->nslots, e->nl, (int)e->sched.size()));
    // P(t) buffer: up to 16 GiB, at most a quarter of free memory.  A round of the
    // search forms one P set per active fit (20,000 fits x 3.6 MB for 58 leaves), so
    // the chunk size sets how many launch pairs (P(t), pruning) a round takes and how
    // often a pruning launch ends in a partly filled wave.
    size_t freeb = 0, totalb = 0;
    CK(cudaMemGetInfo(&freeb, &totalb), "cudaMemGetInfo");
    size_t pset_bytes = (size_t)e->nbr * K2 * (e->prec == PCSF_PREC_FP64 ? 8 : 4);
    if (tc) pset_bytes += (size_t)(e->nbr - e->nl) * 2 * K2 * sizeof(float);   // B operands
    size_t budget = std::min<size_t>(size_t(16) << 30, freeb / 4);
    e->pbuf_psets = std::max<size_t>(1, budget / pset_bytes);
    return PCSF_OK;
}

// ---------------------------------------------------------------------------
// Batched evaluation of (region, model, rho) requests.

struct Eval {
    double lpr, elpr;
    int status;
};

// grad (optional): d lpr / d t_c per request, [nreq][nbr], by the adjoint kernel.
// accurate: on a tensor-core engine, use the compensated FP32 kernel instead
// (every likelihood the engine returns comes from it; see tc_kernels.cu).
// dyn: per-request models (Request.model indexes this table) instead of the
// engine's two fixed models; their P(t) is formed in FP64 (no FP32 grid exists
// for them) and the pruning runs on the SIMT kernels.
// Rate-matrix parameter derivatives for per-request models (OmegaModel kappa, omega):
// per model Q row-major, U, and Bdot_x = U^T D^1/2 (dQ/dx) D^-1/2 U, in the engine's
// arithmetic type.
struct DynGrad {
    const void *Qrow, *Umat, *Bdot;
};

// exact: the float-float kernel (FP64 P(t), ~1e-12 relative) instead of the FP32 one, on
// FP32 and tensor-core engines whose tree fits it; implies accurate.
static int evaluate(pcsf_engine *e, pcsf_batch *b, const std::vector<Request> &reqs_in, std::vector<Eval> &out,
                    std::vector<double> *grad = nullptr, bool accurate = false, const DevModels *dyn = nullptr,
                    std::vector<double> *drho = nullptr, const DynGrad *dg = nullptr, bool exact = false)
{
    const int nreq = (int)reqs_in.size();
    out.assign(nreq, Eval{0.0, 0.0, PCSF_OK});
    if (nreq == 0) return PCSF_OK;
    if (dyn && grad && !dg) return e->fail(PCSF_EINVAL, "gradients for per-request models need their derivatives");
    const int npar = (grad && dg) ? 2 : 0;
    const int gstride = e->nbr + npar;
    if (dyn) accurate = true;
    const bool ff = exact && !dyn && !grad && !drho && e->prec != PCSF_PREC_FP64 && e->ff_grid > 0;
    if (ff) accurate = true;
    const DevModels dmv = dyn ? *dyn : e->dm;
    if (drho && (grad || dyn || accurate || !e->dual_ok))
        return e->fail(PCSF_EINVAL, "d lpr / d rho by the tangent pass needs a tensor-core engine and a tree of <= 4 slots");
    const bool tc = tc_prec(e->prec) && !accurate;
    // the gradient always runs the SIMT adjoint kernel (64-column tiles in FP32)
    const int TC = grad ? (e->prec == PCSF_PREC_FP64 ? 32 : 64)
                        : ff ? ff_tile_cols() : !tc ? simt_tile_cols(e->prec, e->nslots, e->simt_tile)
                                                    : prune_tile_cols(e->prec);
    const int comp = (accurate && tc_prec(e->prec)) ? e->accurate_comp()
                                                                                              : e->comp_mode();

    const int kind = drho ? 3 : grad ? 2 : tc ? 1 : ff ? 4 : 0;
    // a float-float P set (8 B per entry) and its FP64 staging take four times an FP32 one
    const size_t chunk_psets = ff ? std::max<size_t>(1, e->pbuf_psets / 4) : e->pbuf_psets;
    int64_t kind_cols = 0;
    // work items, P-set dedup and chunking (at most pbuf_psets distinct P sets per chunk)
    std::vector<Request> reqs(reqs_in);
    std::vector<int> wib(nreq + 1, 0);
    std::vector<WorkItem> wis;
    std::vector<PSet> psets;
    std::vector<int> chunk_req_begin, chunk_ps_begin;   // chunk boundaries
    // (model, rho bits) -> chunk-local P set; a hash map: a search round asks for
    // ~20,000 distinct tree scales, and an ordered map's lookups showed in the host time
    struct PsKeyHash {
        size_t operator()(const std::pair<int, uint64_t> &k) const
        {
            return std::hash<uint64_t>()(k.second * 0x9E3779B97F4A7C15ull + (uint64_t)(uint32_t)k.first);
        }
    };
    std::unordered_map<std::pair<int, uint64_t>, int, PsKeyHash> cur;
    cur.reserve(std::min<size_t>((size_t)nreq, chunk_psets) * 2);
    wis.reserve((size_t)nreq * 8);
    chunk_req_begin.push_back(0);
    chunk_ps_begin.push_back(0);
    std::vector<int> req_pset_global(nreq);
    for (int r = 0; r < nreq; r++) {
        Request &q = reqs[r];
        uint64_t bits;
        std::memcpy(&bits, &q.rho, 8);
        auto key = std::make_pair(q.model, bits);
        auto it = cur.find(key);
        if (it == cur.end()) {
            if (cur.size() == chunk_psets) {
                chunk_req_begin.push_back(r);
                chunk_ps_begin.push_back((int)psets.size());
                cur.clear();
            }
            int local = (int)cur.size();
            cur[key] = local;
            psets.push_back(PSet{q.model, 0, q.rho});
            q.pset = local;
        } else {
            q.pset = it->second;
        }
        req_pset_global[r] = chunk_ps_begin.back() + q.pset;
        int64_t c0 = b->offs[q.region], c1 = b->offs[q.region + 1];
        q.start = (uint32_t)c0;
        wib[r] = (int)wis.size();
        for (int64_t c = c0; c < c1; c += TC) {
            WorkItem w;
            w.request = r;
            w.ncols = (int)std::min<int64_t>(TC, c1 - c);
            w.col0 = c;
            wis.push_back(w);
        }
        e->stats.column_branches += (c1 - c0) * (int64_t)e->nbr;
        kind_cols += c1 - c0;
    }
    wib[nreq] = (int)wis.size();
    chunk_req_begin.push_back(nreq);
    chunk_ps_begin.push_back((int)psets.size());
    const int nps = (int)psets.size(), nwi = (int)wis.size();
    e->stats.evaluations += nreq;

    CK(e->hps.reserve(nps), "cudaMallocHost");
    CK(e->hreq.reserve(nreq), "cudaMallocHost");
    CK(e->hwi.reserve(nwi), "cudaMallocHost");
    CK(e->hwib.reserve(nreq + 1), "cudaMallocHost");
    CK(e->hstatus.reserve(nps), "cudaMallocHost");
    CK(e->hlpr.reserve(nreq), "cudaMallocHost");
    CK(e->helpr.reserve(nreq), "cudaMallocHost");
    CK(e->dps.reserve(nps), "cudaMalloc");
    CK(e->dreq.reserve(nreq), "cudaMalloc");
    CK(e->dwi.reserve(nwi), "cudaMalloc");
    CK(e->dwib.reserve(nreq + 1), "cudaMalloc");
    CK(e->dstatus.reserve(nps), "cudaMalloc");
    CK(e->dpart.reserve(2 * (size_t)std::max(nwi, 1)), "cudaMalloc");
    CK(e->dlpr.reserve(nreq), "cudaMalloc");
    CK(e->delpr.reserve(nreq), "cudaMalloc");
    if (drho) {
        CK(e->ddpart.reserve(2 * (size_t)std::max(nwi, 1)), "cudaMalloc");
        CK(e->ddrho.reserve(nreq), "cudaMalloc");
        CK(e->ddscr.reserve(nreq), "cudaMalloc");
    }
    size_t pset_bytes = (size_t)e->nbr * K2 * (e->prec == PCSF_PREC_FP64 || ff ? 8 : 4);
    size_t max_chunk_ps = 0;
    for (size_t c = 0; c + 1 < chunk_ps_begin.size(); c++)
        max_chunk_ps = std::max<size_t>(max_chunk_ps, chunk_ps_begin[c + 1] - chunk_ps_begin[c]);
    CK(e->Pbuf.reserve(max_chunk_ps * pset_bytes), "cudaMalloc P(t) buffer");
    // low parts of diag(E) for the SIMT FP32 kernel (not for the tensor-core search)
    const bool want_dlo = e->prec != PCSF_PREC_FP64 && !tc && !grad && !ff;
    if (want_dlo) CK(e->Dlo.reserve(max_chunk_ps * (size_t)e->nbr * K), "cudaMalloc P(t) diagonal buffer");
    float *dlo = want_dlo ? e->Dlo.p : nullptr;
    const bool stage64 = (dyn || e->pt64) && e->prec != PCSF_PREC_FP64 && !ff;   // FP64 formation, then FP32 storage
    if (stage64 || ff) CK(e->Pbuf64.reserve(max_chunk_ps * (size_t)e->nbr * K2), "cudaMalloc P(t) staging buffer");
    const int nbop = e->nbr - e->nl;
    const bool want_bop = tc && !grad && e->prec != PCSF_PREC_BF16X3;   // the BF16 kernel splits E^T itself
    if (want_bop) CK(e->Bop.reserve(max_chunk_ps * (size_t)nbop * 2 * K2), "cudaMalloc tensor-core operand buffer");
    float *bop = want_bop ? e->Bop.p : nullptr;
    size_t gscr = 0;
    if (grad) {
        gscr = grad_scratch_per_cta(e->prec, e->nl, npar, e->grad_recompute);
        CK(e->gscratch.reserve(gscr * (size_t)e->grad_grid), "cudaMalloc gradient scratch");
        CK(e->dgpart.reserve((size_t)std::max(nwi, 1) * gstride), "cudaMalloc");
        CK(e->dgrad.reserve((size_t)nreq * gstride), "cudaMalloc");
        CK(e->hgrad.reserve((size_t)nreq * gstride), "cudaMallocHost");
        if (npar)
            CK(e->dHmat.reserve(max_chunk_ps * (size_t)e->nbr * npar * K2 * (e->prec == PCSF_PREC_FP64 ? 8 : 4)),
               "cudaMalloc derivative matrices");
        if (npar && grad_smem_bytes(e->prec, e->nslots, e->nl, (int)e->sched.size(), npar) > e->smem_optin)
            return e->fail(PCSF_EINVAL, "parameter derivatives need more shared memory than this device has for this tree");
    }

    std::memcpy(e->hps.p, psets.data(), sizeof(PSet) * nps);
    std::memcpy(e->hreq.p, reqs.data(), sizeof(Request) * nreq);
    if (nwi) std::memcpy(e->hwi.p, wis.data(), sizeof(WorkItem) * nwi);
    std::memcpy(e->hwib.p, wib.data(), sizeof(int32_t) * (nreq + 1));
    cudaStream_t s = e->stream;
    CK(cudaMemcpyAsync(e->dps.p, e->hps.p, sizeof(PSet) * nps, cudaMemcpyHostToDevice, s), "H2D psets");
    CK(cudaMemcpyAsync(e->dreq.p, e->hreq.p, sizeof(Request) * nreq, cudaMemcpyHostToDevice, s), "H2D requests");
    if (nwi) CK(cudaMemcpyAsync(e->dwi.p, e->hwi.p, sizeof(WorkItem) * nwi, cudaMemcpyHostToDevice, s), "H2D work");
    CK(cudaMemcpyAsync(e->dwib.p, e->hwib.p, sizeof(int32_t) * (nreq + 1), cudaMemcpyHostToDevice, s), "H2D wib");
    CK(cudaMemsetAsync(e->dstatus.p, 0x7f, sizeof(int32_t) * nps, s), "memset status");

    float pf_ms = 0.f, pr_ms = 0.f;
    const int nchunks = (int)chunk_req_begin.size() - 1;
    for (int c = 0; c < nchunks; c++) {
        int r0 = chunk_req_begin[c], r1 = chunk_req_begin[c + 1];
        int p0 = chunk_ps_begin[c], p1 = chunk_ps_begin[c + 1];
        CK(cudaEventRecord(e->ev[0], s), "event");
        if (ff) {   // FP64 formation, split into hi / lo floats
            CK(launch_pform(true, e->dps.p + p0, p1 - p0, e->dbranch.p, e->nbr, dmv, e->Pbuf64.p, e->dstatus.p + p0, s),
               "P(t) formation launch");
            CK(launch_split_ff(e->Pbuf64.p, reinterpret_cast<float *>(e->Pbuf.p), (size_t)(p1 - p0) * e->nbr, s),
               "P(t) split launch");
            e->stats.kernel_launches += 1;
        } else if (stage64) {
            CK(launch_pform(true, e->dps.p + p0, p1 - p0, e->dbranch.p, e->nbr, dmv, e->Pbuf64.p, e->dstatus.p + p0, s),
               "P(t) formation launch");
            CK(launch_d2f_rows(e->Pbuf64.p, reinterpret_cast<float *>(e->Pbuf.p), (size_t)(p1 - p0) * e->nbr, e->nbr,
                               bop, e->nl, s, dlo), "P(t) conversion launch");
            e->stats.kernel_launches += 1;
        } else if (want_bop && !dyn) {
            CK(launch_pform_tc(e->dps.p + p0, p1 - p0, e->dbranch.p, e->nbr, e->nl, dmv, e->dPfB.p,
                               reinterpret_cast<float *>(e->Pbuf.p), bop, e->dstatus.p + p0, e->derr.p, s),
               "tensor-core P(t) formation launch");
        } else {
            CK(launch_pform(e->prec == PCSF_PREC_FP64 || dyn || ff, e->dps.p + p0, p1 - p0, e->dbranch.p, e->nbr, dmv,
                            e->Pbuf.p, e->dstatus.p + p0, s, false, bop, e->nl, (dyn || ff) ? nullptr : dlo),
               "P(t) formation launch");
        }
        CK(cudaEventRecord(e->ev[1], s), "event");
        PruneArgs pa{};
        pa.wi = e->dwi.p + wib[r0];
        pa.nwi = wib[r1] - wib[r0];
        pa.req = e->dreq.p;
        pa.leaves = b->dleaves.p;
        pa.Pbuf = e->Pbuf.p;
        pa.sched = e->dsched.p;
        pa.n_internal = (int)e->sched.size();
        pa.nl = e->nl;
        pa.nbr = e->nbr;
        pa.nslots = e->nslots;
        pa.m = dmv;
        pa.partials = e->dpart.p + 2 * (size_t)wib[r0];
        pa.Bop = bop;
        pa.nbop = nbop;
        pa.dither = e->prec != PCSF_PREC_FP64;
        pa.dlo = dlo;
        pa.tile = e->simt_tile;
        pa.tc_shape = e->tc_shape;
        if (grad) {
            GradArgs ga{};
            ga.wi = pa.wi;
            ga.nwi = pa.nwi;
            ga.req = pa.req;
            ga.leaves = pa.leaves;
            ga.Pbuf = pa.Pbuf;
            ga.sched = pa.sched;
            ga.n_internal = pa.n_internal;
            ga.nl = pa.nl;
            ga.nbr = pa.nbr;
            ga.nslots = pa.nslots;
            ga.m = pa.m;
            ga.Qrow = dg ? dg->Qrow : e->prec == PCSF_PREC_FP64 ? (const void *)e->dQrowd.p : (const void *)e->dQrowf.p;
            ga.npar = npar;
            ga.Umat = dg ? dg->Umat : nullptr;
            ga.Hmat = e->dHmat.p;
            if (npar)
                CK(launch_hform(e->prec == PCSF_PREC_FP64, e->dps.p + p0, p1 - p0, e->dbranch.p, e->nbr, dmv.lam, dg->Bdot,
                                e->dHmat.p, s), "derivative matrix launch");
            ga.scratch = e->gscratch.p;
            ga.scratch_per_cta = gscr;
            ga.recompute_leaves = e->grad_recompute ? 1 : 0;
            ga.partials = pa.partials;
            ga.gpart = e->dgpart.p + (size_t)wib[r0] * gstride;
            int grid = std::min(e->grad_grid, std::max(pa.nwi, 1));
            const bool tce = tc_prec(e->prec);
            CK(launch_grad(e->prec == PCSF_PREC_FP64 ? PCSF_PREC_FP64 : PCSF_PREC_FP32,
                           tce ? e->accurate_comp() : e->comp_mode(), ga, s, grid), "gradient launch");
        } else if (drho) {
            int grid = std::min(e->sm_count, std::max(pa.nwi, 1));
            CK(launch_prune_tc_dual(pa, e->dQop.p, e->dbranch.p, e->ddpart.p + 2 * (size_t)wib[r0], e->derr.p, s, grid),
               "tensor-core tangent launch");
        } else if (ff) {
            int grid = std::min(e->ff_grid, std::max(pa.nwi, 1));
            CK(launch_prune_ff(pa, s, grid), "float-float pruning launch");
        } else if (tc) {
            int grid = std::min(e->tc_grid, std::max(pa.nwi, 1));
            if (e->prec == PCSF_PREC_BF16X3)
                CK(launch_prune_bf16(pa, e->derr.p, s, grid), "BF16 tensor-core pruning launch");
            else
                CK(launch_prune_tc(e->prec == PCSF_PREC_TF32X3 ? 3 : 1, pa, e->derr.p, s, grid), "tensor-core pruning launch");
        } else {
            int grid = std::min(e->prune_grid, std::max(pa.nwi, 1));
            CK(launch_prune(e->prec == PCSF_PREC_FP64 ? PCSF_PREC_FP64 : PCSF_PREC_FP32, comp, pa, s, grid),
               "pruning launch");
        }
        CK(cudaEventRecord(e->ev[2], s), "event");
        e->stats.pform_launches += (p1 > p0);
        e->stats.prune_launches += (pa.nwi > 0);
        e->stats.kind_launches[kind] += (pa.nwi > 0);
        e->stats.kernel_launches += (p1 > p0) + (pa.nwi > 0);
        CK(cudaEventSynchronize(e->ev[2]), "pruning");
        float t1 = 0.f, t2 = 0.f;
        cudaEventElapsedTime(&t1, e->ev[0], e->ev[1]);
        cudaEventElapsedTime(&t2, e->ev[1], e->ev[2]);
        pf_ms += t1;
        pr_ms += t2;
    }
    CK(cudaEventRecord(e->ev[3], s), "event");
    CK(launch_reduce(e->dpart.p, e->dwib.p, nreq, e->dlpr.p, e->delpr.p, s), "reduce launch");
    e->stats.kernel_launches += 1;
    std::vector<double> hdrho;
    if (drho) {
        CK(launch_reduce(e->ddpart.p, e->dwib.p, nreq, e->ddrho.p, e->ddscr.p, s), "reduce launch");
        e->stats.kernel_launches += 1;
        hdrho.resize(nreq);
        CK(cudaMemcpyAsync(hdrho.data(), e->ddrho.p, sizeof(double) * nreq, cudaMemcpyDeviceToHost, s), "D2H drho");
    }
    if (grad) {
        CK(launch_reduce_grad(e->dgpart.p, e->dwib.p, nreq, gstride, e->dgrad.p, s), "gradient reduce launch");
        e->stats.kernel_launches += 1;
        CK(cudaMemcpyAsync(e->hgrad.p, e->dgrad.p, sizeof(double) * nreq * gstride, cudaMemcpyDeviceToHost, s), "D2H grad");
    }
    CK(cudaEventRecord(e->ev[4], s), "event");
    CK(cudaMemcpyAsync(e->hlpr.p, e->dlpr.p, sizeof(double) * nreq, cudaMemcpyDeviceToHost, s), "D2H lpr");
    CK(cudaMemcpyAsync(e->helpr.p, e->delpr.p, sizeof(double) * nreq, cudaMemcpyDeviceToHost, s), "D2H elpr");
    CK(cudaMemcpyAsync(e->hstatus.p, e->dstatus.p, sizeof(int32_t) * nps, cudaMemcpyDeviceToHost, s), "D2H status");
    int herr = 0;
    CK(cudaMemcpyAsync(&herr, e->derr.p, sizeof(int), cudaMemcpyDeviceToHost, s), "D2H error flag");
    CK(cudaStreamSynchronize(s), "evaluation");
    if (herr) return e->fail(PCSF_ECUDA, "a tensor-core wait timed out; results of this call are invalid");
    float rd_ms = 0.f;
    cudaEventElapsedTime(&rd_ms, e->ev[3], e->ev[4]);
    e->stats.pform_ms += pf_ms;
    e->stats.prune_ms += pr_ms;
    e->stats.kind_ms[kind] += pr_ms;
    e->stats.kind_columns[kind] += kind_cols;
    e->stats.other_ms += rd_ms;
    for (int r = 0; r < nreq; r++) {
        int key = e->hstatus.p[req_pset_global[r]];
        int st = (key >= 0 && key < 0x7f000000) ? (key & 15) : PCSF_OK;
        out[r] = Eval{e->hlpr.p[r], e->helpr.p[r], st};
    }
    if (grad) grad->assign(e->hgrad.p, e->hgrad.p + (size_t)nreq * gstride);
    if (drho) *drho = hdrho;
    return PCSF_OK;
}

// ---------------------------------------------------------------------------
// One maximize_lpr (PhyloCSFModel.ml:84-99) as a resumable state machine.

// In reduced precision the objective carries rounding noise of ~1e-7 relative,
// larger than the change of lpr over Brent's smallest probes (sqrt(eps)|x|).
// A trial point within DERIV_REL*|x| of the best point is therefore valued
// by the first-order expansion f(x) + f'(x)(u - x) with f'(x) from the
// adjoint pass (second-order remainder < 1e-8 relative); every reported value
// is still a direct evaluation.
constexpr double DERIV_REL = 1e-4;
// Central-difference derivative of the search values (deriv_mode 1): f'(x) from f(x (1 +- FD_REL)).
// The tensor-core error's bias is common to two points this close and cancels in the difference;
// what remains is its noise (~2.5e-6 sqrt(columns) nats per difference) over 2 FD_REL x, and the
// truncation (third derivative) x (FD_REL x)^2 / 6: together ~0.03 nats per unit rho at 3,000
// codons, far below the noise band of the search's comparisons, for two search evaluations
// instead of one tangent pass (about half the cost).
constexpr double FD_REL = 2e-3;
// Noise band of a tensor-core search comparison: inside it the compensated kernel decides.
// (measured: the tensor-core error of a difference of nearby points has a standard
// deviation of ~3.3e-6 nats x sqrt(columns); the band is three of those)
constexpr double AMBIGUOUS_PER_SQRT_COL = 1e-5;
// Brent's parabolic step is taken or refused by comparing the parabola's step with
// half the step before last (the GSL fminimizer's test).  That test moves with the
// differences of the three f values it interpolates, so near convergence a tensor-core
// error of a few 1e-4 nats can flip it (seen: 0.966 vs 1.054 of the threshold on a
// 2,960-codon region), and Brent then follows another path and stops at another point.
// The test is therefore repeated with every value moved by +-PARABOLA_BAND_PER_SQRT_COL
// x sqrt(columns); if the outcome can change, the step is computed from accurate values.
constexpr double PARABOLA_BAND_PER_SQRT_COL = 5e-6;

struct Fit {
    int region = 0, model = 0;
    int64_t ncols = 0;
    bool deriv = false;            // derivative-assisted small steps (reduced precision)
    bool tc_search = false;        // search values from the tensor cores: knife-edge decisions re-decided accurately
    bool accurate_final = false;   // report f(x) from the accurate values (acache), or xcache when exact
    bool exact = false;            // report f(x) from the float-float kernel (long regions)
    int prior_kind = 0;            // OmegaModel objectives add a prior on the variable (0: none)
    std::deque<std::pair<double, Eval>> acache;     // rho -> accurate evaluation (compensated FP32 kernel)
    std::deque<std::pair<double, Eval>> xcache;     // rho -> float-float evaluation (returned value of a long region)
    std::deque<std::pair<double, double>> gcache;   // rho -> d lpr / d rho
    double lo = 1e-2, hi = 10.0, init = 1.0, accuracy = 0.01;
    int maxtries = 250;
    enum Phase { FI_START, FI_LOOP, BR_SET, BR_V, BR_PROPOSE, BR_ACCEPT, FINAL, DONE } phase = FI_START;
    std::deque<std::pair<double, Eval>> cache;   // deque: element addresses survive push_back
    // find_init
    double flo = 0, fhi = 0, x = 0, fx = 0;
    int tries = 0;
    uint64_t rng = 0;
    // Brent on -lpr
    double blo = 0, bhi = 0, bflo = 0, bfhi = 0, bx = 0, bfx = 0, w = 0, fw = 0, v = 0, fv = 0, d_keep = 0, e_keep = 0;
    double u = 0;
    int iters = 0;
    // results
    int status = PCSF_OK;
    double rho = 0, lpr = 0, elpr = 0;

    const Eval *get(double r) const
    {
        for (auto &c : cache)
            if (c.first == r) return &c.second;
        return nullptr;
    }
    const Eval *geta(double r) const
    {
        for (auto &c : acache)
            if (c.first == r) return &c.second;
        return nullptr;
    }
    const Eval *getx(double r) const
    {
        for (auto &c : xcache)
            if (c.first == r) return &c.second;
        return nullptr;
    }
    const double *getg(double r) const
    {
        for (auto &c : gcache)
            if (c.first == r) return &c.second;
        return nullptr;
    }
    double band() const { return AMBIGUOUS_PER_SQRT_COL * std::sqrt((double)ncols); }
};

// One Brent proposal (the GSL fminimizer's step) from the state of f and the values
// fz = F(bx), fw = F(w), fv = F(v) of the minimised function F = -lpr.
struct Proposal {
    double u, e_keep, d_keep;
    bool tried, parabolic;
};
static Proposal brent_propose(const Fit &f, double fz, double fw, double fv)
{
    // parabolic step through (x, w, v) if acceptable, else golden section; the two
    // remembered step lengths swap slots between iterations as in the GSL
    // implementation the reference drives
    const double z = f.bx;
    double d = f.e_keep, ee = f.d_keep;
    const double tol = SQRT_DBL_EPS * std::fabs(z);
    const double mid = 0.5 * (f.blo + f.bhi);
    const double left = z - f.blo, right = f.bhi - z;
    double p = 0.0, q = 0.0, r = 0.0;
    Proposal out{};
    if (std::fabs(ee) > tol) {
        out.tried = true;
        r = (z - f.w) * (fz - fv);
        q = (z - f.v) * (fz - fw);
        p = (z - f.v) * q - (z - f.w) * r;
        q = 2.0 * (q - r);
        if (q > 0.0) p = -p;
        else q = -q;
        r = ee;
        ee = d;
    }
    if (std::fabs(p) < std::fabs(0.5 * q * r) && p < q * left && p < q * right) {
        out.parabolic = true;
        d = p / q;
        double uu = z + d;
        if ((uu - f.blo) < 2.0 * tol || (f.bhi - uu) < 2.0 * tol) d = (z < mid) ? tol : -tol;
    } else {
        ee = (z < mid) ? (f.bhi - z) : -(z - f.blo);
        d = GOLDEN * ee;
    }
    out.u = (std::fabs(d) >= tol) ? z + d : z + ((d > 0.0) ? tol : -tol);
    out.e_keep = ee;
    out.d_keep = d;
    return out;
}

// Advance until a value outside the cache is needed (appended to `need`, to
// `need_grad` for a gradient, or to `need_acc` for an accurate evaluation) or done.
static double prior_value(int kind, double x);

static void advance(Fit &f, std::vector<double> &need, std::vector<double> &need_grad, std::vector<double> &need_acc,
                    std::vector<double> &need_exact)
{
    auto ask = [&](double r) -> const Eval * {
        const Eval *ev = f.get(r);
        if (ev) return ev;
        if (f.ncols == 0) {   // empty region: the likelihood term is identically 0
            f.cache.push_back({r, Eval{prior_value(f.prior_kind, r), 0.0, PCSF_OK}});
            return &f.cache.back().second;
        }
        need.push_back(r);
        return nullptr;
    };
    auto ask_acc = [&](double r) -> const Eval * {
        const Eval *ev = f.geta(r);
        if (!ev) need_acc.push_back(r);
        return ev;
    };
    auto failed = [&](const Eval *ev) {
        if (ev->status != PCSF_OK) {
            f.status = ev->status;
            f.phase = Fit::DONE;
            return true;
        }
        return false;
    };
    // lpr(a) >= lpr(b) (a at least as good as b), given the search's values la, lb at a, b.
    // On a tensor-core search, a comparison inside the noise band is decided by the
    // accurate values of both points instead; -1: those values are needed first (asked for).
    // Points closer than DERIV_REL |a| keep the search's comparison (their difference is
    // below the accurate kernel's own rounding noise).
    auto at_least = [&](double a, double la, double b, double lb) -> int {
        if (!f.tc_search || f.ncols == 0 || a == b || std::fabs(la - lb) > f.band() ||
            std::fabs(a - b) <= DERIV_REL * std::fabs(a))
            return la >= lb;
        const Eval *ea = ask_acc(a), *eb = ask_acc(b);
        if (!ea || !eb) return -1;
        if (failed(ea) || failed(eb)) return -2;
        return ea->lpr >= eb->lpr;
    };
    for (;;) {
        switch (f.phase) {
        case Fit::FI_START: {
            const Eval *a = ask(f.lo), *b = ask(f.hi), *c = ask(f.init);
            if (!a || !b || !c) return;
            if (failed(a) || failed(b) || failed(c)) return;
            f.flo = a->lpr;
            f.fhi = b->lpr;
            f.x = f.init;
            f.fx = c->lpr;
            f.tries = 0;
            f.rng = 0;
            f.phase = Fit::FI_LOOP;
            break;
        }
        case Fit::FI_LOOP: {
            // find_init's test f(x) <= f(lo) || f(x) <= f(hi) (Fit.ml:39-45), knife edges settled accurately
            bool retry = false;
            if (f.tries < f.maxtries) {
                const int nlo = at_least(f.lo, f.flo, f.x, f.fx);
                const int nhi = at_least(f.hi, f.fhi, f.x, f.fx);
                if (nlo == -2 || nhi == -2) return;
                if (nlo < 0 || nhi < 0) return;
                retry = nlo == 1 || nhi == 1;
            }
            if (retry) {
                // speculatively request the next few restart points of the deterministic stream
                const double width = std::log(f.hi) - std::log(f.lo);
                uint64_t s = f.rng;
                double cand = std::exp(std::log(f.lo) + uniform01(s) * width);
                const Eval *ev = f.get(cand);
                if (!ev && f.ncols == 0) ev = ask(cand);
                if (!ev) {
                    uint64_t s2 = f.rng;
                    int k = 0;
                    for (int t = f.tries; t < f.maxtries && k < 16; t++, k++) {
                        double c2 = std::exp(std::log(f.lo) + uniform01(s2) * width);
                        if (!f.get(c2)) need.push_back(c2);
                    }
                    return;
                }
                if (failed(ev)) return;
                f.rng = s;
                f.x = cand;
                f.fx = ev->lpr;
                f.tries++;
                break;
            }
            if (f.tries == f.maxtries) f.x = (f.flo > f.fhi) ? f.lo : f.hi;
            if (f.lo < f.x && f.x < f.hi) f.phase = Fit::BR_SET;
            else f.phase = Fit::FINAL;
            break;
        }
        case Fit::BR_SET: {
            const Eval *a = ask(f.lo), *b = ask(f.hi), *c = ask(f.x);
            if (!a || !b || !c) return;
            if (failed(a) || failed(b) || failed(c)) return;
            f.blo = f.lo;
            f.bhi = f.hi;
            f.bflo = -a->lpr;
            f.bfhi = -b->lpr;
            f.bx = f.x;
            f.bfx = -c->lpr;
            if (!(f.bfx < f.bflo && f.bfx < f.bfhi)) {
                f.status = PCSF_EBRACKET;
                f.phase = Fit::DONE;
                return;
            }
            f.v = f.w = f.blo + GOLDEN * (f.bhi - f.blo);
            f.phase = Fit::BR_V;
            break;
        }
        case Fit::BR_V: {
            const Eval *a = ask(f.v);
            if (!a) return;
            if (failed(a)) return;
            f.fv = f.fw = -a->lpr;
            f.d_keep = f.e_keep = 0.0;
            f.iters = 0;
            f.phase = Fit::BR_PROPOSE;
            break;
        }
        case Fit::BR_PROPOSE: {
            Proposal pr = brent_propose(f, f.bfx, f.fw, f.fv);
            // Only a parabola through well-separated points is re-decided: a point reached by a
            // small step carries the first-order value f(x) + f'(x)(u - x), whose difference to
            // its neighbour is already exact to first order, while any direct evaluation of two
            // points that close (< DERIV_REL |x| apart) is dominated by rounding noise.
            const double sep = DERIV_REL * std::fabs(f.bx);
            const bool separated = std::fabs(f.bx - f.w) > sep && std::fabs(f.bx - f.v) > sep && std::fabs(f.w - f.v) > sep;
            if (f.tc_search && f.ncols > 0 && pr.tried && separated) {
                // is the parabolic test within reach of the search values' noise?
                const double h = PARABOLA_BAND_PER_SQRT_COL * std::sqrt((double)f.ncols);
                bool amb = false;
                for (int m = 0; m < 8 && !amb; m++) {
                    const Proposal pp = brent_propose(f, f.bfx + ((m & 1) ? h : -h), f.fw + ((m & 2) ? h : -h),
                                                      f.fv + ((m & 4) ? h : -h));
                    amb = pp.parabolic != pr.parabolic;
                }
                if (amb) {
                    const Eval *az = ask_acc(f.bx), *aw = ask_acc(f.w), *av = ask_acc(f.v);
                    if (!az || !aw || !av) return;
                    if (failed(az) || failed(aw) || failed(av)) return;
                    pr = brent_propose(f, -az->lpr, -aw->lpr, -av->lpr);
                }
            }
            f.u = pr.u;
            f.e_keep = pr.e_keep;
            f.d_keep = pr.d_keep;
            f.phase = Fit::BR_ACCEPT;
            break;
        }
        case Fit::BR_ACCEPT: {
            double fu;
            bool better;
            const double u = f.u;
            const bool small = f.deriv && std::fabs(u - f.bx) <= DERIV_REL * std::fabs(f.bx) && f.ncols > 0;
            if (small) {
                const Eval *bx = f.get(f.bx);
                const double *g = f.getg(f.bx);
                if (!bx || !g) {
                    need_grad.push_back(f.bx);
                    return;
                }
                if (failed(bx)) return;
                fu = -(bx->lpr + (*g) * (u - f.bx));
                better = fu <= f.bfx;
            } else {
                const Eval *a = ask(u);
                if (!a) return;
                if (failed(a)) return;
                fu = -a->lpr;
                // search values from the tensor cores: a comparison inside their noise band is
                // decided by the accurate values of both points instead (the state keeps the
                // search values, so later comparisons stay like for like)
                const int c = at_least(u, -fu, f.bx, -f.bfx);
                if (c < 0) return;
                better = c == 1;
            }
            if (better) {
                if (u < f.bx) { f.bhi = f.bx; f.bfhi = f.bfx; }
                else { f.blo = f.bx; f.bflo = f.bfx; }
                f.v = f.w; f.fv = f.fw;
                f.w = f.bx; f.fw = f.bfx;
                f.bx = u; f.bfx = fu;
            } else {
                // which remembered point u replaces: fu <= fw, else fu <= fv (knife edges
                // settled accurately, except for the first-order values of small steps)
                bool le_w = fu <= f.fw, le_v = fu <= f.fv;
                if (!small && f.w != f.bx) {
                    const int c = at_least(u, -fu, f.w, -f.fw);
                    if (c < 0) return;
                    le_w = c == 1;
                }
                if (!small && !(le_w || f.w == f.bx) && f.v != f.bx && f.v != f.w) {
                    const int c = at_least(u, -fu, f.v, -f.fv);
                    if (c < 0) return;
                    le_v = c == 1;
                }
                if (u < f.bx) { f.blo = u; f.bflo = fu; }
                else { f.bhi = u; f.bfhi = fu; }
                if (le_w || f.w == f.bx) {
                    f.v = f.w; f.fv = f.fw;
                    f.w = u; f.fw = fu;
                } else if (le_v || f.v == f.bx || f.v == f.w) {
                    f.v = u; f.fv = fu;
                }
            }
            f.iters++;
            if ((f.bhi - f.blo) / f.bx > f.accuracy && f.iters < 1000) f.phase = Fit::BR_PROPOSE;
            else {
                f.x = f.bx;
                f.phase = Fit::FINAL;
            }
            break;
        }
        case Fit::FINAL: {
            const Eval *a = nullptr;
            if (f.accurate_final && f.ncols > 0) {
                if (f.exact) {
                    a = f.getx(f.x);
                    if (!a) need_exact.push_back(f.x);
                } else {
                    a = ask_acc(f.x);
                }
                if (!a) return;
            } else {
                a = ask(f.x);
                if (!a) return;
            }
            if (failed(a)) return;
            f.rho = f.x;
            f.lpr = a->lpr;
            f.elpr = a->elpr;
            f.phase = Fit::DONE;
            return;
        }
        case Fit::DONE:
            return;
        }
    }
}

static double decibans(double x) { return 10.0 * x / std::log(10.0); }

// Does a region of ncols columns take its returned values from the float-float kernel?
static bool is_exact(const pcsf_engine *e, int64_t ncols)
{
    return e->prec != PCSF_PREC_FP64 && e->ff_grid > 0 && ncols > 0 &&
           ncols * (int64_t)std::max(e->nl - 2, 1) >= e->exact_min_units;
}

// Returned values: the float-float kernel for long regions, the engine's accurate
// kernel (compensated FP32 SIMT; FP64 on the FP64 engine) for the others.
static int evaluate_returned(pcsf_engine *e, pcsf_batch *b, const std::vector<Request> &reqs, std::vector<Eval> &out)
{
    std::vector<Request> ra, rx;
    std::vector<int> ia, ix;
    for (int r = 0; r < (int)reqs.size(); r++) {
        const int64_t nc = b->offs[reqs[r].region + 1] - b->offs[reqs[r].region];
        (is_exact(e, nc) ? rx : ra).push_back(reqs[r]);
        (is_exact(e, nc) ? ix : ia).push_back(r);
    }
    out.assign(reqs.size(), Eval{0.0, 0.0, PCSF_OK});
    std::vector<Eval> res;
    if (!ra.empty()) {
        int rc = evaluate(e, b, ra, res, nullptr, true);
        if (rc) return rc;
        for (size_t k = 0; k < ra.size(); k++) out[ia[k]] = res[k];
    }
    if (!rx.empty()) {
        int rc = evaluate(e, b, rx, res, nullptr, true, nullptr, nullptr, nullptr, true);
        if (rc) return rc;
        for (size_t k = 0; k < rx.size(); k++) out[ix[k]] = res[k];
    }
    return PCSF_OK;
}

static int run_fits(pcsf_engine *e, pcsf_batch *b, std::vector<Fit> &fits)
{
    // PCSF_TRACE_REGION=<r>: print every evaluation of region r's fits to stderr
    const char *tr = std::getenv("PCSF_TRACE_REGION");
    const int trace = tr ? std::atoi(tr) : -1;
    std::vector<Request> reqs, greqs, areqs, xreqs;
    std::vector<std::pair<int, double>> owner, gowner, aowner, xowner;
    // central differences: (fit, rho, index in reqs of the request at rho (1 - FD_REL); the one at
    // rho (1 + FD_REL) follows it)
    struct FdPart { int fit; double rho; int k; };
    std::vector<FdPart> fdown;
    const bool fd = e->deriv_mode == 1 && tc_prec(e->prec);
    std::vector<Eval> res, gres, ares, xres;
    std::vector<double> grad, drho;
    for (;;) {
        reqs.clear();
        owner.clear();
        greqs.clear();
        gowner.clear();
        areqs.clear();
        aowner.clear();
        xreqs.clear();
        xowner.clear();
        fdown.clear();
        std::vector<double> need, needg, needa, needx;     // reused across fits (no allocation per fit)
        for (int i = 0; i < (int)fits.size(); i++) {
            need.clear();
            needg.clear();
            needa.clear();
            needx.clear();
            advance(fits[i], need, needg, needa, needx);
            for (auto *lst : {&need, &needg, &needa, &needx}) {
                std::sort(lst->begin(), lst->end());
                lst->erase(std::unique(lst->begin(), lst->end()), lst->end());
            }
            bool bad = false;
            for (double r : need) bad |= !(r > 0.0) || !std::isfinite(r);
            for (double r : needg) bad |= !(r > 0.0) || !std::isfinite(r);
            for (double r : needa) bad |= !(r > 0.0) || !std::isfinite(r);
            for (double r : needx) bad |= !(r > 0.0) || !std::isfinite(r);
            if (bad) {
                fits[i].status = PCSF_EINVAL;
                fits[i].phase = Fit::DONE;
                continue;
            }
            for (double r : need) {
                Request q{};
                q.region = fits[i].region;
                q.model = fits[i].model;
                q.rho = r;
                reqs.push_back(q);
                owner.push_back({i, r});
            }
            for (double r : needg) {
                Request q{};
                q.region = fits[i].region;
                q.model = fits[i].model;
                q.rho = r;
                if (fd) {
                    // two search evaluations beside the point (and the point itself if not yet known)
                    if (!fits[i].get(r)) {
                        reqs.push_back(q);
                        owner.push_back({i, r});
                    }
                    fdown.push_back({i, r, (int)reqs.size()});
                    for (double sgn : {-1.0, 1.0}) {
                        Request d = q;
                        d.rho = r * (1.0 + sgn * FD_REL);
                        reqs.push_back(d);
                        owner.push_back({i, d.rho});
                    }
                    continue;
                }
                greqs.push_back(q);
                gowner.push_back({i, r});
            }
            for (double r : needa) {
                Request q{};
                q.region = fits[i].region;
                q.model = fits[i].model;
                q.rho = r;
                areqs.push_back(q);
                aowner.push_back({i, r});
            }
            for (double r : needx) {
                Request q{};
                q.region = fits[i].region;
                q.model = fits[i].model;
                q.rho = r;
                xreqs.push_back(q);
                xowner.push_back({i, r});
            }
        }
        if (reqs.empty() && greqs.empty() && areqs.empty() && xreqs.empty()) break;
        e->stats.rounds += 1;
        if (!reqs.empty()) {
            int rc = evaluate(e, b, reqs, res);
            if (rc) return rc;
        }
        const bool tangent = e->dual_ok && (e->prec == PCSF_PREC_TF32X3 || e->prec == PCSF_PREC_TF32);
        if (!greqs.empty()) {
            int rc = tangent ? evaluate(e, b, greqs, gres, nullptr, false, nullptr, &drho)
                             : evaluate(e, b, greqs, gres, &grad);
            if (rc) return rc;
        }
        if (!areqs.empty()) {
            int rc = evaluate(e, b, areqs, ares, nullptr, true);
            if (rc) return rc;
        }
        if (!xreqs.empty()) {
            int rc = evaluate(e, b, xreqs, xres, nullptr, true, nullptr, nullptr, nullptr, true);
            if (rc) return rc;
        }
        for (int pass = 0; pass < 2; pass++) {
            const auto &rq = pass ? xreqs : areqs;
            const auto &ow = pass ? xowner : aowner;
            const auto &rs = pass ? xres : ares;
            for (size_t k = 0; k < rq.size(); k++) {
                Fit &f = fits[ow[k].first];
                (pass ? f.xcache : f.acache).push_back({ow[k].second, rs[k]});
                if (f.region == trace)
                    std::fprintf(stderr, "trace region %d model %d round %lld accurate%s rho %.17g lpr %.17g | phase %d\n",
                                 f.region, f.model, (long long)e->stats.rounds, pass ? " (float-float)" : "",
                                 ow[k].second, rs[k].lpr, (int)f.phase);
            }
        }
        for (size_t k = 0; k < reqs.size(); k++) {
            Fit &f = fits[owner[k].first];
            f.cache.push_back({owner[k].second, res[k]});
            if (f.region == trace)
                std::fprintf(stderr, "trace region %d model %d round %lld rho %.17g lpr %.17g status %d | phase %d bx %.17g [%.17g %.17g]\n",
                             f.region, f.model, (long long)e->stats.rounds, owner[k].second, res[k].lpr, res[k].status,
                             (int)f.phase, f.bx, f.blo, f.bhi);
        }
        for (const FdPart &d : fdown) {
            Fit &f = fits[d.fit];
            const Eval &m = res[d.k], &p = res[d.k + 1];
            if (m.status != PCSF_OK || p.status != PCSF_OK) {
                f.status = m.status != PCSF_OK ? m.status : p.status;
                f.phase = Fit::DONE;
                continue;
            }
            const double dr = (p.lpr - m.lpr) / (reqs[d.k + 1].rho - reqs[d.k].rho);
            f.gcache.push_back({d.rho, dr});
            if (f.region == trace)
                std::fprintf(stderr, "trace region %d model %d round %lld central difference at rho %.17g dlpr/drho %.17g\n",
                             f.region, f.model, (long long)e->stats.rounds, d.rho, dr);
        }
        for (size_t k = 0; k < greqs.size(); k++) {
            Fit &f = fits[gowner[k].first];
            const double r = gowner[k].second;
            double dr = 0.0;
            if (tangent) dr = drho[k];
            else
                for (int c = 0; c < e->nbr; c++) dr += e->branch[c] * grad[k * e->nbr + c];
            f.gcache.push_back({r, dr});
            if (!f.get(r)) f.cache.push_back({r, gres[k]});
            if (f.region == trace)
                std::fprintf(stderr, "trace region %d model %d round %lld grad at rho %.17g lpr %.17g dlpr/drho %.17g\n",
                             f.region, f.model, (long long)e->stats.rounds, r, gres[k].lpr, dr);
        }
    }
    return PCSF_OK;
}

static int score_impl(pcsf_engine *e, pcsf_batch *b, int strategy, pcsf_result *out)
{
    if (strategy != PCSF_FIXED && strategy != PCSF_MLE) return e->fail(PCSF_EINVAL, "strategy %d", strategy);
    const int nreg = b->nreg;
    std::vector<Fit> fits(2 * (size_t)nreg);
    for (int r = 0; r < nreg; r++)
        for (int m = 0; m < 2; m++) {
            Fit &f = fits[2 * r + m];
            f.region = r;
            f.model = m;
            f.ncols = b->offs[r + 1] - b->offs[r];
            f.deriv = e->prec != PCSF_PREC_FP64;
            f.tc_search = tc_prec(e->prec);
            f.exact = is_exact(e, f.ncols);
            f.accurate_final = f.tc_search || f.exact;
            if (strategy == PCSF_FIXED) {
                // llr_FixedLik 1.0: a single evaluation at rho = 1
                f.x = 1.0;
                f.phase = Fit::FINAL;
            }
        }
    int rc = run_fits(e, b, fits);
    if (rc) return rc;
    for (int r = 0; r < nreg; r++) {
        const Fit &c = fits[2 * r], &nf = fits[2 * r + 1];
        pcsf_result &o = out[r];
        std::memset(&o, 0, sizeof o);
        o.status = c.status != PCSF_OK ? c.status : nf.status;
        o.rho_c = c.rho;
        o.rho_n = nf.rho;
        o.lpr_c = c.lpr;
        o.lpr_n = nf.lpr;
        o.elpr_c = c.elpr;
        o.elpr_n = nf.elpr;
        o.score = decibans(c.lpr - nf.lpr);
        o.anc_comp_score = decibans(c.elpr - nf.elpr);
        o.evals = (int32_t)(c.cache.size() + nf.cache.size() + c.gcache.size() + nf.gcache.size() + c.acache.size() +
                            nf.acache.size() + c.xcache.size() + nf.xcache.size());
    }
    return PCSF_OK;
}

// ---------------------------------------------------------------------------
// Outside-pass products: expected branch counts and node posteriors
// (PhyloLik.ml:96-174, PhyloEM.ml:14-20), one FP64 or FP32 P set per region.

static int outside_impl(pcsf_engine *e, pcsf_batch *b, int model, const double *rho, double *counts, int n_sel,
                        const int32_t *nodes, double *post, double *lpr, int32_t *status)
{
    const int nreg = b->nreg;
    const bool fp64 = e->prec == PCSF_PREC_FP64;
    const size_t es = fp64 ? 8 : 4;
    const int comp = e->accurate_comp();
    const int TC = outside_tile_cols();
    std::vector<int32_t> sel;
    if (n_sel > 0) {
        sel.assign(e->n, -1);
        for (int k = 0; k < n_sel; k++) {
            if (nodes[k] < 0 || nodes[k] >= e->n) return e->fail(PCSF_EINVAL, "node %d is not in the tree", nodes[k]);
            sel[nodes[k]] = k;   // a node listed twice is written to its last row
        }
    }
    const size_t smem = outside_smem_bytes(fp64, e->nslots, e->nl, (int)e->sched.size());
    if (smem > e->smem_optin) return e->fail(PCSF_EINVAL, "this tree needs %zu B of shared memory for the outside pass", smem);
    const size_t scr = outside_scratch_per_cta(fp64, e->nl);
    const size_t pset_bytes = (size_t)e->nbr * K2 * es;
    const size_t cnt_bytes = counts ? (size_t)e->nbr * K2 * sizeof(double) : 0;
    // regions per launch: P sets and counts of a chunk within ~2 GiB
    const int chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)std::max(nreg, 1),
                                                                (size_t(2) << 30) / (pset_bytes + cnt_bytes)));
    const int grid = std::max(1, std::min(e->sm_count, chunk));
    DevBuf<unsigned char> dP, dscr;
    DevBuf<double> dcnt, dlpr, dpost;
    DevBuf<PSet> dps;
    DevBuf<Request> dreq;
    DevBuf<WorkItem> dwi;
    DevBuf<int32_t> dwib, dstatus, dsel;
    CK(dP.reserve((size_t)chunk * pset_bytes), "cudaMalloc P(t)");
    CK(dscr.reserve((size_t)grid * scr), "cudaMalloc outside-pass scratch");
    if (counts) CK(dcnt.reserve((size_t)chunk * e->nbr * K2), "cudaMalloc counts");
    CK(dlpr.reserve(chunk), "cudaMalloc");
    CK(dps.reserve(chunk), "cudaMalloc");
    CK(dreq.reserve(chunk), "cudaMalloc");
    CK(dwib.reserve(chunk + 1), "cudaMalloc");
    CK(dstatus.reserve(chunk), "cudaMalloc");
    cudaStream_t s = e->stream;
    if (n_sel > 0) {
        CK(dsel.reserve(e->n), "cudaMalloc");
        CK(dpost.reserve((size_t)n_sel * std::max<int64_t>(b->total_cols, 1) * K), "cudaMalloc posteriors");
        CK(cudaMemcpyAsync(dsel.p, sel.data(), sizeof(int32_t) * e->n, cudaMemcpyHostToDevice, s), "H2D");
    }
    for (int r0 = 0; r0 < nreg; r0 += chunk) {
        const int r1 = std::min(nreg, r0 + chunk), nr = r1 - r0;
        std::vector<PSet> ps(nr);
        std::vector<Request> rq(nr);
        std::vector<WorkItem> wis;
        std::vector<int32_t> wib(nr + 1);
        for (int r = 0; r < nr; r++) {
            const int reg = r0 + r;
            if (!(rho[reg] > 0.0) || !std::isfinite(rho[reg])) return e->fail(PCSF_EINVAL, "rho[%d] = %g", reg, rho[reg]);
            ps[r] = PSet{model, 0, rho[reg]};
            rq[r] = Request{reg, model, r, (uint32_t)b->offs[reg], rho[reg]};
            wib[r] = (int)wis.size();
            for (int64_t c = b->offs[reg]; c < b->offs[reg + 1]; c += TC)
                wis.push_back(WorkItem{r, (int32_t)std::min<int64_t>(TC, b->offs[reg + 1] - c), c});
        }
        wib[nr] = (int)wis.size();
        CK(dwi.reserve(std::max<size_t>(wis.size(), 1)), "cudaMalloc");
        CK(cudaMemcpyAsync(dps.p, ps.data(), sizeof(PSet) * nr, cudaMemcpyHostToDevice, s), "H2D");
        CK(cudaMemcpyAsync(dreq.p, rq.data(), sizeof(Request) * nr, cudaMemcpyHostToDevice, s), "H2D");
        if (!wis.empty()) CK(cudaMemcpyAsync(dwi.p, wis.data(), sizeof(WorkItem) * wis.size(), cudaMemcpyHostToDevice, s), "H2D");
        CK(cudaMemcpyAsync(dwib.p, wib.data(), sizeof(int32_t) * (nr + 1), cudaMemcpyHostToDevice, s), "H2D");
        CK(cudaMemsetAsync(dstatus.p, 0x7f, sizeof(int32_t) * nr, s), "memset");
        if (counts) CK(cudaMemsetAsync(dcnt.p, 0, sizeof(double) * (size_t)nr * e->nbr * K2, s), "memset");
        CK(launch_pform(fp64, dps.p, nr, e->dbranch.p, e->nbr, e->dm, dP.p, dstatus.p, s), "P(t) formation launch");
        OutsideArgs oa{};
        oa.wi = dwi.p;
        oa.wi_begin = dwib.p;
        oa.nreq = nr;
        oa.req = dreq.p;
        oa.leaves = b->dleaves.p;
        oa.Pbuf = dP.p;
        oa.sched = e->dsched.p;
        oa.n_internal = (int)e->sched.size();
        oa.nl = e->nl;
        oa.nbr = e->nbr;
        oa.nslots = e->nslots;
        oa.m = e->dm;
        oa.scratch = dscr.p;
        oa.scratch_per_cta = scr;
        oa.lpr = dlpr.p;
        oa.counts = counts ? dcnt.p : nullptr;
        oa.sel = n_sel > 0 ? dsel.p : nullptr;
        oa.post = dpost.p;
        oa.total_cols = b->total_cols;
        CK(launch_outside(fp64, comp, oa, s, std::min(grid, nr)), "outside-pass launch");
        e->stats.kernel_launches += 2;
        std::vector<int32_t> keys(nr);
        std::vector<double> hl(nr);
        CK(cudaMemcpyAsync(keys.data(), dstatus.p, sizeof(int32_t) * nr, cudaMemcpyDeviceToHost, s), "D2H");
        CK(cudaMemcpyAsync(hl.data(), dlpr.p, sizeof(double) * nr, cudaMemcpyDeviceToHost, s), "D2H");
        if (counts)
            CK(cudaMemcpyAsync(counts + (size_t)r0 * e->nbr * K2, dcnt.p, sizeof(double) * (size_t)nr * e->nbr * K2,
                               cudaMemcpyDeviceToHost, s), "D2H counts");
        CK(cudaStreamSynchronize(s), "outside pass");
        for (int r = 0; r < nr; r++) {
            if (lpr) lpr[r0 + r] = hl[r];
            if (status) status[r0 + r] = (keys[r] >= 0 && keys[r] < 0x7f000000) ? (keys[r] & 15) : PCSF_OK;
        }
    }
    if (n_sel > 0 && b->total_cols > 0)
        CK(cudaMemcpy(post, dpost.p, sizeof(double) * (size_t)n_sel * b->total_cols * K, cudaMemcpyDeviceToHost),
           "D2H posteriors");
    return PCSF_OK;
}

// PhyloEM.ell (PhyloEM.ml:22-73) of counts [nbr][K][K] at tree scale rho: the branches'
// sum of counts x log P (positive counts only) with P(t) formed in FP64, plus the root
// prior term from the row sums of the root's left child's counts.
static int ell_impl(pcsf_engine *e, int model, double rho, const double *counts, double *ell)
{
    DevBuf<double> dP;
    DevBuf<PSet> dps;
    DevBuf<int32_t> dst;
    CK(dP.reserve((size_t)e->nbr * K2), "cudaMalloc");
    CK(dps.reserve(1), "cudaMalloc");
    CK(dst.reserve(1), "cudaMalloc");
    PSet ps{model, 0, rho};
    CK(cudaMemcpyAsync(dps.p, &ps, sizeof ps, cudaMemcpyHostToDevice, e->stream), "H2D");
    CK(cudaMemsetAsync(dst.p, 0x7f, sizeof(int32_t), e->stream), "memset");
    CK(launch_pform(true, dps.p, 1, e->dbranch.p, e->nbr, e->dm, dP.p, dst.p, e->stream), "P(t) launch");
    e->stats.kernel_launches += 1;
    std::vector<double> Et((size_t)e->nbr * K2);
    int32_t key = STATUS_NONE;
    CK(cudaMemcpyAsync(Et.data(), dP.p, sizeof(double) * Et.size(), cudaMemcpyDeviceToHost, e->stream), "D2H");
    CK(cudaMemcpyAsync(&key, dst.p, sizeof(int32_t), cudaMemcpyDeviceToHost, e->stream), "D2H");
    CK(cudaStreamSynchronize(e->stream), "P(t)");
    if (key >= 0 && key < 0x7f000000) return e->fail(key & 15, "P(t) formation failed at tree scale %g", rho);
    double tot = 0.0;
    for (int i = 0; i < e->nbr; i++)
        for (int a = 0; a < K; a++)
            for (int c = 0; c < K; c++) {
                const double x = counts[((size_t)i * K + a) * K + c];
                if (x > 0.0) tot += x * std::log(Et[(size_t)i * K2 + (size_t)c * K + a] + (a == c ? 1.0 : 0.0));
            }
    const double *cl = counts + (size_t)e->lch[e->n - 1] * K2;
    for (int a = 0; a < K; a++) {
        double r = 0.0;
        for (int c = 0; c < K; c++) r += cl[a * K + c];
        if (r > 0.0) tot += r * std::log(e->prior[model][a]);
    }
    *ell = tot;
    return PCSF_OK;
}

// ---------------------------------------------------------------------------
// Read-only view of an engine's device state for pcsf_lpr_noalloc (noalloc.cu).

int pcsf_internal_noalloc_ctx(pcsf_engine *e, NoallocCtx *c)
{
    if (!e || !c) return PCSF_EINVAL;
    if (!e->derr.p || !e->dsched.p || !e->dbranch.p) return e->fail(PCSF_EINVAL, "engine is not initialised");
    c->device = e->device;
    c->stream = e->stream;
    c->prec = e->prec;
    const bool tcprec = tc_prec(e->prec);
    // pcsf_lpr's returned values: the SIMT kernel with the accurate summation on
    // tensor-core engines, the engine's own summation otherwise
    c->comp = tcprec ? e->accurate_comp() : e->comp_mode();
    c->pt64 = e->pt64;
    c->tc_direct = e->tc_direct;
    c->has_models = e->has_models;
    c->nl = e->nl;
    c->nbr = e->nbr;
    c->n_internal = (int)e->sched.size();
    c->nslots = e->nslots;
    c->branch = e->dbranch.p;
    c->sched = e->dsched.p;
    c->m = e->dm;
    c->prune_grid = e->prune_grid;
    c->simt_tile = e->simt_tile;
    c->ff_grid = e->prec != PCSF_PREC_FP64 ? e->ff_grid : 0;
    c->exact_min_units = e->exact_min_units;
    c->derr = e->derr.p;
    return PCSF_OK;
}

int pcsf_internal_fail(pcsf_engine *e, int code, const char *msg) { return e->fail(code, "%s", msg); }


// ---------------------------------------------------------------------------
// OmegaModel (src/OmegaModel.ml): parametric codon Q, priors, and the H0/H1
// maximum-a-posteriori fits of rho and kappa.

typedef std::array<double, 12> OmegaKey;   // kappa, omega, sigma, F3x4 (A, C, G relative to T) x 3 positions

// pi_exprs (OmegaModel.ml:21-40) and the rate matrix q_p14n / q_scale (:42-80).
static void omega_q(const OmegaKey &q, double *Q, double *pi)
{
    static const char *aa = "KNKNTTTTRSRSIIMIQHQHPPPPRRRRLLLLEDEDAAAAGGGGVVVV*Y*YSSSS*CWCLFLF";
    auto nuc = [](int i, int pos) { return pos == 0 ? i / 16 : pos == 1 ? (i / 4) % 4 : i % 4; };
    auto sc = [&](int i) {
        double out = 1.0;
        for (int pos = 0; pos < 3; pos++) {
            const int n = nuc(i, pos), base = 3 + 3 * pos;
            const double num = (n == 3) ? 1.0 : q[base + n];
            const double den = q[base] + (q[base + 1] + (q[base + 2] + 1.0));
            out *= num / den;
        }
        return out;
    };
    const double denom = 1.0 - (1.0 - q[2]) * (sc(48) + (sc(50) + sc(56)));
    for (int i = 0; i < K; i++) pi[i] = sc(i) / denom;
    auto is_stop = [](int i) { return i == 48 || i == 50 || i == 56; };
    for (int i = 0; i < K; i++) {
        double tot = 0.0;
        for (int j = 0; j < K; j++) {
            double v = 0.0;
            if (i != j) {
                int nd = 0, a = 0, b = 0;
                for (int pos = 0; pos < 3; pos++)
                    if (nuc(i, pos) != nuc(j, pos)) { nd++; a = nuc(i, pos); b = nuc(j, pos); }
                if (nd == 1) {
                    const bool transition = (a + b == 2 && a != 1 && b != 1) || (a + b == 4 && a != 2 && b != 2);
                    const double kp = transition ? q[0] : 1.0;
                    const double op = (!is_stop(i) && !is_stop(j) && aa[i] != aa[j]) ? q[1] : 1.0;
                    v = pi[j] * (kp * op);
                }
            }
            Q[i * K + j] = v;
            if (i != j) tot = v + tot;
        }
        Q[i * K + i] = 0.0 - tot;
    }
    double scale = 0.0;
    for (int i = 0; i < K; i++) scale = scale - pi[i] * Q[i * K + i];
    for (int i = 0; i < K2; i++) Q[i] = Q[i] / scale;
}

// dQ/dx of the scaled OmegaModel rate matrix for x = kappa (0) or omega (1): with
// R the unscaled matrix (R_ij = pi_j kappa^[transition] omega^[nonsynonymous]) and
// s = -sum_i pi_i R_ii, Q = R / s and dQ/dx = R'/s - R s'/s^2 (pi does not depend on
// kappa or omega).
static void omega_dq(const OmegaKey &q, int x, double *dQ)
{
    std::vector<double> Q(K2), pi(K), R(K2), dR(K2);
    omega_q(q, Q.data(), pi.data());
    static const char *aa = "KNKNTTTTRSRSIIMIQHQHPPPPRRRRLLLLEDEDAAAAGGGGVVVV*Y*YSSSS*CWCLFLF";
    auto nuc = [](int i, int pos) { return pos == 0 ? i / 16 : pos == 1 ? (i / 4) % 4 : i % 4; };
    auto is_stop = [](int i) { return i == 48 || i == 50 || i == 56; };
    for (int i = 0; i < K; i++) {
        double tot = 0.0, dtot = 0.0;
        for (int j = 0; j < K; j++) {
            double v = 0.0, dv = 0.0;
            if (i != j) {
                int nd = 0, a = 0, bb = 0;
                for (int pos = 0; pos < 3; pos++)
                    if (nuc(i, pos) != nuc(j, pos)) { nd++; a = nuc(i, pos); bb = nuc(j, pos); }
                if (nd == 1) {
                    const bool transition = (a + bb == 2 && a != 1 && bb != 1) || (a + bb == 4 && a != 2 && bb != 2);
                    const bool nonsyn = !is_stop(i) && !is_stop(j) && aa[i] != aa[j];
                    v = pi[j] * ((transition ? q[0] : 1.0) * (nonsyn ? q[1] : 1.0));
                    if (x == 0 && transition) dv = v / q[0];
                    if (x == 1 && nonsyn) dv = v / q[1];
                }
            }
            R[i * K + j] = v;
            dR[i * K + j] = dv;
            tot += v;
            dtot += dv;
        }
        R[i * K + i] = -tot;
        dR[i * K + i] = -dtot;
    }
    double sc = 0.0, dsc = 0.0;
    for (int i = 0; i < K; i++) {
        sc -= pi[i] * R[i * K + i];
        dsc -= pi[i] * dR[i * K + i];
    }
    for (int i = 0; i < K2; i++) dQ[i] = dR[i] / sc - R[i] * dsc / (sc * sc);
}

// half_cauchy_lpdf ~mode:1 ~scale:0.5 (OmegaModel.ml:148-156) and the Gamma(7, 0.25)
// density of kappa - 1 (OmegaModel.ml:157; GSL gamma_pdf with shape a, scale b).
static double prior_value(int kind, double x)
{
    if (kind == 1) {
        const double PI = std::acos(-1.0), mode = 1.0, scale = 0.5;
        const double numer = 1.0 / (PI * scale * (1.0 + std::pow((x - mode) / scale, 2.0)));
        const double cdf = std::atan((0.0 - mode) / scale) / PI + 0.5;
        return std::log(numer) - std::log(1.0 - cdf);
    }
    if (kind == 2) {
        const double y = x - 1.0 + 2.220446049250313e-16, a = 7.0, b = 0.25;
        if (!(y > 0.0)) return -INFINITY;
        return (a - 1.0) * std::log(y) - y / b - std::lgamma(a) - a * std::log(b);
    }
    return 0.0;
}

// Eigensystems of per-request models, cached by parameter vector, and the
// device table of the models a round needs.
struct DynModels {
    std::map<OmegaKey, int> index;                  // key -> cache slot
    std::vector<std::vector<double>> U, lam, eq;    // host cache
    DevBuf<double> dU, dlam, dsq, disq, dwrow, dprior, dwlog;
    DevBuf<int16_t> dwlist;
    DevBuf<float> dUf;
    DevModels dm{};
    DevBuf<unsigned char> dQrow, dBdot;             // parameter derivatives (dyn_derivs)
};

static int dyn_prepare(pcsf_engine *e, DynModels &dmod, const std::vector<OmegaKey> &keys, std::vector<int> &slot)
{
    // eigendecompose the models not seen before, in one batched launch
    std::vector<int> fresh;
    slot.resize(keys.size());
    for (size_t i = 0; i < keys.size(); i++) {
        auto it = dmod.index.find(keys[i]);
        if (it == dmod.index.end()) {
            int id = (int)dmod.U.size();
            dmod.index[keys[i]] = id;
            dmod.U.emplace_back(K2);
            dmod.lam.emplace_back(K);
            dmod.eq.emplace_back(K);
            fresh.push_back((int)i);
            slot[i] = id;
        } else {
            slot[i] = it->second;
        }
    }
    if (!fresh.empty()) {
        const int nf = (int)fresh.size();
        std::vector<double> A((size_t)nf * K2), Q(K2), pi(K);
        for (int f = 0; f < nf; f++) {
            omega_q(keys[fresh[f]], Q.data(), pi.data());
            std::vector<double> &eqv = dmod.eq[slot[fresh[f]]];
            for (int i = 0; i < K; i++) eqv[i] = pi[i];
            for (int i = 0; i < K; i++)
                for (int j = 0; j < K; j++) {
                    const double aij = std::sqrt(pi[i]) * Q[i * K + j] / std::sqrt(pi[j]);
                    const double aji = std::sqrt(pi[j]) * Q[j * K + i] / std::sqrt(pi[i]);
                    A[(size_t)f * K2 + i * K + j] = 0.5 * (aij + aji);
                }
        }
        DevBuf<double> dA, dUo, dlo;
        DevBuf<int> dst;
        CK(dA.reserve((size_t)nf * K2), "cudaMalloc");
        CK(dUo.reserve((size_t)nf * K2), "cudaMalloc");
        CK(dlo.reserve((size_t)nf * K), "cudaMalloc");
        CK(dst.reserve(nf), "cudaMalloc");
        CK(cudaMemcpyAsync(dA.p, A.data(), sizeof(double) * nf * K2, cudaMemcpyHostToDevice, e->stream), "H2D");
        CK(launch_jacobi(dA.p, dUo.p, dlo.p, dst.p, nf, e->stream), "eigensolver launch");
        e->stats.kernel_launches += 1;
        std::vector<double> Uh((size_t)nf * K2), lh((size_t)nf * K);
        std::vector<int> sth(nf);
        CK(cudaMemcpyAsync(Uh.data(), dUo.p, sizeof(double) * nf * K2, cudaMemcpyDeviceToHost, e->stream), "D2H");
        CK(cudaMemcpyAsync(lh.data(), dlo.p, sizeof(double) * nf * K, cudaMemcpyDeviceToHost, e->stream), "D2H");
        CK(cudaMemcpyAsync(sth.data(), dst.p, sizeof(int) * nf, cudaMemcpyDeviceToHost, e->stream), "D2H");
        CK(cudaStreamSynchronize(e->stream), "eigensolver");
        for (int f = 0; f < nf; f++) {
            if (sth[f]) return e->fail(PCSF_EEIG, "eigensolver did not converge for an OmegaModel rate matrix");
            std::copy(Uh.begin() + (size_t)f * K2, Uh.begin() + (size_t)(f + 1) * K2, dmod.U[slot[fresh[f]]].begin());
            std::copy(lh.begin() + (size_t)f * K, lh.begin() + (size_t)(f + 1) * K, dmod.lam[slot[fresh[f]]].begin());
        }
    }
    // device table for this round: model m of the round = keys[m]
    const int M = (int)keys.size();
    std::vector<double> U((size_t)M * K2), lam((size_t)M * K), sq((size_t)M * K), isq((size_t)M * K),
        wrow((size_t)M * K), prior((size_t)M * K), wlog((size_t)M * K);
    std::vector<float> Uf((size_t)M * K2);
    std::vector<int16_t> wlist((size_t)M * WLIST);
    for (int m = 0; m < M; m++) {
        const int id = slot[m];
        const std::vector<double> &eqv = dmod.eq[id];
        double tot = 0.0;
        for (int i = 0; i < K; i++) tot += eqv[i];
        for (int i = 0; i < K; i++) {
            sq[(size_t)m * K + i] = std::sqrt(eqv[i]);
            isq[(size_t)m * K + i] = 1.0 / std::sqrt(eqv[i]);
            prior[(size_t)m * K + i] = eqv[i] / tot;     // the equilibrium, normalised (PhyloModel.ml:25-29)
            wlog[(size_t)m * K + i] = prior[(size_t)m * K + i] * std::log(prior[(size_t)m * K + i]);
            lam[(size_t)m * K + i] = dmod.lam[id][i];
        }
        for (int i = 0; i < K2; i++) {
            U[(size_t)m * K2 + i] = dmod.U[id][i];
            Uf[(size_t)m * K2 + i] = (float)dmod.U[id][i];
        }
        const double nrm = std::sqrt(tot);
        for (int mm = 0; mm < K; mm++) {
            double w = 0.0;
            for (int j = 0; j < K; j++) w += dmod.U[id][j * K + mm] * sq[(size_t)m * K + j];
            wrow[(size_t)m * K + mm] = (std::fabs(w) > 1e-9 * nrm) ? w : 0.0;
        }
        make_wlist(&wrow[(size_t)m * K], &wlist[(size_t)m * WLIST]);
    }
    CK(dmod.dwlist.reserve((size_t)M * WLIST), "cudaMalloc");
    CK(cudaMemcpyAsync(dmod.dwlist.p, wlist.data(), sizeof(int16_t) * M * WLIST, cudaMemcpyHostToDevice, e->stream),
       "H2D");
    CK(dmod.dU.reserve((size_t)M * K2), "cudaMalloc");
    CK(dmod.dUf.reserve((size_t)M * K2), "cudaMalloc");
    for (auto *bp : {&dmod.dlam, &dmod.dsq, &dmod.disq, &dmod.dwrow, &dmod.dprior, &dmod.dwlog})
        CK(bp->reserve((size_t)M * K), "cudaMalloc");
    CK(cudaMemcpyAsync(dmod.dU.p, U.data(), sizeof(double) * M * K2, cudaMemcpyHostToDevice, e->stream), "H2D");
    CK(cudaMemcpyAsync(dmod.dUf.p, Uf.data(), sizeof(float) * M * K2, cudaMemcpyHostToDevice, e->stream), "H2D");
    CK(cudaMemcpyAsync(dmod.dlam.p, lam.data(), sizeof(double) * M * K, cudaMemcpyHostToDevice, e->stream), "H2D");
    CK(cudaMemcpyAsync(dmod.dsq.p, sq.data(), sizeof(double) * M * K, cudaMemcpyHostToDevice, e->stream), "H2D");
    CK(cudaMemcpyAsync(dmod.disq.p, isq.data(), sizeof(double) * M * K, cudaMemcpyHostToDevice, e->stream), "H2D");
    CK(cudaMemcpyAsync(dmod.dwrow.p, wrow.data(), sizeof(double) * M * K, cudaMemcpyHostToDevice, e->stream), "H2D");
    CK(cudaMemcpyAsync(dmod.dprior.p, prior.data(), sizeof(double) * M * K, cudaMemcpyHostToDevice, e->stream), "H2D");
    CK(cudaMemcpyAsync(dmod.dwlog.p, wlog.data(), sizeof(double) * M * K, cudaMemcpyHostToDevice, e->stream), "H2D");
    CK(cudaStreamSynchronize(e->stream), "model upload");
    dmod.dm = DevModels{};
    dmod.dm.U = dmod.dU.p;
    dmod.dm.Uf = dmod.dUf.p;
    dmod.dm.lam = dmod.dlam.p;
    dmod.dm.sq = dmod.dsq.p;
    dmod.dm.isq = dmod.disq.p;
    dmod.dm.wrow = dmod.dwrow.p;
    dmod.dm.wlist = dmod.dwlist.p;
    dmod.dm.prior = dmod.dprior.p;
    dmod.dm.wlog = dmod.dwlog.p;
    dmod.dm.tol = e->tol;
    dmod.dm.grid_n = 0;
    return PCSF_OK;
}

// For the round's models (as laid out by dyn_prepare): Q row-major and
// Bdot_x = U^T D^1/2 (dQ/dx) D^-1/2 U for x = kappa, omega, in the engine's
// arithmetic type, on the device; dg points at them and at the round's U.
static int dyn_derivs(pcsf_engine *e, DynModels &dmod, const std::vector<OmegaKey> &keys, const std::vector<int> &slot,
                      DynGrad &dg)
{
    const int M = (int)keys.size();
    const bool fp64 = e->prec == PCSF_PREC_FP64;
    std::vector<double> Qall((size_t)M * K2), Ball((size_t)M * 2 * K2);
    auto work = [&](int m0, int m1) {
        std::vector<double> Q(K2), pi(K), dQ(K2), A(K2), T1(K2);
        for (int m = m0; m < m1; m++) {
            omega_q(keys[m], Q.data(), pi.data());
            std::copy(Q.begin(), Q.end(), Qall.begin() + (size_t)m * K2);
            const std::vector<double> &U = dmod.U[slot[m]];
            const std::vector<double> &eq = dmod.eq[slot[m]];
            for (int x = 0; x < 2; x++) {
                omega_dq(keys[m], x, dQ.data());
                for (int i = 0; i < K; i++)
                    for (int j = 0; j < K; j++) A[i * K + j] = std::sqrt(eq[i]) * dQ[i * K + j] / std::sqrt(eq[j]);
                // T1 = A U, Bdot = U^T T1
                for (int i = 0; i < K; i++)
                    for (int j = 0; j < K; j++) {
                        double acc = 0.0;
                        for (int k = 0; k < K; k++) acc += A[i * K + k] * U[k * K + j];
                        T1[i * K + j] = acc;
                    }
                double *Bd = &Ball[((size_t)m * 2 + x) * K2];
                for (int i = 0; i < K; i++)
                    for (int j = 0; j < K; j++) {
                        double acc = 0.0;
                        for (int k = 0; k < K; k++) acc += U[k * K + i] * T1[k * K + j];
                        Bd[i * K + j] = acc;
                    }
            }
        }
    };
    const int nth = std::max(1, std::min<int>(16, (int)std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (int t = 0; t < nth; t++) th.emplace_back(work, (int)((int64_t)M * t / nth), (int)((int64_t)M * (t + 1) / nth));
    for (auto &t : th) t.join();
    const size_t es = fp64 ? 8 : 4;
    CK(dmod.dQrow.reserve((size_t)M * K2 * es), "cudaMalloc");
    CK(dmod.dBdot.reserve((size_t)M * 2 * K2 * es), "cudaMalloc");
    if (fp64) {
        CK(cudaMemcpyAsync(dmod.dQrow.p, Qall.data(), sizeof(double) * Qall.size(), cudaMemcpyHostToDevice, e->stream), "H2D");
        CK(cudaMemcpyAsync(dmod.dBdot.p, Ball.data(), sizeof(double) * Ball.size(), cudaMemcpyHostToDevice, e->stream), "H2D");
        CK(cudaStreamSynchronize(e->stream), "derivative upload");
    } else {
        std::vector<float> qf(Qall.begin(), Qall.end()), bf(Ball.begin(), Ball.end());
        CK(cudaMemcpyAsync(dmod.dQrow.p, qf.data(), sizeof(float) * qf.size(), cudaMemcpyHostToDevice, e->stream), "H2D");
        CK(cudaMemcpyAsync(dmod.dBdot.p, bf.data(), sizeof(float) * bf.size(), cudaMemcpyHostToDevice, e->stream), "H2D");
        CK(cudaStreamSynchronize(e->stream), "derivative upload");
    }
    dg.Qrow = dmod.dQrow.p;
    dg.Bdot = dmod.dBdot.p;
    dg.Umat = fp64 ? (const void *)dmod.dm.U : (const void *)dmod.dm.Uf;
    return PCSF_OK;
}

struct OmegaRegion {
    int region = 0;
    int64_t ncols = 0;
    int hyp = 0, round = 0, stage = 0;   // stage 0: rho, 1: kappa
    OmegaKey q{};
    double rho = 1.0, lpr_last = 0.0;
    double lpr_h0 = 0.0, rho_h0 = 0.0, kappa_h0 = 0.0;
    bool done = false;
    int status = PCSF_OK, evals = 0;
    Fit fit;

    void start_fit()
    {
        fit = Fit{};
        fit.region = region;
        fit.ncols = ncols;
        fit.accuracy = 0.01;
        if (stage == 0) {           // kr_map: rho in [0.001, 10] from the current rho
            fit.lo = 0.001;
            fit.hi = 10.0;
            fit.init = rho;
            fit.prior_kind = 1;
        } else {                    // kappa in [1, 10] from the current kappa
            fit.lo = 1.0;
            fit.hi = 10.0;
            fit.init = q[0];
            fit.prior_kind = 2;
        }
    }
};

// update_f3x4 (OmegaModel.ml:102-134): per region and codon position, nucleotide
// counts over the leaves (pseudocount 1), relative to T
static int region_f3x4(pcsf_engine *e, pcsf_batch *b, std::vector<std::array<double, 9>> &out)
{
    out.assign(b->nreg, {});
    std::vector<uint8_t> lv((size_t)b->total_cols * e->nl);
    if (!lv.empty()) CK(cudaMemcpy(lv.data(), b->dleaves.p, lv.size(), cudaMemcpyDeviceToHost), "D2H leaves");
    for (int r = 0; r < b->nreg; r++) {
        double counts[3][4];
        for (auto &row : counts)
            for (double &c : row) c = 1.0;
        for (size_t i = (size_t)b->offs[r] * e->nl; i < (size_t)b->offs[r + 1] * e->nl; i++) {
            const int c = lv[i];
            if (c >= K) continue;
            counts[0][c / 16] += 1.0;
            counts[1][(c / 4) % 4] += 1.0;
            counts[2][c % 4] += 1.0;
        }
        for (int pos = 0; pos < 3; pos++)
            for (int n = 0; n < 3; n++) out[r][3 * pos + n] = counts[pos][n] / counts[pos][3];
    }
    return PCSF_OK;
}

static int omega_impl(pcsf_engine *e, pcsf_batch *b, double omega_h1, double sigma_h1, pcsf_omega_result *out)
{
    const int nreg = b->nreg;
    std::vector<OmegaRegion> regs(nreg);
    for (int r = 0; r < nreg; r++) {
        OmegaRegion &R = regs[r];
        R.region = r;
        R.ncols = b->offs[r + 1] - b->offs[r];
        // new_instance ~kappa:2.5 (omega = sigma = 1), then update_f3x4 from the leaves (OmegaModel.ml:95-134)
        R.q[0] = 2.5;
        R.q[1] = 1.0;
        R.q[2] = 1.0;
        R.start_fit();
    }
    {
        std::vector<std::array<double, 9>> f;
        int rc = region_f3x4(e, b, f);
        if (rc) return rc;
        for (int r = 0; r < nreg; r++)
            for (int k = 0; k < 9; k++) regs[r].q[3 + k] = f[r][k];
    }
    DynModels dmod;
    std::vector<Request> reqs;
    std::vector<std::pair<int, double>> owner;
    std::vector<OmegaKey> keys;
    std::map<OmegaKey, int> kidx;
    std::vector<int> slot;
    std::vector<Eval> res;
    for (;;) {
        reqs.clear();
        owner.clear();
        keys.clear();
        kidx.clear();
        for (int r = 0; r < nreg; r++) {
            OmegaRegion &R = regs[r];
            while (!R.done) {
                std::vector<double> need, needg, needa, needx;
                advance(R.fit, need, needg, needa, needx);
                if (R.fit.phase != Fit::DONE) {
                    std::sort(need.begin(), need.end());
                    need.erase(std::unique(need.begin(), need.end()), need.end());
                    for (double x : need) {
                        if (!(x > 0.0) || !std::isfinite(x)) {
                            R.status = PCSF_EINVAL;
                            R.done = true;
                            break;
                        }
                        OmegaKey key = R.q;
                        double rho = R.rho;
                        if (R.stage == 0) rho = x;
                        else key[0] = x;
                        auto it = kidx.find(key);
                        int m;
                        if (it == kidx.end()) {
                            m = (int)keys.size();
                            kidx[key] = m;
                            keys.push_back(key);
                        } else {
                            m = it->second;
                        }
                        Request q{};
                        q.region = r;
                        q.model = m;
                        q.rho = rho;
                        reqs.push_back(q);
                        owner.push_back({r, x});
                    }
                    break;
                }
                // a fit finished: move along kr_map (OmegaModel.ml:171-190) and score (:195-219)
                R.evals += (int)R.fit.cache.size();
                if (R.fit.status != PCSF_OK) {
                    R.status = R.fit.status;
                    R.done = true;
                    break;
                }
                if (R.stage == 0) {
                    R.rho = R.fit.rho;
                    R.stage = 1;
                } else {
                    R.q[0] = R.fit.rho;
                    R.lpr_last = R.fit.lpr;
                    R.stage = 0;
                    R.round++;
                }
                if (R.round == 3) {
                    if (R.hyp == 0) {
                        R.lpr_h0 = R.lpr_last;
                        R.rho_h0 = R.rho;
                        R.kappa_h0 = R.q[0];
                        R.hyp = 1;
                        R.round = 0;
                        R.q[1] = omega_h1;
                        R.q[2] = sigma_h1;
                    } else {
                        R.done = true;
                        break;
                    }
                }
                R.start_fit();
            }
        }
        if (reqs.empty()) break;
        e->stats.rounds += 1;
        int rc = dyn_prepare(e, dmod, keys, slot);
        if (rc) return rc;
        rc = evaluate(e, b, reqs, res, nullptr, true, &dmod.dm);
        if (rc) return rc;
        for (size_t k = 0; k < reqs.size(); k++) {
            OmegaRegion &R = regs[owner[k].first];
            Eval ev = res[k];
            ev.lpr = prior_value(R.fit.prior_kind, owner[k].second) + ev.lpr;
            R.fit.cache.push_back({owner[k].second, ev});
        }
    }
    for (int r = 0; r < nreg; r++) {
        const OmegaRegion &R = regs[r];
        pcsf_omega_result &o = out[r];
        std::memset(&o, 0, sizeof o);
        o.status = R.status;
        o.lpr_h0 = R.lpr_h0;
        o.lpr_h1 = R.lpr_last;
        o.rho_h0 = R.rho_h0;
        o.kappa_h0 = R.kappa_h0;
        o.rho_h1 = R.rho;
        o.kappa_h1 = R.q[0];
        o.score = 10.0 * (R.lpr_last - R.lpr_h0) / std::log(10.0);
        o.evals = R.evals;
    }
    return PCSF_OK;
}

// ---------------------------------------------------------------------------
// C-ABI

extern "C" {

int pcsf_engine_create(const pcsf_tree *tree, const double *S_c, const double *pi_c, const double *S_n,
                       const double *pi_n, int32_t flags, pcsf_engine **out)
{
    if (!out) {
        g_static_error = "pcsf_engine_create: out is NULL";
        return PCSF_EINVAL;
    }
    *out = nullptr;
    if (!S_c || !pi_c || !S_n || !pi_n) {
        g_static_error = "pcsf_engine_create: null model pointer";
        return PCSF_EINVAL;
    }
    double Q[2][K2];
    const double *S[2] = {S_c, S_n}, *pi[2] = {pi_c, pi_n};
    for (int m = 0; m < 2; m++) {
        if (assemble_q(S[m], pi[m], Q[m]) != PCSF_OK) {
            g_static_error = "CamlPaml.P14n.instantiate_q: Q scale evaluated to a non-positive value";
            return PCSF_ESCALE;
        }
    }
    const double *Qp[2] = {Q[0], Q[1]};
    return pcsf_engine_create_q(tree, Qp[0], pi_c, pi_c, Qp[1], pi_n, pi_n, flags, out);
}

int pcsf_engine_create_q(const pcsf_tree *tree, const double *Q_c, const double *eq_c, const double *prior_c,
                         const double *Q_n, const double *eq_n, const double *prior_n, int32_t flags,
                         pcsf_engine **out)
{
    if (!out) {
        g_static_error = "pcsf_engine_create_q: out is NULL";
        return PCSF_EINVAL;
    }
    *out = nullptr;
    if (!Q_c || !eq_c || !prior_c || !Q_n || !eq_n || !prior_n) {
        g_static_error = "pcsf_engine_create_q: null model pointer";
        return PCSF_EINVAL;
    }
    pcsf_engine *e = new (std::nothrow) pcsf_engine();
    if (!e) {
        g_static_error = "out of host memory";
        return PCSF_ENOMEM;
    }
    int rc = engine_init_common(e, tree, flags);
    if (rc == PCSF_OK) {
        const double *Q[2] = {Q_c, Q_n}, *eq[2] = {eq_c, eq_n}, *pr[2] = {prior_c, prior_n};
        rc = setup_models(e, Q, eq, pr);
    }
    if (rc != PCSF_OK) {
        g_static_error = e->err;
        delete e;
        return rc;
    }
    *out = e;
    return PCSF_OK;
}

int pcsf_engine_create_tree(const pcsf_tree *tree, int32_t flags, pcsf_engine **out)
{
    if (!out) {
        g_static_error = "pcsf_engine_create_tree: out is NULL";
        return PCSF_EINVAL;
    }
    *out = nullptr;
    pcsf_engine *e = new (std::nothrow) pcsf_engine();
    if (!e) {
        g_static_error = "out of host memory";
        return PCSF_ENOMEM;
    }
    int rc = engine_init_common(e, tree, flags);
    if (rc != PCSF_OK) {
        g_static_error = e->err;
        delete e;
        return rc;
    }
    *out = e;
    return PCSF_OK;
}

int pcsf_omega_score(pcsf_engine *e, pcsf_batch *b, double omega_h1, double sigma_h1, pcsf_omega_result *out)
{
    if (!e) return PCSF_EINVAL;
    CK(cudaSetDevice(e->device), "cudaSetDevice");
    if (!b || b->e != e) return e->fail(PCSF_EINVAL, "pcsf_omega_score: batch does not belong to this engine");
    if (b->nreg > 0 && !out) return e->fail(PCSF_EINVAL, "pcsf_omega_score: out is NULL");
    if (!(omega_h1 >= 0.0) || !(sigma_h1 >= 0.0))
        return e->fail(PCSF_EINVAL, "CamlPaml.P14n.instantiate_q: domain violation (omega_H1, sigma_H1 must be >= 0)");
    return omega_impl(e, b, omega_h1, sigma_h1, out);
}

int pcsf_omega_grad(pcsf_engine *e, pcsf_batch *b, const double *kappa, const double *omega, double sigma,
                    const double *rho, double *lpr, double *d_branch, double *d_rho, double *d_kappa, double *d_omega,
                    int32_t *status)
{
    if (!e) return PCSF_EINVAL;
    CK(cudaSetDevice(e->device), "cudaSetDevice");
    if (!b || b->e != e) return e->fail(PCSF_EINVAL, "pcsf_omega_grad: batch does not belong to this engine");
    const int nreg = b->nreg;
    if (nreg > 0 && (!kappa || !omega || !rho || !lpr)) return e->fail(PCSF_EINVAL, "pcsf_omega_grad: null argument");
    if (!(sigma >= 0.0)) return e->fail(PCSF_EINVAL, "CamlPaml.P14n.instantiate_q: domain violation (sigma must be >= 0)");
    if (nreg == 0) return PCSF_OK;
    std::vector<std::array<double, 9>> f;
    int rc = region_f3x4(e, b, f);
    if (rc) return rc;
    std::vector<OmegaKey> keys(nreg);
    std::vector<Request> reqs(nreg);
    for (int r = 0; r < nreg; r++) {
        if (!(kappa[r] > 0.0) || !(omega[r] > 0.0) || !(rho[r] > 0.0) || !std::isfinite(rho[r]))
            return e->fail(PCSF_EINVAL, "pcsf_omega_grad: region %d: kappa, omega and rho must be > 0", r);
        keys[r][0] = kappa[r];
        keys[r][1] = omega[r];
        keys[r][2] = sigma;
        for (int k = 0; k < 9; k++) keys[r][3 + k] = f[r][k];
        reqs[r] = Request{r, r, 0, 0, rho[r]};     // request r uses the round's model r
    }
    DynModels dmod;
    std::vector<int> slot;
    rc = dyn_prepare(e, dmod, keys, slot);
    if (rc) return rc;
    DynGrad dg{};
    rc = dyn_derivs(e, dmod, keys, slot, dg);
    if (rc) return rc;
    std::vector<Eval> res;
    std::vector<double> g;
    rc = evaluate(e, b, reqs, res, &g, false, &dmod.dm, nullptr, &dg);
    if (rc) return rc;
    const int gs = e->nbr + 2;
    for (int r = 0; r < nreg; r++) {
        lpr[r] = res[r].lpr;
        if (status) status[r] = res[r].status;
        double dr = 0.0;
        for (int c = 0; c < e->nbr; c++) {
            const double gc = g[(size_t)r * gs + c];
            if (d_branch) d_branch[(size_t)r * e->nbr + c] = gc;
            dr += e->branch[c] * gc;
        }
        if (d_rho) d_rho[r] = dr;
        if (d_kappa) d_kappa[r] = g[(size_t)r * gs + e->nbr];
        if (d_omega) d_omega[r] = g[(size_t)r * gs + e->nbr + 1];
    }
    return PCSF_OK;
}

void pcsf_engine_destroy(pcsf_engine *e)
{
    if (e) cudaSetDevice(e->device);
    delete e;
}

const char *pcsf_last_error(const pcsf_engine *e) { return e ? e->err.c_str() : g_static_error.c_str(); }

int pcsf_engine_get_stats(const pcsf_engine *e, pcsf_stats *out)
{
    if (!e || !out) return PCSF_EINVAL;
    *out = e->stats;
    out->prune_grid = e->prune_grid;
    out->tc_grid = e->tc_grid;
    out->tc_shape = (e->prec == PCSF_PREC_TF32X3 || e->prec == PCSF_PREC_TF32) ? e->tc_shape : -1;
    out->simt_tile = simt_tile_cols(e->prec, e->nslots, e->simt_tile);
    return PCSF_OK;
}

int pcsf_engine_autotune(pcsf_engine *e, pcsf_batch *b, int32_t *tile)
{
    if (!e) return PCSF_EINVAL;
    if (!e->has_models) return e->fail(PCSF_EINVAL, "this engine has no coding / noncoding models");
    CK(cudaSetDevice(e->device), "cudaSetDevice");
    if (!b || b->e != e) return e->fail(PCSF_EINVAL, "pcsf_engine_autotune: batch does not belong to this engine");
    if (e->prec == PCSF_PREC_FP64 || b->nreg == 0) {
        if (tile) *tile = simt_tile_cols(e->prec, e->nslots, e->simt_tile);
        return PCSF_OK;
    }
    // up to 256 regions at evenly spaced length quantiles, both models at rho = 1
    std::vector<int> order(b->nreg);
    for (int r = 0; r < b->nreg; r++) order[r] = r;
    std::stable_sort(order.begin(), order.end(),
                     [&](int x, int y) { return b->offs[x + 1] - b->offs[x] < b->offs[y + 1] - b->offs[y]; });
    const int ns = std::min(b->nreg, 256);
    std::vector<Request> reqs;
    for (int k = 0; k < ns; k++) {
        const int r = order[(size_t)k * (b->nreg - 1) / std::max(ns - 1, 1)];
        for (int m = 0; m < 2; m++) reqs.push_back(Request{r, m, 0, 0, 1.0});
    }
    const int saved_tile = e->simt_tile, saved_grid = e->prune_grid;
    const int64_t saved_exact = e->exact_min_units;
    const pcsf_stats saved_stats = e->stats;
    e->exact_min_units = INT64_MAX;   // time the FP32 kernel on every sampled region
    int best = 0;
    double best_ms = 1e300;
    int rc = PCSF_OK;
    for (int cand : {64, 32}) {
        if (prune_smem_bytes(e->prec, e->nslots, e->nl, (int)e->sched.size(), cand) > e->smem_optin) continue;
        e->simt_tile = cand;
        e->prune_grid = simt_grid(e, cand);
        double ms = 0.0;
        std::vector<Eval> res;
        for (int it = 0; it < 3 && rc == PCSF_OK; it++) {
            const double before = e->stats.kind_ms[0];
            rc = evaluate(e, b, reqs, res, nullptr, true);
            if (it > 0) ms += e->stats.kind_ms[0] - before;
        }
        if (rc != PCSF_OK) break;
        if (ms < best_ms) {
            best_ms = ms;
            best = cand;
        }
    }
    e->exact_min_units = saved_exact;
    e->stats = saved_stats;
    if (rc != PCSF_OK || best == 0) {
        e->simt_tile = saved_tile;
        e->prune_grid = saved_grid;
        return rc != PCSF_OK ? rc : e->fail(PCSF_EINVAL, "pcsf_engine_autotune: no tile fits this tree");
    }
    e->simt_tile = best;
    e->prune_grid = simt_grid(e, best);
    if (tile) *tile = best;
    // the TF32 search kernel's shape (the values do not depend on it), timed on the same
    // sample's search evaluations
    if (e->prec == PCSF_PREC_TF32X3 || e->prec == PCSF_PREC_TF32) {
        const int saved_shape = e->tc_shape, saved_tc_grid = e->tc_grid;
        const pcsf_stats keep = e->stats;
        int best_s = -1;
        double best_s_ms = 1e300;
        for (int cand = 0; cand < PCSF_TC_SHAPES; cand++) {
            e->tc_shape = cand;
            e->tc_grid = e->sm_count * prune_tc_ctas_per_sm(e->nslots, e->nl, (int)e->sched.size(), cand);
            double ms = 0.0;
            std::vector<Eval> res;
            for (int it = 0; it < 3 && rc == PCSF_OK; it++) {
                const double before = e->stats.kind_ms[1];
                rc = evaluate(e, b, reqs, res, nullptr, false);
                if (it > 0) ms += e->stats.kind_ms[1] - before;
            }
            if (rc != PCSF_OK) break;
            e->tc_shape_ms[cand] = ms / 2.0;
            if (ms < best_s_ms) {
                best_s_ms = ms;
                best_s = cand;
            }
        }
        e->stats = keep;
        if (rc != PCSF_OK || best_s < 0) {
            e->tc_shape = saved_shape;
            e->tc_grid = saved_tc_grid;
            return rc != PCSF_OK ? rc : e->fail(PCSF_EINVAL, "pcsf_engine_autotune: no tensor-core shape fits");
        }
        e->tc_shape = best_s;
        e->tc_grid = e->sm_count * prune_tc_ctas_per_sm(e->nslots, e->nl, (int)e->sched.size(), best_s);
    }
    return PCSF_OK;
}

int pcsf_engine_set_tc_shape(pcsf_engine *e, int32_t shape)
{
    if (!e) return PCSF_EINVAL;
    if (!(e->prec == PCSF_PREC_TF32X3 || e->prec == PCSF_PREC_TF32))
        return e->fail(PCSF_EINVAL, "pcsf_engine_set_tc_shape: this engine has no TF32 tensor-core search kernel");
    if (!prune_tc_shape_ok(shape))
        return e->fail(PCSF_EINVAL, "pcsf_engine_set_tc_shape: shape must be 0..%d", PCSF_TC_SHAPES - 1);
    CK(cudaSetDevice(e->device), "cudaSetDevice");
    e->tc_shape = shape;
    e->tc_grid = e->sm_count * prune_tc_ctas_per_sm(e->nslots, e->nl, (int)e->sched.size(), shape);
    return PCSF_OK;
}

int pcsf_engine_tc_shape_times(const pcsf_engine *e, double *ms, int32_t n)
{
    if (!e || !ms || n < 0) return PCSF_EINVAL;
    for (int i = 0; i < n && i < PCSF_TC_SHAPES; i++) ms[i] = e->tc_shape_ms[i];
    return PCSF_OK;
}

int pcsf_engine_set_derivative_mode(pcsf_engine *e, int32_t mode)
{
    if (!e) return PCSF_EINVAL;
    if (mode != 0 && mode != 1) return e->fail(PCSF_EINVAL, "pcsf_engine_set_derivative_mode: mode must be 0 or 1");
    e->deriv_mode = mode;
    return PCSF_OK;
}

int pcsf_engine_set_grad_recompute(pcsf_engine *e, int32_t on)
{
    if (!e) return PCSF_EINVAL;
    e->grad_recompute = on != 0;
    return PCSF_OK;
}

int64_t pcsf_engine_grad_scratch_bytes(const pcsf_engine *e, int32_t n_rate_params)
{
    if (!e || (n_rate_params != 0 && n_rate_params != 2)) return -1;
    return (int64_t)grad_scratch_per_cta(e->prec == PCSF_PREC_FP64 ? PCSF_PREC_FP64 : PCSF_PREC_FP32, e->nl,
                                         n_rate_params, e->grad_recompute);
}

int pcsf_engine_set_exact_threshold(pcsf_engine *e, int64_t units)
{
    if (!e) return PCSF_EINVAL;
    if (units < 0) return e->fail(PCSF_EINVAL, "pcsf_engine_set_exact_threshold: units must be >= 0");
    e->exact_min_units = units;
    return PCSF_OK;
}

int pcsf_engine_exact_available(const pcsf_engine *e) { return e && e->ff_grid > 0 ? 1 : 0; }

int pcsf_engine_reset_stats(pcsf_engine *e)
{
    if (!e) return PCSF_EINVAL;
    e->stats = pcsf_stats{};
    return PCSF_OK;
}

int pcsf_engine_stream(const pcsf_engine *e, void **stream)
{
    if (!e || !stream) return PCSF_EINVAL;
    *stream = (void *)e->stream;
    return PCSF_OK;
}

int pcsf_engine_eigensystem(const pcsf_engine *e, int32_t model, double *U, double *lambda)
{
    if (!e || model < 0 || model > 1 || !U || !lambda) return PCSF_EINVAL;
    std::memcpy(U, e->U[model], sizeof(double) * K2);
    std::memcpy(lambda, e->lam[model], sizeof(double) * K);
    return PCSF_OK;
}

int pcsf_engine_pt(pcsf_engine *e, int32_t model, int32_t n_t, const double *t, double *P, int32_t *status)
{
    if (!e) return PCSF_EINVAL;
    if (!e->has_models) return e->fail(PCSF_EINVAL, "this engine has no coding / noncoding models");
    CK(cudaSetDevice(e->device), "cudaSetDevice");
    if (model < 0 || model > 1 || n_t <= 0 || !t || !P || !status) return e->fail(PCSF_EINVAL, "pcsf_engine_pt: bad argument");
    for (int i = 0; i < n_t; i++)
        if (!(t[i] >= 0.0) || !std::isfinite(t[i])) return e->fail(PCSF_EINVAL, "pcsf_engine_pt: t[%d] = %g", i, t[i]);
    const bool fp64 = e->prec == PCSF_PREC_FP64;
    const size_t es = fp64 ? 8 : 4;
    DevBuf<double> dt;
    DevBuf<unsigned char> dP;
    DevBuf<PSet> dps;
    DevBuf<int32_t> dst;
    CK(dt.reserve(n_t), "cudaMalloc");
    CK(dP.reserve((size_t)n_t * K2 * es), "cudaMalloc");
    CK(dps.reserve(1), "cudaMalloc");
    CK(dst.reserve(1), "cudaMalloc");
    PSet ps{model, 0, 1.0};
    CK(cudaMemcpyAsync(dt.p, t, sizeof(double) * n_t, cudaMemcpyHostToDevice, e->stream), "H2D");
    CK(cudaMemcpyAsync(dps.p, &ps, sizeof ps, cudaMemcpyHostToDevice, e->stream), "H2D");
    std::vector<int32_t> keys(n_t, STATUS_NONE);
    // one launch per matrix so that each gets its own status key
    std::vector<unsigned char> raw((size_t)n_t * K2 * es);
    for (int i = 0; i < n_t; i++) {
        CK(cudaMemsetAsync(dst.p, 0x7f, sizeof(int32_t), e->stream), "memset");
        CK(launch_pform(fp64, dps.p, 1, dt.p + i, 1, e->dm, dP.p + (size_t)i * K2 * es, dst.p, e->stream), "P(t) launch");
        e->stats.kernel_launches += 1;
        CK(cudaMemcpyAsync(&keys[i], dst.p, sizeof(int32_t), cudaMemcpyDeviceToHost, e->stream), "D2H");
    }
    CK(cudaMemcpyAsync(raw.data(), dP.p, raw.size(), cudaMemcpyDeviceToHost, e->stream), "D2H P");
    CK(cudaStreamSynchronize(e->stream), "P(t)");
    for (int i = 0; i < n_t; i++) {
        status[i] = (keys[i] >= 0 && keys[i] < 0x7f000000) ? (keys[i] & 15) : PCSF_OK;
        for (int r = 0; r < K; r++)
            for (int c = 0; c < K; c++) {
                size_t src = (size_t)i * K2 + (size_t)c * K + r;   // stored as E^T
                double ev = fp64 ? reinterpret_cast<double *>(raw.data())[src] : reinterpret_cast<float *>(raw.data())[src];
                P[(size_t)i * K2 + r * K + c] = ev + (r == c ? 1.0 : 0.0);
            }
    }
    return PCSF_OK;
}

int pcsf_engine_pt_search(pcsf_engine *e, int32_t model, int32_t n_t, const double *t, double *P, int32_t *status)
{
    if (!e) return PCSF_EINVAL;
    if (!e->has_models) return e->fail(PCSF_EINVAL, "this engine has no coding / noncoding models");
    CK(cudaSetDevice(e->device), "cudaSetDevice");
    if (!(e->prec == PCSF_PREC_TF32X3 || e->prec == PCSF_PREC_TF32) || !e->dPfB.p)
        return e->fail(PCSF_EINVAL, "pcsf_engine_pt_search: this engine forms no tensor-core P(t)");
    if (model < 0 || model > 1 || n_t <= 0 || n_t > 320 || !t || !P)
        return e->fail(PCSF_EINVAL, "pcsf_engine_pt_search: bad argument (1 <= n_t <= 320)");
    for (int i = 0; i < n_t; i++)
        if (!(t[i] >= 0.0) || !std::isfinite(t[i])) return e->fail(PCSF_EINVAL, "pcsf_engine_pt_search: t[%d] = %g", i, t[i]);
    DevBuf<double> dt;
    DevBuf<float> dP;
    DevBuf<PSet> dps;
    DevBuf<int32_t> dst;
    CK(dt.reserve(n_t), "cudaMalloc");
    CK(dP.reserve((size_t)n_t * K2), "cudaMalloc");
    CK(dps.reserve(1), "cudaMalloc");
    CK(dst.reserve(1), "cudaMalloc");
    PSet ps{model, 0, 1.0};
    CK(cudaMemcpyAsync(dt.p, t, sizeof(double) * n_t, cudaMemcpyHostToDevice, e->stream), "H2D");
    CK(cudaMemcpyAsync(dps.p, &ps, sizeof ps, cudaMemcpyHostToDevice, e->stream), "H2D");
    CK(cudaMemsetAsync(dst.p, 0x7f, sizeof(int32_t), e->stream), "memset");
    CK(cudaMemsetAsync(e->derr.p, 0, sizeof(int), e->stream), "memset");
    // every matrix written as E^T (all "branches" above leaves): t plays the branch lengths at rho = 1
    CK(launch_pform_tc(dps.p, 1, dt.p, n_t, n_t, e->dm, e->dPfB.p, dP.p, nullptr, dst.p, e->derr.p, e->stream),
       "tensor-core P(t) launch");
    e->stats.kernel_launches += 1;
    std::vector<float> raw((size_t)n_t * K2);
    int32_t key = STATUS_NONE;
    int herr = 0;
    CK(cudaMemcpyAsync(raw.data(), dP.p, sizeof(float) * raw.size(), cudaMemcpyDeviceToHost, e->stream), "D2H");
    CK(cudaMemcpyAsync(&key, dst.p, sizeof(int32_t), cudaMemcpyDeviceToHost, e->stream), "D2H");
    CK(cudaMemcpyAsync(&herr, e->derr.p, sizeof(int), cudaMemcpyDeviceToHost, e->stream), "D2H");
    CK(cudaStreamSynchronize(e->stream), "P(t)");
    if (herr) return e->fail(PCSF_ECUDA, "pcsf_engine_pt_search: a tensor-core wait timed out");
    const int st = (key >= 0 && key < 0x7f000000) ? (key & 15) : PCSF_OK;
    for (int i = 0; i < n_t; i++) {
        if (status) status[i] = st;
        for (int r = 0; r < K; r++)
            for (int c = 0; c < K; c++)
                P[(size_t)i * K2 + r * K + c] = (double)raw[(size_t)i * K2 + (size_t)c * K + r] + (r == c ? 1.0 : 0.0);
    }
    return PCSF_OK;
}

int pcsf_batch_create(pcsf_engine *e, int32_t n_regions, const int64_t *col_offsets, const uint8_t *leaves,
                      pcsf_batch **out)
{
    if (!e) return PCSF_EINVAL;
    CK(cudaSetDevice(e->device), "cudaSetDevice");
    if (!out) return e->fail(PCSF_EINVAL, "pcsf_batch_create: out is NULL");
    *out = nullptr;
    if (n_regions < 0 || (n_regions > 0 && !col_offsets)) return e->fail(PCSF_EINVAL, "pcsf_batch_create: bad regions");
    pcsf_batch *b = new (std::nothrow) pcsf_batch();
    if (!b) return e->fail(PCSF_ENOMEM, "out of host memory");
    b->e = e;
    b->device = e->device;
    b->nreg = n_regions;
    b->offs.assign(n_regions + 1, 0);
    if (n_regions > 0) {
        if (col_offsets[0] != 0) {
            delete b;
            return e->fail(PCSF_EINVAL, "pcsf_batch_create: col_offsets[0] must be 0");
        }
        for (int r = 0; r <= n_regions; r++) {
            b->offs[r] = col_offsets[r];
            if (r > 0 && col_offsets[r] < col_offsets[r - 1]) {
                delete b;
                return e->fail(PCSF_EINVAL, "pcsf_batch_create: col_offsets not non-decreasing at %d", r);
            }
        }
    }
    b->total_cols = b->offs[n_regions];
    if (b->total_cols > 0 && !leaves) {
        delete b;
        return e->fail(PCSF_EINVAL, "pcsf_batch_create: leaves is NULL");
    }
    const size_t nbytes = (size_t)b->total_cols * e->nl;
    // the codes are checked on the device after the upload (a host loop over a
    // multi-GB batch would cost more than scoring it)
    unsigned long long bad = ~0ull;
    cudaError_t ce = b->dleaves.reserve(nbytes + 16);
    if (ce == cudaSuccess) ce = e->dbadcode.reserve(1);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(e->dbadcode.p, &bad, sizeof(bad), cudaMemcpyHostToDevice, e->stream);
    if (ce == cudaSuccess && nbytes)
        ce = cudaMemcpyAsync(b->dleaves.p, leaves, nbytes, cudaMemcpyHostToDevice, e->stream);
    if (ce == cudaSuccess) ce = launch_check_codes(b->dleaves.p, nbytes, e->dbadcode.p, e->stream);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(&bad, e->dbadcode.p, sizeof(bad), cudaMemcpyDeviceToHost, e->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->stream);
    if (ce != cudaSuccess) {
        delete b;
        return e->cuda_fail(ce, "batch upload");
    }
    if (bad != ~0ull) {
        const size_t col = (size_t)(bad / (unsigned long long)e->nl);
        const int lf = (int)(bad % (unsigned long long)e->nl);
        const int code = leaves[bad];
        delete b;
        return e->fail(PCSF_EINVAL, "pcsf_batch_create: leaf code %d at column %zu leaf %d (max %d)", code, col, lf,
                       PCSF_MARGINALIZE);
    }
    *out = b;
    return PCSF_OK;
}

void pcsf_batch_destroy(pcsf_batch *b)
{
    // the engine may already be destroyed: only the batch's own fields are read
    if (b) cudaSetDevice(b->device);
    delete b;
}

int pcsf_score(pcsf_engine *e, pcsf_batch *b, int32_t strategy, pcsf_result *out)
{
    if (!e) return PCSF_EINVAL;
    if (!e->has_models) return e->fail(PCSF_EINVAL, "this engine has no coding / noncoding models");
    CK(cudaSetDevice(e->device), "cudaSetDevice");
    if (!b || b->e != e) return e->fail(PCSF_EINVAL, "pcsf_score: batch does not belong to this engine");
    if (b->nreg > 0 && !out) return e->fail(PCSF_EINVAL, "pcsf_score: out is NULL");
    return score_impl(e, b, strategy, out);
}

int pcsf_score_batch(pcsf_engine *e, int32_t n_regions, const int64_t *col_offsets, const uint8_t *leaves,
                     int32_t strategy, pcsf_result *out)
{
    pcsf_batch *b = nullptr;
    int rc = pcsf_batch_create(e, n_regions, col_offsets, leaves, &b);
    if (rc) return rc;
    rc = pcsf_score(e, b, strategy, out);
    pcsf_batch_destroy(b);
    return rc;
}

int pcsf_lpr(pcsf_engine *e, pcsf_batch *b, int32_t model, const double *rho, double *lpr, double *elpr,
             int32_t *status)
{
    if (!e) return PCSF_EINVAL;
    if (!e->has_models) return e->fail(PCSF_EINVAL, "this engine has no coding / noncoding models");
    CK(cudaSetDevice(e->device), "cudaSetDevice");
    if (!b || b->e != e) return e->fail(PCSF_EINVAL, "pcsf_lpr: batch does not belong to this engine");
    if (model < 0 || model > 1) return e->fail(PCSF_EINVAL, "pcsf_lpr: model %d", model);
    if (b->nreg > 0 && (!rho || !lpr)) return e->fail(PCSF_EINVAL, "pcsf_lpr: null output");
    std::vector<Request> reqs(b->nreg);
    for (int r = 0; r < b->nreg; r++) {
        if (!(rho[r] > 0.0) || !std::isfinite(rho[r])) return e->fail(PCSF_EINVAL, "pcsf_lpr: rho[%d] = %g", r, rho[r]);
        reqs[r] = Request{r, model, 0, 0, rho[r]};
    }
    std::vector<Eval> res;
    int rc = e->tc_direct ? evaluate(e, b, reqs, res) : evaluate_returned(e, b, reqs, res);
    if (rc) return rc;
    for (int r = 0; r < b->nreg; r++) {
        lpr[r] = res[r].lpr;
        if (elpr) elpr[r] = res[r].elpr;
        if (status) status[r] = res[r].status;
    }
    return PCSF_OK;
}

int pcsf_branch_counts(pcsf_engine *e, pcsf_batch *b, int32_t model, const double *rho, double *counts, double *lpr,
                       int32_t *status)
{
    if (!e) return PCSF_EINVAL;
    if (!e->has_models) return e->fail(PCSF_EINVAL, "this engine has no coding / noncoding models");
    CK(cudaSetDevice(e->device), "cudaSetDevice");
    if (!b || b->e != e) return e->fail(PCSF_EINVAL, "pcsf_branch_counts: batch does not belong to this engine");
    if (model < 0 || model > 1) return e->fail(PCSF_EINVAL, "pcsf_branch_counts: model %d", model);
    if (b->nreg > 0 && (!rho || !counts)) return e->fail(PCSF_EINVAL, "pcsf_branch_counts: null argument");
    return outside_impl(e, b, model, rho, counts, 0, nullptr, nullptr, lpr, status);
}

int pcsf_node_posteriors(pcsf_engine *e, pcsf_batch *b, int32_t model, const double *rho, int32_t n_nodes,
                         const int32_t *nodes, double *post, int32_t *status)
{
    if (!e) return PCSF_EINVAL;
    if (!e->has_models) return e->fail(PCSF_EINVAL, "this engine has no coding / noncoding models");
    CK(cudaSetDevice(e->device), "cudaSetDevice");
    if (!b || b->e != e) return e->fail(PCSF_EINVAL, "pcsf_node_posteriors: batch does not belong to this engine");
    if (model < 0 || model > 1) return e->fail(PCSF_EINVAL, "pcsf_node_posteriors: model %d", model);
    if (n_nodes < 0 || (n_nodes > 0 && (!nodes || !post)) || (b->nreg > 0 && !rho))
        return e->fail(PCSF_EINVAL, "pcsf_node_posteriors: null argument");
    if (n_nodes == 0) return PCSF_OK;
    return outside_impl(e, b, model, rho, nullptr, n_nodes, nodes, post, nullptr, status);
}

int pcsf_ell(pcsf_engine *e, int32_t model, double rho, const double *counts, double *ell)
{
    if (!e) return PCSF_EINVAL;
    if (!e->has_models) return e->fail(PCSF_EINVAL, "this engine has no coding / noncoding models");
    CK(cudaSetDevice(e->device), "cudaSetDevice");
    if (model < 0 || model > 1 || !counts || !ell) return e->fail(PCSF_EINVAL, "pcsf_ell: bad argument");
    if (!(rho > 0.0) || !std::isfinite(rho)) return e->fail(PCSF_EINVAL, "pcsf_ell: rho = %g", rho);
    return ell_impl(e, model, rho, counts, ell);
}

int pcsf_grad(pcsf_engine *e, pcsf_batch *b, int32_t model, const double *rho, double *lpr, double *d_branch,
              double *d_rho, int32_t *status)
{
    if (!e) return PCSF_EINVAL;
    if (!e->has_models) return e->fail(PCSF_EINVAL, "this engine has no coding / noncoding models");
    CK(cudaSetDevice(e->device), "cudaSetDevice");
    if (!b || b->e != e) return e->fail(PCSF_EINVAL, "pcsf_grad: batch does not belong to this engine");
    if (model < 0 || model > 1) return e->fail(PCSF_EINVAL, "pcsf_grad: model %d", model);
    if (b->nreg > 0 && (!rho || !lpr)) return e->fail(PCSF_EINVAL, "pcsf_grad: null output");
    std::vector<Request> reqs(b->nreg);
    for (int r = 0; r < b->nreg; r++) {
        if (!(rho[r] > 0.0) || !std::isfinite(rho[r])) return e->fail(PCSF_EINVAL, "pcsf_grad: rho[%d] = %g", r, rho[r]);
        reqs[r] = Request{r, model, 0, 0, rho[r]};
    }
    std::vector<Eval> res;
    std::vector<double> g;
    if (!d_branch && e->tc_direct && e->dual_ok) {
        // precision-study mode: lpr and d lpr / d rho straight from the tensor-core tangent pass
        std::vector<double> dr;
        int rc = evaluate(e, b, reqs, res, nullptr, false, nullptr, &dr);
        if (rc) return rc;
        for (int r = 0; r < b->nreg; r++) {
            lpr[r] = res[r].lpr;
            if (status) status[r] = res[r].status;
            if (d_rho) d_rho[r] = dr[r];
        }
        return PCSF_OK;
    }
    int rc = evaluate(e, b, reqs, res, &g);
    if (rc) return rc;
    for (int r = 0; r < b->nreg; r++) {
        lpr[r] = res[r].lpr;
        if (status) status[r] = res[r].status;
        // t_c = rho * b_c: d lpr / d rho = sum_c b_c d lpr / d t_c
        double dr = 0.0;
        for (int c = 0; c < e->nbr; c++) {
            double gc = g[(size_t)r * e->nbr + c];
            if (d_branch) d_branch[(size_t)r * e->nbr + c] = gc;
            dr += e->branch[c] * gc;
        }
        if (d_rho) d_rho[r] = dr;
    }
    return PCSF_OK;
}

}  // extern "C"
