// Internal declarations shared by the host runtime and the CUDA kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/phylocsf_engine.h"

namespace pcsf {

constexpr int K = 64;          // codon states (Code.Codon64.dim)
constexpr int K2 = K * K;
constexpr int MAX_LEAVES = 512;

// One internal node of the pruning schedule, in evaluation order.  A child
// slot of -1 means the child is a leaf (its partial is a one-hot gather).
struct SchedNode {
    int16_t node, lc, rc;
    int8_t lslot, rslot, oslot, pad;
};
static_assert(sizeof(SchedNode) == 10, "SchedNode layout");

// A distinct (model, tree scale) pair: one set of P(t) matrices for every branch.
struct PSet {
    int32_t model;
    int32_t pad;
    double rho;
};

// A likelihood evaluation: region, model (0 coding / 1 noncoding), tree scale,
// and the index of its P set within the launch chunk.
struct Request {
    int32_t region;
    int32_t model;
    int32_t pset;
    uint32_t start;    // low 32 bits of the region's first global column (set by the launcher)
    double rho;
};

// A pruning work item: a tile of columns of one request's region.
struct WorkItem {
    int32_t request;   // index into the launch's request array
    int32_t ncols;     // columns in this tile (<= tile width)
    int64_t col0;      // first global column of the tile
};

// Device view of the two models' eigensystems (all arrays [2][...]).
constexpr int WLIST = 4;
struct DevModels {
    const double *U;        // [2][K][K]  eigenvectors of D^1/2 Q D^-1/2 (columns)
    const float *Uf;        // [2][K][K]  FP32 copy
    const double *lam;      // [2][K]
    const double *sq;       // [2][K]     sqrt(pi)
    const double *isq;      // [2][K]     1/sqrt(pi)
    const double *wrow;     // [2][K]     w_m = sum_j U_jm sqrt(pi_j)  (row-sum identity)
    const int16_t *wlist;   // [2][WLIST] the m with w_m != 0, -1 padded; wlist[0] = -2: more than WLIST
    const double *prior;    // [2][K]     root prior
    const double *wlog;     // [2][K]     prior_a * log(prior_a)
    double tol;             // Q.Diag tol (1e-6)
    // FP32 P(t) formation: E(t) = E(t_g) + D^-1/2 U diag(e^{lam t} - e^{lam t_g}) U^T D^1/2
    // around the nearest point t_g of a geometric grid whose E(t_g) were formed
    // in FP64; below the first grid point E(t) = t Q + t^2/2 Q^2.
    const float *gridT;     // [2][G][K][K]  E(t_g)^T in FP32
    const double *grid_t;   // [G]
    const float *grid_eg;   // [2][G][K]     e^{lam_m t_g}
    int grid_n;
    double grid_lr;         // log of the grid ratio
    const float *Qf;        // [2][K][K]  Q (row-major)
    const float *Q2f;       // [2][K][K]  Q^2
};

// Status keys: ((branch*K + row) << 4) | code, min-reduced so the first error
// in the reference's (branch, row) order wins.  INT32_MAX = no error.
constexpr int32_t STATUS_NONE = 0x7f7f7f7f;   // what cudaMemset(0x7f) leaves

struct LaunchStats {
    float ms = 0.f;
};

// ---- kernels (kernels.cu) -------------------------------------------------
// Jacobi eigensolver: A [nmat][K][K] symmetric -> U [nmat][K][K], lam [nmat][K].
cudaError_t launch_jacobi(const double *A, double *U, double *lam, int *status, int nmat, cudaStream_t s);

// P(t) formation for P sets [nps]: writes E^T = (P - I)^T per branch into
// Pbuf ([nps][nbr][K][K], element (j,i) = E[i][j]) in FP64 or FP32.
// raw = true skips the row rule (used to form the FP64 grid itself).
// bop (FP32 only, may be null): tensor-core B operands, [set][nbr - bop_nl][hi, lo][64 x 64],
// of the branches b >= bop_nl (the branches above internal nodes when bop_nl = n_leaves)
// dlo (FP32 only, may be null): [set][nbr][K] low parts of the diagonal of E, so that
// E_ii + dlo_i carries the row rule's diagonal to ~2^-48 (see k_prune)
cudaError_t launch_pform(bool fp64, const PSet *ps, int nps, const double *branch, int nbr,
                         DevModels m, void *Pbuf, int32_t *status_key, cudaStream_t s, bool raw = false,
                         float *bop = nullptr, int bop_nl = 0, float *dlo = nullptr);
cudaError_t launch_d2f(const double *in, float *out, size_t n, cudaStream_t s);
cudaError_t launch_d2f_rows(const double *in, float *out, size_t nmat, int nbr, float *bop, int bop_nl, cudaStream_t s,
                            float *dlo = nullptr);
// Leaf codes of an uploaded batch: *first_bad = the smallest index of a byte > 64
// (PCSF_MARGINALIZE), left unchanged when every code is valid.
cudaError_t launch_check_codes(const uint8_t *codes, size_t n, unsigned long long *first_bad, cudaStream_t s);

// Pruning over work items [nwi]; partials [nwi][2] (lpr, elpr).
struct PruneArgs {
    const WorkItem *wi;
    int nwi;
    const Request *req;
    const uint8_t *leaves;   // [total_cols][nl]
    const void *Pbuf;        // per chunk-local P set: [nbr][K][K] E^T
    const SchedNode *sched;  // [n_internal]
    int n_internal;
    int nl;
    int nbr;
    int nslots;
    DevModels m;
    double *partials;        // [nwi][2]
    const void *Bop;         // tensor-core kernel: per chunk-local P set, [nbop][hi, lo][64 x 64] B operands
    int nbop;                //   of the branches above internal nodes (node nl + k)
    int dither;              // SIMT FP32 kernel: per-column dithering of the leaf partials (prune_common.cuh)
    const float *dlo;        // SIMT FP32 kernel, may be null: per chunk-local P set [nbr][K] low parts of diag(E)
    int tile;                // SIMT FP32 kernel: column tile 32 or 64, 0 = the default rule (simt_tile_cols)
    int tc_shape;            // TF32 tensor-core kernel: 0 alpha kept in registers, 1 read back (identical values)
};
// comp: 0 plain FP32 sums, 1 Kahan, 2 blocked Kahan (see prune_common.cuh)
cudaError_t launch_prune(int prec, int comp, const PruneArgs &a, cudaStream_t s, int grid);
int prune_tile_cols(int prec);
int simt_tile_cols(int prec, int nslots, int tile = 0);   // the SIMT kernel's column tile (k_prune)
size_t prune_smem_bytes(int prec, int nslots, int nl, int nint, int tile = 0);

// Adjoint gradient over work items (grad_kernels.cu): per work item the lpr /
// elpr partials and d lpr / d t_c for every branch c.
struct GradArgs {
    const WorkItem *wi;
    int nwi;
    const Request *req;
    const uint8_t *leaves;
    const void *Pbuf;
    const SchedNode *sched;
    int n_internal;
    int nl;
    int nbr;
    int nslots;
    DevModels m;
    const void *Qrow;        // [model][K][K] Q row-major in the arithmetic type
    void *scratch;           // gridDim.x * scratch_per_cta bytes
    size_t scratch_per_cta;
    double *partials;        // [nwi][2]
    double *gpart;           // [nwi][nbr + npar]
    // rate-matrix parameter derivatives (OmegaModel kappa, omega): d lpr / d x =
    // sum_c sum_col inter_c^T (dP_c / dx) alpha_c / z, with dP/dx = D^-1/2 U (F o Bdot_x) U^T D^1/2
    int npar;                // 0 or 2
    const void *Hmat;        // [pset][nbr][npar][K][K] (F(t_c) o Bdot_x)^T, arithmetic type
    const void *Umat;        // [model][K][K] U row-major, arithmetic type
    int recompute_leaves;    // leaf children's partials recomputed in the outside pass, not stored
};
cudaError_t launch_grad(int prec, int comp, const GradArgs &a, cudaStream_t s, int grid);
size_t grad_scratch_per_cta(int prec, int nl, int npar, bool recompute_leaves);
size_t grad_smem_bytes(int prec, int nslots, int nl, int nint, int npar);
// H_x = (F(t) o Bdot_x)^T for every (P set, branch, parameter): F_ij = (e^{lam_i t} - e^{lam_j t}) /
// (lam_i - lam_j), t e^{lam_i t} on the diagonal (Frechet derivative of exp in the eigenbasis)
cudaError_t launch_hform(bool fp64, const PSet *ps, int nps, const double *branch, int nbr, const double *lam,
                         const void *Bdot, void *H, cudaStream_t s);
cudaError_t launch_reduce_grad(const double *gpart, const int32_t *wi_begin, int nreq, int nbr, double *grad,
                               cudaStream_t s);

// Tensor-core pruning (tc_kernels.cu): nprod 3 = TF32 hi/lo split, 1 = single TF32.
cudaError_t launch_prune_tc(int nprod, const PruneArgs &a, int *err, cudaStream_t s, int grid);
size_t prune_tc_smem_bytes(int nl, int nint);
bool prune_tc_supported(int nslots, int nl);
constexpr int PCSF_TC_SHAPES = 2;
int prune_tc_ctas_per_sm(int nslots, int nl, int nint, int shape);
bool prune_tc_shape_ok(int shape);
// Tensor-core pruning with BF16 split products (tc_bf16.cu): x = h + m + l, six
// products on tcgen05 kind::f16, FP32 accumulation; E^T of every branch in Pbuf (FP32).
cudaError_t launch_prune_bf16(const PruneArgs &a, int *err, cudaStream_t s, int grid);
size_t prune_bf16_smem_bytes(int nl, int nint);
bool prune_bf16_supported(int nslots, int nl);
int prune_bf16_ctas_per_sm(int nslots, int nl, int nint);
// tensor-core P(t) formation for the search evaluations (tc_pform.cu): E^T of the
// branches above leaves into Pbuf, B operands of the branches above internal
// nodes into Bop; Bpf = per model the pre-split B = U^T D^1/2 [2][hi, lo][64 x 64]
cudaError_t launch_pform_tc(const PSet *ps, int nps, const double *branch, int nbr, int nl, DevModels m,
                            const float *Bpf, float *Pbuf, float *Bop, int32_t *status_key, int *err, cudaStream_t s);
// tensor-core tangent pass (tc_dual.cu): lpr / elpr partials as k_prune_tc plus
// d lpr / d rho partials dpart [nwi][2] (second entry 0); Qop = per model the
// pre-split B operand of Q [2][hi, lo][64 x 64]; branch = the tree's lengths
cudaError_t launch_prune_tc_dual(const PruneArgs &a, const float *Qop, const double *branch, double *dpart, int *err,
                                 cudaStream_t s, int grid);
size_t prune_tc_dual_smem_bytes(int nl, int nint);
bool prune_tc_dual_supported(int nslots, int nl);

// Sum the partials of each request's contiguous work items in fixed order.
// out_index (may be null): request r's sums go to out_*[out_index[r]] instead of out_*[r].
cudaError_t launch_reduce(const double *partials, const int32_t *wi_begin, int nreq, double *out_lpr,
                          double *out_elpr, cudaStream_t s, const int32_t *out_index = nullptr);

// Float-float SIMT pruning (ff_kernels.cu): returned values that agree with the FP64
// path to ~1e-12 relative.  Pbuf holds split E^T sets, per P set [nbr][hi K2 | lo K2]
// floats, made from the FP64 P(t) formation's output by launch_split_ff; tiles of
// ff_tile_cols() columns; partials as k_prune.
cudaError_t launch_prune_ff(const PruneArgs &a, cudaStream_t s, int grid);
cudaError_t launch_split_ff(const double *in, float *out, size_t nmat, cudaStream_t s);
int ff_tile_cols();
size_t prune_ff_smem_bytes(int nslots, int nl, int nint);
int prune_ff_ctas_per_sm(int nslots, int nl, int nint);

// Outside-pass products (outside_kernels.cu): per request (one CTA at a time, tiles of
// outside_tile_cols() columns in order) the log-likelihood, optionally the expected
// substitution counts of every branch and the posteriors of selected nodes.
struct OutsideArgs {
    const WorkItem *wi;          // work items, contiguous per request
    const int32_t *wi_begin;     // [nreq + 1]
    int nreq;
    const Request *req;          // Request.pset indexes Pbuf
    const uint8_t *leaves;       // [total_cols][nl]
    const void *Pbuf;            // per P set [nbr][K][K] E^T, FP64 or FP32
    const SchedNode *sched;
    int n_internal, nl, nbr, nslots;
    DevModels m;
    void *scratch;               // gridDim.x * scratch_per_cta bytes
    size_t scratch_per_cta;
    double *lpr;                 // [nreq]
    double *counts;              // [nreq][nbr][K][K], zeroed by the caller; null: none
    const int32_t *sel;          // [n] output row of each node, -1 if not selected; null: no posteriors
    double *post;                // [n_selected][total_cols][K]
    int64_t total_cols;
};
cudaError_t launch_outside(bool fp64, int comp, const OutsideArgs &a, cudaStream_t s, int grid);
int outside_tile_cols();
size_t outside_smem_bytes(bool fp64, int nslots, int nl, int nint);
size_t outside_scratch_per_cta(bool fp64, int nl);

// Read-only view of an engine's device state for the allocation-free entry point
// (noalloc.cu; filled by engine.cpp).
struct NoallocCtx {
    int device;
    cudaStream_t stream;
    int prec;              // PCSF_PREC_*
    int comp;              // summation mode of the returned-value kernel (as pcsf_lpr uses it)
    bool pt64;             // P(t) formed in FP64 and rounded to FP32 (PCSF_PT_FP64)
    bool tc_direct;        // pcsf_lpr returns tensor-core values (PCSF_TC_DIRECT)
    bool has_models;
    int nl, nbr, n_internal, nslots;
    const double *branch;
    const SchedNode *sched;
    DevModels m;
    int prune_grid;
    int simt_tile;         // SIMT column tile chosen for the engine (0: the default rule)
    int ff_grid;           // CTAs of the float-float kernel (0: not available)
    int64_t exact_min_units;   // regions with columns x (nl - 2) >= this use the float-float kernel
    int *derr;             // device error flag of timed-out waits
};

}  // namespace pcsf
