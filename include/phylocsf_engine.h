/*
 * phylocsf_engine.h -- C-ABI of the GB300 (sm_103a) PhyloCSF likelihood engine.
 *
 * The engine replaces everything below PhyloCSF's per-region `evaluator`
 * closure (src/PhyloCSF.ml:437-467, called at :317-322): P(t) formation from an
 * FP64 eigendecomposition of each codon rate matrix, Felsenstein pruning, the
 * rho maximum-likelihood search and the coding-vs-noncoding LLR in decibans.
 * Paths cited below are relative to the mlin/PhyloCSF source tree.
 *
 * Conventions
 *   - Plain C types only; the caller owns every buffer it passes in.  The
 *     engine owns its device memory and CUDA stream.
 *   - One engine per host thread.  Calls on one engine are serialised by the
 *     caller; distinct engines may be used from distinct threads.
 *   - Every call returns a status (PCSF_OK = 0).  Per-region failures are
 *     reported in pcsf_result.status and do not fail the whole call, mirroring
 *     the reference's per-region `exception` lines (PhyloCSF.ml:323-349).
 *   - No CPU fallback: creating an engine without a usable GB300 fails with
 *     PCSF_ECUDA.
 *   - Create no engine before fork(): a CUDA context must not cross fork().
 */
#ifndef PHYLOCSF_ENGINE_H
#define PHYLOCSF_ENGINE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PCSF_ABI_VERSION 1

/* status codes */
#define PCSF_OK 0
#define PCSF_EINVAL 1     /* invalid argument (tree shape, sizes, leaf codes)       */
#define PCSF_ECUDA 2      /* CUDA error or no usable device                          */
#define PCSF_ENOMEM 3     /* device or host allocation failed                        */
#define PCSF_ENEGP 4      /* expm(tQ) entry below -tol             (Q.ml:234-236)   */
#define PCSF_EROWSUM 5    /* |sum of a P(t) row - 1| > tol         (Q.ml:243-244)   */
#define PCSF_EDIAG 6      /* renormalised P(t) diagonal not in (0,1] (Q.ml:245)     */
#define PCSF_EBRACKET 7   /* Brent set-up found no bracketed maximum (Fit.ml:13)   */
#define PCSF_EEIG 8       /* eigensolver did not converge                            */
#define PCSF_ESCALE 9     /* Q scale evaluated to <= 0             (PhyloModel.ml:98) */
#define PCSF_ERANGE 10    /* batch larger than a fixed capacity                      */

/* strategies (PhyloCSFModel.ml:138-146) */
#define PCSF_FIXED 0      /* rho = 1                                                 */
#define PCSF_MLE 1        /* rho maximised in [0.01, 10] by find_init + Brent        */

/* arithmetic of the pruning contractions (engine flags, low byte) */
#define PCSF_PREC_FP64 0  /* FP64 everywhere: the oracle-matched plain GPU path      */
#define PCSF_PREC_FP32 1  /* FP32 contractions on P(t)-I, FP64 eigensystem and sums  */
#define PCSF_PREC_TF32X3 2 /* tcgen05 TF32 hi/lo split (3 products), FP32 accumulate */
#define PCSF_PREC_BF16X3 3 /* tcgen05 BF16 split x = h + m + l (exact), the 6 products
                              that reach FP32 accuracy, FP32 accumulate                 */
#define PCSF_PREC_TF32 4  /* tcgen05 single TF32 product (precision study only)      */

/* engine flag: compensated (Kahan) summation in the FP32 contractions.  FP32
 * accumulation of many small positive terms into a large sum drops the ones
 * below half an ulp, a bias that accumulates over thousands of columns. */
#define PCSF_COMPENSATED (1 << 16)
/* engine flag: blocked compensation -- eight products summed plainly, each block
 * folded in with Kahan's correction (about a ninth of the plain bias, a third of
 * the cost of PCSF_COMPENSATED).  Also selects the kernel that produces the
 * returned values of the tensor-core modes. */
#define PCSF_BLOCK_COMPENSATED (1 << 18)

/* engine flag for the tensor-core modes: pcsf_lpr returns the tensor-core
 * kernel's values instead of the compensated FP32 kernel's (precision study). */
#define PCSF_TC_DIRECT (1 << 17)

/* engine flag for the FP32 and tensor-core modes: form every P(t) in FP64 (as
 * the FP64 engine does) and round it to FP32, re-forming each diagonal from its
 * rounded row, instead of the FP32 grid correction.  Much slower (FP64 GEMMs);
 * for accuracy studies. */
#define PCSF_PT_FP64 (1 << 19)

/* engine flags, bits 8..15: CUDA device ordinal + 1 (0 = the calling thread's
 * current device).  Every call on an engine runs on the engine's device. */
#define PCSF_DEVICE(d) ((((int32_t)(d)) + 1) << 8)

/* leaf code for a marginalised leaf (gap, N, absent species; PhyloCSF.ml:231-238) */
#define PCSF_MARGINALIZE 64

typedef struct pcsf_engine pcsf_engine;
typedef struct pcsf_batch pcsf_batch;

/* Tree in CamlPaml T order (lib/CamlPaml/T.ml:57-112): leaves 0..nl-1 in Newick
 * left-to-right order, internal nodes numbered post-order, root = 2nl-2.
 * parent[root] = -1; branch[i] = length of the branch leading into node i. */
typedef struct {
    int32_t n_leaves;
    const int32_t *parent;  /* [2*n_leaves-1] */
    const double *branch;   /* [2*n_leaves-2] */
} pcsf_tree;

/* One region's score (PhyloCSFModel.score, PhyloCSFModel.ml:113-146). */
typedef struct {
    double score;           /* decibans, 10*(lpr_c - lpr_n)/ln 10        */
    double anc_comp_score;  /* decibans, 10*(elpr_c - elpr_n)/ln 10      */
    double rho_c, rho_n;    /* tree scale used for each model            */
    double lpr_c, lpr_n;    /* natural-log likelihoods                    */
    double elpr_c, elpr_n;  /* expected log prior of the root state       */
    int32_t status;         /* PCSF_OK or the first error for this region */
    int32_t evals;          /* distinct likelihood evaluations, both models */
} pcsf_result;

/* Engine statistics since creation (or the last pcsf_engine_reset_stats). */
typedef struct {
    int64_t kernel_launches;     /* launches of this library's kernels          */
    int64_t evaluations;         /* (region, model, rho) likelihood evaluations */
    int64_t column_branches;     /* codon-column x branch units processed       */
    int64_t rounds;              /* lockstep optimisation rounds                */
    double prune_ms;             /* device time of pruning kernels              */
    double pform_ms;             /* device time of P(t) formation kernels       */
    double other_ms;             /* device time of the other kernels            */
    int64_t prune_launches;
    int64_t pform_launches;
    /* by pruning-kernel kind: 0 SIMT (returned values), 1 tensor core (search),
     * 2 adjoint gradient, 3 tensor-core tangent (d lpr / d rho for the search),
     * 4 float-float SIMT (returned values of long regions, and the search
     * decisions of long regions that the tensor-core values cannot settle) */
    int64_t kind_launches[5];
    int64_t kind_columns[5];     /* codon-column evaluations (columns x requests)  */
    double kind_ms[5];           /* device time (these sum to prune_ms)            */
    int32_t prune_grid;     /* launch configuration (not counters): CTAs of the SIMT pruning kernel, */
    int32_t tc_grid;        /* and of the tensor-core kernel (0 if the engine has none),             */
    int32_t simt_tile;      /* and the SIMT kernel's column tile                                     */
    int32_t tc_shape;       /* and the TF32 tensor-core search kernel's shape (-1: none; see below)  */
} pcsf_stats;

/* ---------------------------------------------------------------- engine */

/* Create an engine for one tree and the coding / noncoding ECMs.
 * S_*: 64x64 row-major exchangeabilities (symmetric, zero diagonal), pi_*: 64
 * equilibrium frequencies, as read by ECM.import_parameters (src/ECM.ml:18-72).
 * Q is assembled and scaled as PhyloCSFModel.make_q_p14n / qscale
 * (PhyloCSFModel.ml:11-30), eigendecomposed in FP64 on the GPU (replaces
 * Q.Diag.of_Q, Q.ml:124-141).  The root prior is pi (PhyloCSFModel.ml:56).
 * flags: PCSF_PREC_* in the low byte.
 * Replaces PhyloCSFModel.make (PhyloCSFModel.ml:107-110). */
int pcsf_engine_create(const pcsf_tree *tree, const double *S_c, const double *pi_c, const double *S_n,
                       const double *pi_n, int32_t flags, pcsf_engine **out);

/* Create an engine from explicit reversible rate matrices (no scaling applied).
 * Q_*: 64x64 row-major rate matrices reversible with respect to eq_*; prior_*
 * is the root distribution.  Used for models that are not ECMs (for example a
 * smaller alphabet embedded in the 64 codon states).
 * Replaces PhyloModel.make with explicit Q.Diag.t values (PhyloModel.ml:12-25). */
int pcsf_engine_create_q(const pcsf_tree *tree, const double *Q_c, const double *eq_c, const double *prior_c,
                         const double *Q_n, const double *eq_n, const double *prior_n, int32_t flags,
                         pcsf_engine **out);

/* Create an engine for one tree without fixed models, for the OmegaModel test
 * (pcsf_omega_score), whose rate matrices change with every kappa. */
int pcsf_engine_create_tree(const pcsf_tree *tree, int32_t flags, pcsf_engine **out);

void pcsf_engine_destroy(pcsf_engine *e);

/* Last error message of this engine (static storage if e == NULL). */
const char *pcsf_last_error(const pcsf_engine *e);

int pcsf_engine_get_stats(const pcsf_engine *e, pcsf_stats *out);
int pcsf_engine_reset_stats(pcsf_engine *e);

/* Long regions on FP32 and tensor-core engines: a region whose columns x
 * (n_leaves - 2) reach `units` takes its returned values -- and the search
 * decisions that the search values cannot settle -- from the float-float kernel
 * (FP64 P(t), partials carried as float pairs, ~1e-12 relative to the FP64 path)
 * instead of the compensated FP32 kernel, whose error grows with the region's
 * length (about 1.9e-9 dB per column x internal node: 3e-4 dB at 2,000 codons on a
 * 100-leaf tree).  Default 150000 (2,679 codons on 58 leaves, 1,531 on 100).  0: every returned value from the
 * float-float kernel.  Ignored by the FP64 engine.  No reference counterpart (the
 * reference computes in FP64 throughout). */
int pcsf_engine_set_exact_threshold(pcsf_engine *e, int64_t units);

/* 1 if the engine has the float-float kernel (FP32 and tensor-core engines whose
 * tree fits its shared memory), else 0. */
int pcsf_engine_exact_available(const pcsf_engine *e);

/* Autotuner of the column tile of the compensated FP32 kernel (the returned values
 * and the accurate search decisions).  Each candidate tile (32 and 64 columns, with
 * the CTAs per SM its shared memory allows) is timed on the engine's stream over up
 * to 256 regions of the batch at evenly spaced length quantiles (both models,
 * rho = 1, one warm-up and two timed passes each); the fastest is kept for every
 * later call on this engine and written to *tile (may be NULL).  The choice depends
 * on the tree (partial slots and leaves) and the precision.  The FP64 engine has one
 * tile (32) and keeps it.  TF32 tensor-core engines also time the search kernel's
 * shapes on the same sample and keep the faster (pcsf_stats.tc_shape):
 *   0: each column's partial (alpha) kept in registers from the operand staging to the
 *      epilogue;  1: alpha read back from the MMA operands in the epilogue.
 * Both issue the same MMAs on the same operands: the values are identical.
 * No reference counterpart (the reference has no device). */
int pcsf_engine_autotune(pcsf_engine *e, pcsf_batch *b, int32_t *tile);

/* Derivative of the search values for the derivative rule of reduced-precision mle
 * searches (a trial point within 1e-4 |x| of the best point x is valued as
 * f(x) + f'(x)(u - x)): mode 1 = central difference of two search evaluations at
 * x (1 +- 2e-3) (the default of tensor-core engines: about half the cost of the
 * tangent pass), 0 = the analytic derivative (the tensor-core tangent pass where the
 * tree fits it, else the adjoint; the default of the other engines). */
int pcsf_engine_set_derivative_mode(pcsf_engine *e, int32_t mode);

/* Adjoint memory (pcsf_grad, pcsf_omega_grad and the derivative rule of engines without
 * the tangent pass): with on != 0 the outside pass recomputes the partials of leaf
 * children (one gathered row of P each) instead of storing them, a third less scratch
 * per CTA for ~5 % more adjoint time; the gradients are identical either way.  Default
 * off.  pcsf_engine_grad_scratch_bytes gives the scratch per CTA under the current
 * setting (n_rate_params 0, or 2 for pcsf_omega_grad), -1 on a bad argument. */
int pcsf_engine_set_grad_recompute(pcsf_engine *e, int32_t on);
int64_t pcsf_engine_grad_scratch_bytes(const pcsf_engine *e, int32_t n_rate_params);

/* Set the TF32 tensor-core search kernel's shape (0 or 1, above) by hand; TF32
 * tensor-core engines only. */
int pcsf_engine_set_tc_shape(pcsf_engine *e, int32_t shape);

/* The autotuner's device time per pass of each search-kernel shape (ms; 0 where
 * untimed), n entries at most. */
int pcsf_engine_tc_shape_times(const pcsf_engine *e, double *ms, int32_t n);

/* The CUDA stream (a cudaStream_t) on which the engine launches all of its
 * work, so that callers can time it with events on that stream.  No reference
 * counterpart (the reference has no device). */
int pcsf_engine_stream(const pcsf_engine *e, void **stream);

/* Device eigensystem of model m (0 coding, 1 noncoding): U (64x64 row-major,
 * eigenvectors in columns of D^1/2 Q D^-1/2) and lambda (64). */
int pcsf_engine_eigensystem(const pcsf_engine *e, int32_t model, double *U, double *lambda);

/* Form P(t) for model m at the given branch lengths (n_t of them) with the
 * clamp / renormalise rule of Q.Diag.real_to_Pt (Q.ml:211-249).
 * P: [n_t][64][64] row-major FP64.  Per-matrix status in status[n_t]. */
int pcsf_engine_pt(pcsf_engine *e, int32_t model, int32_t n_t, const double *t, double *P, int32_t *status);

/* P(t) as the tensor-core search forms it (TF32 hi/lo products around the FP32
 * grid, k_pform_tc), for checking: P: [n_t][64][64] row-major (1 <= n_t <= 320),
 * status [n_t] (one status for the call) may be NULL.  TF32 tensor-core engines
 * only.  Replaces nothing in the reference: the search's P(t) has no counterpart
 * (the reference forms every P(t) by Q.Diag.to_Pt, Q.ml:211-256). */
int pcsf_engine_pt_search(pcsf_engine *e, int32_t model, int32_t n_t, const double *t, double *P, int32_t *status);

/* ---------------------------------------------------------------- batches */

/* Upload a batch of regions.  Region r is columns [col_offsets[r],
 * col_offsets[r+1]); leaves is [total_cols][n_leaves] uint8 codon indices
 * 16*n1+4*n2+n3 (Code.ml:140-141), PCSF_MARGINALIZE for a marginalised leaf
 * (this packs PhyloCSF.pleaves' output, PhyloCSF.ml:219-246).  The codes are
 * checked on the device after the upload; a code above PCSF_MARGINALIZE fails the
 * call with PCSF_EINVAL, naming the first bad column and leaf. */
int pcsf_batch_create(pcsf_engine *e, int32_t n_regions, const int64_t *col_offsets, const uint8_t *leaves,
                      pcsf_batch **out);
/* Frees the batch's device memory; valid before or after its engine is destroyed. */
void pcsf_batch_destroy(pcsf_batch *b);

/* Score every region of a resident batch (PhyloCSFModel.score,
 * PhyloCSFModel.ml:142-146, for all regions at once; MLE fits advance in
 * lockstep rounds on the device).  out: [n_regions]. */
int pcsf_score(pcsf_engine *e, pcsf_batch *b, int32_t strategy, pcsf_result *out);

/* One-shot scoring from host buffers: upload, score, free.  This is the call
 * a batching ForkMaybe.map would make over its region list (PhyloCSF.ml:317). */
int pcsf_score_batch(pcsf_engine *e, int32_t n_regions, const int64_t *col_offsets, const uint8_t *leaves,
                     int32_t strategy, pcsf_result *out);

/* Log-likelihood of every region under model m at tree scale rho[r]
 * (PhyloCSFModel.lpr_leaves, PhyloCSFModel.ml:67-82).  lpr, elpr, status:
 * [n_regions]; elpr and status may be NULL. */
int pcsf_lpr(pcsf_engine *e, pcsf_batch *b, int32_t model, const double *rho, double *lpr, double *elpr,
             int32_t *status);

/* Gradient of lpr by the adjoint (outside) pass: d lpr / d branch_i at
 * t_i = rho*b_i for every branch (d_branch: [n_regions][2*n_leaves-2], may be
 * NULL) and d lpr / d rho (d_rho: [n_regions]).  The reference's
 * equivalent is PhyloEM.d_ell_dtree via branch posteriors (PhyloEM.ml:140-182,
 * PhyloLik.ml:96-174, Q.ml:260-275); it is the backward of pcsf_lpr in the
 * sense of an autograd.Function.  On a tensor-core engine created with
 * PCSF_TC_DIRECT, d_branch == NULL selects the forward-mode tangent pass on the
 * tensor cores (lpr and d lpr / d rho only), the derivative the engine's own
 * rho search uses. */
int pcsf_grad(pcsf_engine *e, pcsf_batch *b, int32_t model, const double *rho, double *lpr, double *d_branch,
              double *d_rho, int32_t *status);

/* ---------------------------------------------- outside-pass statistics */

/* Expected substitution counts of every branch, summed over each region's columns,
 * for model m at tree scale rho[r]:
 *   counts[r][i][a][b] = sum_col beta_p[a] (P_s alpha_s)[a] P_i[a][b] alpha_i[b] / z
 * (p the parent of node i, s its sibling, P_i = P(rho[r] b_i)).  This is
 * PhyloLik.add_branch_posteriors (lib/CamlPaml/PhyloLik.ml:140-174) accumulated over
 * the columns as PhyloEM.collect_sufficient_statistics does (lib/CamlPaml/PhyloEM.ml:14-20).
 * Each branch's counts sum to the number of columns with z > 0.  counts:
 * [n_regions][2*n_leaves-2][64][64]; lpr and status ([n_regions]) may be NULL.
 * Computed in FP64 on the FP64 engine, in FP32 with compensated sums otherwise. */
int pcsf_branch_counts(pcsf_engine *e, pcsf_batch *b, int32_t model, const double *rho, double *counts, double *lpr,
                       int32_t *status);

/* Expected log-likelihood of sufficient statistics (PhyloEM.ell,
 * lib/CamlPaml/PhyloEM.ml:22-73) for model m at tree scale rho: the sum over
 * branches of counts x log P(rho b_i) over the positive counts, plus the root prior
 * term from the row sums of the counts of the root's left child.  counts:
 * [2*n_leaves-2][64][64] (one region's counts from pcsf_branch_counts, or a sum of
 * several).  P(t) is formed in FP64. */
int pcsf_ell(pcsf_engine *e, int32_t model, double rho, const double *counts, double *ell);

/* Posterior state distributions of selected nodes at every column of a batch, for
 * model m at tree scale rho[r] of each region (PhyloLik.node_posterior,
 * lib/CamlPaml/PhyloLik.ml:127-138): alpha_i[a] beta_i[a] / z for an internal node or
 * the root, the leaf's own vector (one-hot, or all ones when marginalised) for a
 * leaf, and zeros where z = 0.  nodes: [n_nodes] in T order; post:
 * [n_nodes][total_cols][64]; status [n_regions] may be NULL. */
int pcsf_node_posteriors(pcsf_engine *e, pcsf_batch *b, int32_t model, const double *rho, int32_t n_nodes,
                         const int32_t *nodes, double *post, int32_t *status);

/* ------------------------------------------------------- allocation-free */

/* Size of the fixed device scratch area behind pcsf_lpr_noalloc. */
#define PCSF_NOALLOC_SCRATCH_BYTES (24u << 20)

/* lpr and elpr of every region under model m at one tree scale rho, without
 * allocating anything.  No counterpart in the reference: it exists for callers
 * that cannot call cudaMalloc when they need a likelihood (a host framework
 * that owns all device memory through its own pool, a latency-critical thread
 * that cannot take cudaMalloc's implicit synchronisation, a process at a hard
 * device-memory cap).  d_leaves ([total_cols][n_leaves], codes as in
 * pcsf_batch_create), d_lpr and d_elpr ([n_regions]; d_elpr may be NULL) are
 * DEVICE pointers owned by the caller; col_offsets is a host array.  The leaf
 * codes are checked on the device first: a code above PCSF_MARGINALIZE, or a
 * NULL d_leaves with columns to read, fails with PCSF_EINVAL.  The values are
 * those pcsf_lpr returns on the same engine (same kernels, summation and P(t)
 * formation); engines made with PCSF_TC_DIRECT are refused with PCSF_EINVAL.
 * Scratch comes from one PCSF_NOALLOC_SCRATCH_BYTES array compiled into the
 * library (held by every GPU that loads it until exit); a batch that does not
 * fit (more than 32768 regions, more than 131072 column tiles, or more than
 * the area) fails with PCSF_ERANGE.  The first call on a device looks up the
 * array's device address, so make it before any stream capture.  Calls share
 * the area: calls that overlap on the GPU, or run concurrently from several
 * host threads, race.  Returns after the results are written. */
int pcsf_lpr_noalloc(pcsf_engine *e, int32_t model, double rho, int32_t n_regions, const int64_t *col_offsets,
                     const uint8_t *d_leaves, double *d_lpr, double *d_elpr);

/* ------------------------------------------------------------ OmegaModel */

/* One region's dN/dS test (OmegaModel.score, src/OmegaModel.ml:195-219). */
typedef struct {
    double score;               /* decibans, 10*(lpr_H1 - lpr_H0)/ln 10           */
    double lpr_h0, lpr_h1;      /* log posterior at the fitted kappa (prior included) */
    double rho_h0, kappa_h0;    /* H0 (omega = sigma = 1) estimates                */
    double rho_h1, kappa_h1;    /* H1 (omega = omega_h1, sigma = sigma_h1)          */
    int32_t status;
    int32_t evals;
} pcsf_omega_result;

/* The OmegaModel test for every region of a batch: F3x4 codon frequencies from
 * the region's leaves (OmegaModel.ml:102-134), then for H0 and H1 three rounds
 * of rho (half-Cauchy prior) and kappa (Gamma prior) maximisation
 * (kr_map, OmegaModel.ml:160-190).  Every kappa change is a new rate matrix,
 * eigendecomposed in FP64 on the GPU; its P(t) is formed in FP64.  The
 * reference defaults are omega_h1 = 0.2, sigma_h1 = 0.01. */
int pcsf_omega_score(pcsf_engine *e, pcsf_batch *b, double omega_h1, double sigma_h1, pcsf_omega_result *out);

/* Gradient of the OmegaModel log-likelihood (priors excluded) of every region
 * at its own kappa[r], omega[r], the common sigma, the F3x4 frequencies of the
 * region's leaves (update_f3x4, OmegaModel.ml:102-134) and tree scale rho[r]:
 * lpr, d lpr / d branch ([n_regions][2*n_leaves-2], may be NULL), d / d rho,
 * d / d kappa, d / d omega (each may be NULL).  The rate-parameter derivatives
 * contract the adjoint pass's weights with dP(t)/dx, the eigenbasis (Frechet)
 * derivative of exp(tQ) -- Q.Diag.dPt_dQ_dx, Q.ml:283-304 -- taken in the
 * symmetric form D^1/2 Q D^-1/2 of the reversible Q; P(t) and Q are formed in
 * FP64, the adjoint runs in the engine's precision.  Replaces the derivative
 * the reference's PhyloEM.d_ell_dQ_dx computes (PhyloEM.ml:76-138). */
int pcsf_omega_grad(pcsf_engine *e, pcsf_batch *b, const double *kappa, const double *omega, double sigma,
                    const double *rho, double *lpr, double *d_branch, double *d_rho, double *d_kappa, double *d_omega,
                    int32_t *status);

#ifdef __cplusplus
}
#endif
#endif /* PHYLOCSF_ENGINE_H */
