/*
 * phylocsf_oracle.c -- CPU FP64 restatement of PhyloCSF's likelihood path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle and the timed CPU
 * baseline ("port").  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it; the product library never links or calls it.
 *
 * What it restates (paths are relative to the mlin/PhyloCSF source tree):
 *   - Q assembly and mean-rate scaling ......... src/PhyloCSFModel.ml:11-30,
 *                                                lib/CamlPaml/PhyloModel.ml:76-84,94-106
 *   - eigendecomposition of Q .................. lib/CamlPaml/Q.ml:124-141
 *       (the reference calls GSL's nonsymmetric eigensolver plus a complex LU
 *       inverse; every Q on this path is reversible, so the oracle
 *       diagonalises the symmetric similarity transform D^1/2 Q D^-1/2 with a
 *       cyclic Jacobi method instead.  P(t) is basis-independent.)
 *   - P(t) with the clamp / renormalise rule ... lib/CamlPaml/Q.ml:211-249
 *   - inside pass (dense, leaves included) ..... lib/CamlPaml/PhyloLik.ml:11-19,68-93
 *   - root posterior, lpr / elpr_anc ........... lib/CamlPaml/PhyloLik.ml:127-138,
 *                                                src/PhyloCSFModel.ml:67-82
 *   - outside pass and branch posteriors ....... lib/CamlPaml/PhyloLik.ml:96-120,140-174
 *   - sufficient statistics and ELL ............ lib/CamlPaml/PhyloEM.ml:14-20,22-73
 *   - dP/dt in the eigenbasis .................. lib/CamlPaml/Q.ml:260-275
 *   - find_init ................................ lib/CamlPaml/Fit.ml:27-48
 *   - bounded Brent maximiser .................. lib/CamlPaml/Fit.ml:3-24 (GSL "brent"
 *       fminimizer; restated from Brent 1973 "localmin" with GSL's conventions:
 *       the second/third points start at the golden-section point of the
 *       bracket, tolerance sqrt(DBL_EPSILON)*|x|, no absolute tolerance)
 *   - maximize_lpr, FixedLik / MaxLik LLR ...... src/PhyloCSFModel.ml:84-99,113-146
 *
 * One documented divergence: when find_init has to draw random restarts, the
 * reference uses OCaml's stdlib Random seeded with 0, whose stream depends on
 * the (unpinned) OCaml version.  The oracle draws from SplitMix64 seeded with 0.
 * Regions whose optimum needs restarts are therefore not pinned to the
 * reference's exact iterates.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_OK 0
#define ORC_EARG 1      /* invalid argument                                    */
#define ORC_ENEG 2      /* P(t) entry below -tol           (Q.ml:234-236)      */
#define ORC_EROWSUM 3   /* |row sum - 1| > tol              (Q.ml:243-244)      */
#define ORC_ESCALE 4    /* Q scale evaluated to <= 0        (PhyloModel.ml:98) */
#define ORC_EEIG 5      /* Jacobi sweeps did not converge                      */
#define ORC_EBRACKET 6  /* Brent set-up: endpoints do not enclose a minimum    */
#define ORC_EDIAG 7     /* renormalised diagonal not in (0,1] (Q.ml:245)       */
#define ORC_ENAN 8      /* objective produced NaN                              */

typedef struct {
    int nl;               /* leaves; node ids 0..nl-1 are leaves (T.ml:57-112)     */
    int n;                /* nodes = 2*nl-1; root = n-1; internal ids post-ordered */
    const int *lchild;    /* [n]; -1 for leaves                                    */
    const int *rchild;    /* [n]; -1 for leaves                                    */
    const int *parent;    /* [n]; -1 for the root                                  */
    const double *branch; /* [n-1]; length of the branch leading into node i       */
} orc_tree;

typedef struct {
    int k;              /* state count (64 for codons)                              */
    const double *U;    /* [k*k] row-major; column m = m-th eigenvector of D^1/2QD^-1/2 */
    const double *lam;  /* [k] eigenvalues                                          */
    const double *pi;   /* [k] equilibrium distribution used for the similarity     */
    const double *prior;/* [k] root prior (PhyloCSF passes pi explicitly)          */
    double tol;         /* Q.Diag tol (1e-6 by default, Q.ml:124)                  */
} orc_model;

typedef struct {
    double score;   /* decibans: 10*(lpr_c - lpr_n)/ln 10       */
    double anc;     /* decibans: 10*(elpr_c - elpr_n)/ln 10     */
    double rho_c, rho_n;
    double lpr_c, lpr_n;
    double elpr_c, elpr_n;
    int status;
    int evals;      /* likelihood evaluations (both models)     */
} orc_result;

/* ------------------------------------------------------------------------ */
/* Q assembly: q_ij = s_ij * pi_j (i != j), q_ii = -sum_{j!=i} q_ij, then
 * divide every entry by scale = -sum_i pi_i q_ii.  The summation orders follow
 * the expression trees built in PhyloCSFModel.ml:11-30 / PhyloModel.ml:76-84
 * (ascending j, then ascending i), so the result is bit-identical to the
 * reference's Expr.eval. */
int orc_build_q(int k, const double *S, const double *pi, double *Q)
{
    if (k < 2 || !S || !pi || !Q) return ORC_EARG;
    double *tot = (double *)malloc(sizeof(double) * k);
    for (int i = 0; i < k; i++) {
        double t = 0.0;
        for (int j = 0; j < k; j++) {
            double q = (i == j) ? 0.0 : S[i * k + j] * pi[j];
            Q[i * k + j] = q;
            if (i != j) t = q + t;
        }
        tot[i] = t;
        Q[i * k + i] = 0.0 - t;
    }
    double scale = 0.0;
    for (int i = 0; i < k; i++)
        if (Q[i * k + i] != 0.0) scale = scale - pi[i] * Q[i * k + i];
    free(tot);
    if (!(scale > 0.0)) return ORC_ESCALE;
    for (int i = 0; i < k * k; i++) Q[i] = Q[i] / scale;
    return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* Eigendecomposition of a reversible Q with stationary pi:
 *   A = D^1/2 Q D^-1/2 is symmetric; A = U diag(lam) U^T (cyclic Jacobi).
 *   Then Q = S diag(lam) S^-1 with S = D^-1/2 U, S^-1 = U^T D^1/2. */
int orc_eigen_reversible(int k, const double *Q, const double *pi, double *U, double *lam)
{
    if (k < 2 || !Q || !pi || !U || !lam) return ORC_EARG;
    double *A = (double *)malloc(sizeof(double) * k * k);
    double *sq = (double *)malloc(sizeof(double) * k);
    for (int i = 0; i < k; i++) {
        if (!(pi[i] > 0.0)) { free(A); free(sq); return ORC_EARG; }
        sq[i] = sqrt(pi[i]);
    }
    for (int i = 0; i < k; i++)
        for (int j = 0; j < k; j++) {
            double aij = sq[i] * Q[i * k + j] / sq[j];
            double aji = sq[j] * Q[j * k + i] / sq[i];
            A[i * k + j] = 0.5 * (aij + aji);
        }
    for (int i = 0; i < k * k; i++) U[i] = 0.0;
    for (int i = 0; i < k; i++) U[i * k + i] = 1.0;

    double norm2 = 0.0;
    for (int i = 0; i < k * k; i++) norm2 += A[i] * A[i];
    int converged = 0;
    for (int sweep = 0; sweep < 100 && !converged; sweep++) {
        double off = 0.0;
        for (int p = 0; p < k; p++)
            for (int q = p + 1; q < k; q++) off += A[p * k + q] * A[p * k + q];
        if (off <= 1e-32 * norm2) { converged = 1; break; }
        for (int p = 0; p < k - 1; p++) {
            for (int q = p + 1; q < k; q++) {
                double apq = A[p * k + q];
                if (apq == 0.0) continue;
                double app = A[p * k + p], aqq = A[q * k + q];
                /* rotation angle that annihilates A[p][q] */
                double theta = (aqq - app) / (2.0 * apq);
                double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int r = 0; r < k; r++) {
                    double arp = A[r * k + p], arq = A[r * k + q];
                    A[r * k + p] = c * arp - s * arq;
                    A[r * k + q] = s * arp + c * arq;
                }
                for (int r = 0; r < k; r++) {
                    double apr = A[p * k + r], aqr = A[q * k + r];
                    A[p * k + r] = c * apr - s * aqr;
                    A[q * k + r] = s * apr + c * aqr;
                }
                A[p * k + q] = A[q * k + p] = 0.0;
                for (int r = 0; r < k; r++) {
                    double urp = U[r * k + p], urq = U[r * k + q];
                    U[r * k + p] = c * urp - s * urq;
                    U[r * k + q] = s * urp + c * urq;
                }
            }
        }
    }
    for (int i = 0; i < k; i++) lam[i] = A[i * k + i];
    free(A);
    free(sq);
    return converged ? ORC_OK : ORC_EEIG;
}

/* ------------------------------------------------------------------------ */
/* P(t) = D^-1/2 U diag(exp(lam t)) U^T D^1/2, followed by the row rule of
 * Q.ml:226-247: the raw row sum (taken before clamping) must be within tol of 1,
 * negatives within tol become 0 (below -tol is an error), and the diagonal is
 * replaced by 1 - sum of the (clamped) off-diagonal entries. */
int orc_pt(const orc_model *m, double t, double *P)
{
    int k = m->k;
    if (t < 0.0) return ORC_EARG;
    double *e = (double *)malloc(sizeof(double) * k);
    double *sq = (double *)malloc(sizeof(double) * k);
    for (int c = 0; c < k; c++) e[c] = exp(t * m->lam[c]);
    for (int i = 0; i < k; i++) sq[i] = sqrt(m->pi[i]);
    for (int i = 0; i < k; i++)
        for (int j = 0; j < k; j++) {
            double acc = 0.0;
            for (int c = 0; c < k; c++) acc += m->U[i * k + c] * e[c] * m->U[j * k + c];
            P[i * k + j] = acc * sq[j] / sq[i];
        }
    free(e);
    free(sq);
    for (int i = 0; i < k; i++) {
        double tot = 0.0, diag = 1.0;
        for (int j = 0; j < k; j++) {
            double x = P[i * k + j];
            tot += x;
            if (x < 0.0) {
                if (fabs(x) > m->tol) return ORC_ENEG;
                P[i * k + j] = 0.0;
            }
            if (i != j) diag -= P[i * k + j];
        }
        if (fabs(tot - 1.0) > m->tol) return ORC_EROWSUM;
        if (!(diag <= 1.0 && diag > 0.0)) return ORC_EDIAG;
        P[i * k + i] = diag;
    }
    return ORC_OK;
}

/* dP/dt = D^-1/2 U diag(lam exp(lam t)) U^T D^1/2 (Q.ml:260-275 in the real basis). */
int orc_dpt_dt(const orc_model *m, double t, double *dP)
{
    int k = m->k;
    for (int i = 0; i < k; i++)
        for (int j = 0; j < k; j++) {
            double acc = 0.0;
            for (int c = 0; c < k; c++)
                acc += m->U[i * k + c] * m->lam[c] * exp(t * m->lam[c]) * m->U[j * k + c];
            dP[i * k + j] = acc * sqrt(m->pi[j]) / sqrt(m->pi[i]);
        }
    return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* Inside pass for one column, dense on every branch as PhyloLik.ensure_alpha
 * does (leaves are one-hot or all-ones vectors, PhyloLik.ml:11-19).
 *   leaves[i] in [0,k) = Certain, < 0 = Marginalize.
 *   alpha: workspace [n*k]; rows 0..nl-1 hold the leaf vectors.
 * Returns z = alpha_root . prior; fills post_root (k) when non-NULL
 * (node_posterior at the root, PhyloLik.ml:127-138). */
static int g_sparse_leaves = 0;

/* When set, leaf branches are evaluated as gathers (Certain) and sequential row
 * sums (Marginalize) instead of dense dots.  Adding exact zeros does not change
 * a floating-point sum, so the result is bit-identical to the dense loop; the
 * switch only makes the test suite faster.  The timed CPU baseline keeps the
 * dense loop of the reference. */
void orc_set_sparse_leaves(int on) { g_sparse_leaves = on; }

static double leaf_dot(int k, const double *prow, int s)
{
    if (s >= 0) return prow[s];
    double d = 0.0;
    for (int b = 0; b < k; b++) d += prow[b];
    return d;
}

static double column_inside(int k, const orc_tree *tr, const double *const *Ps, const double *prior,
                            const int *leaves, double *alpha, double *post_root)
{
    int nl = tr->nl, n = tr->n;
    for (int i = 0; i < nl; i++) {
        double *a = alpha + (size_t)i * k;
        int s = leaves[i];
        for (int x = 0; x < k; x++) a[x] = (s < 0) ? 1.0 : (x == s ? 1.0 : 0.0);
    }
    for (int i = nl; i < n; i++) {
        int lc = tr->lchild[i], rc = tr->rchild[i];
        const double *pl = Ps[lc], *pr = Ps[rc];
        const double *al = alpha + (size_t)lc * k, *ar = alpha + (size_t)rc * k;
        double *ai = alpha + (size_t)i * k;
        for (int a = 0; a < k; a++) {
            double dl = 0.0, dr = 0.0;
            if (g_sparse_leaves && lc < nl) dl = leaf_dot(k, pl + a * k, leaves[lc]);
            else for (int b = 0; b < k; b++) dl += pl[a * k + b] * al[b];
            if (g_sparse_leaves && rc < nl) dr = leaf_dot(k, pr + a * k, leaves[rc]);
            else for (int b = 0; b < k; b++) dr += pr[a * k + b] * ar[b];
            ai[a] = dl * dr;
        }
    }
    const double *ar = alpha + (size_t)(n - 1) * k;
    double z = 0.0;
    for (int a = 0; a < k; a++) z += ar[a] * prior[a];
    if (post_root) {
        for (int a = 0; a < k; a++) post_root[a] = (z == 0.0) ? 0.0 : ar[a] * prior[a] / z;
    }
    return z;
}

/* Likelihood of one column given explicit P matrices ([n-1][k*k], branch i
 * into node i).  Exposed for the 2-state known-answer test of PhyloLik. */
double orc_column_likelihood(int k, const orc_tree *tr, const double *Pflat, const double *prior,
                             const int *leaves, double *post_root)
{
    const double **Ps = (const double **)malloc(sizeof(double *) * (tr->n - 1));
    for (int i = 0; i < tr->n - 1; i++) Ps[i] = Pflat + (size_t)i * k * k;
    double *alpha = (double *)malloc(sizeof(double) * (size_t)tr->n * k);
    double z = column_inside(k, tr, Ps, prior, leaves, alpha, post_root);
    free(alpha);
    free((void *)Ps);
    return z;
}

/* Outside pass (PhyloLik.ml:96-120) and node posteriors for every node
 * (PhyloLik.ml:127-138).  post: [n*k]. */
double orc_column_posteriors(int k, const orc_tree *tr, const double *Pflat, const double *prior,
                             const int *leaves, double *post)
{
    int n = tr->n, nl = tr->nl;
    const double **Ps = (const double **)malloc(sizeof(double *) * (n - 1));
    for (int i = 0; i < n - 1; i++) Ps[i] = Pflat + (size_t)i * k * k;
    double *alpha = (double *)malloc(sizeof(double) * (size_t)n * k);
    double *beta = (double *)malloc(sizeof(double) * (size_t)n * k);
    double *inter = (double *)malloc(sizeof(double) * k);
    double z = column_inside(k, tr, Ps, prior, leaves, alpha, NULL);
    for (int a = 0; a < k; a++) beta[(size_t)(n - 1) * k + a] = prior[a];
    for (int i = n - 2; i >= 0; i--) {
        int p = tr->parent[i];
        int s = (tr->lchild[p] == i) ? tr->rchild[p] : tr->lchild[p];
        const double *ps = Ps[s], *pi_ = Ps[i];
        for (int a = 0; a < k; a++) {
            double d = 0.0;
            for (int b = 0; b < k; b++) d += ps[a * k + b] * alpha[(size_t)s * k + b];
            inter[a] = beta[(size_t)p * k + a] * d;
        }
        for (int b = 0; b < k; b++) {
            double acc = 0.0;
            for (int a = 0; a < k; a++) acc += inter[a] * pi_[a * k + b];
            beta[(size_t)i * k + b] = acc;
        }
    }
    for (int i = 0; i < n; i++)
        for (int a = 0; a < k; a++)
            post[(size_t)i * k + a] = (z == 0.0) ? 0.0
                                    : (i < nl ? alpha[(size_t)i * k + a]
                                              : alpha[(size_t)i * k + a] * beta[(size_t)i * k + a] / z);
    free(alpha);
    free(beta);
    free(inter);
    free((void *)Ps);
    return z;
}

/* ------------------------------------------------------------------------ */
/* lpr_leaves (PhyloCSFModel.ml:67-82): P(rho*b_i) for every branch, then the
 * inside pass per column; lpr = sum log z, elpr = sum_col post_root . log(prior).
 * leaves: [ncols*nl] column-major by column (one column = nl leaf states). */
int orc_lpr_leaves(const orc_model *m, const orc_tree *tr, double rho, int ncols, const int *leaves,
                   double *lpr_out, double *elpr_out)
{
    int k = m->k, n = tr->n, nl = tr->nl;
    if (!(rho > 0.0)) return ORC_EARG;
    double *Pflat = (double *)malloc(sizeof(double) * (size_t)(n - 1) * k * k);
    const double **Ps = (const double **)malloc(sizeof(double *) * (n - 1));
    int st = ORC_OK;
    for (int i = 0; i < n - 1 && st == ORC_OK; i++) {
        Ps[i] = Pflat + (size_t)i * k * k;
        st = orc_pt(m, rho * tr->branch[i], Pflat + (size_t)i * k * k);
    }
    if (st != ORC_OK) { free(Pflat); free((void *)Ps); return st; }
    double *alpha = (double *)malloc(sizeof(double) * (size_t)n * k);
    double *post = (double *)malloc(sizeof(double) * k);
    double *lp = (double *)malloc(sizeof(double) * k);
    for (int a = 0; a < k; a++) lp[a] = log(m->prior[a]);
    double lpr = 0.0, elpr = 0.0;
    for (int c = 0; c < ncols; c++) {
        double z = column_inside(k, tr, Ps, m->prior, leaves + (size_t)c * nl, alpha, post);
        lpr = lpr + log(z);
        double d = 0.0;
        for (int a = 0; a < k; a++) d += post[a] * lp[a];
        elpr = elpr + d;
    }
    free(alpha);
    free(post);
    free(lp);
    free(Pflat);
    free((void *)Ps);
    *lpr_out = lpr;
    if (elpr_out) *elpr_out = elpr;
    return ORC_OK;
}

/* Gradient of lpr with respect to every branch length t_i = rho*b_i, by the
 * outside pass and branch posteriors (PhyloLik.ml:96-174) contracted with
 * dP/dt (Q.ml:260-275): d lpr / d t_i = sum_col sum_ab inter_a alpha_i[b] dP_i[a,b]/dt / z.
 * grad: [n-1].  d lpr / d rho = sum_i b_i grad[i]. */
int orc_grad_branches(const orc_model *m, const orc_tree *tr, double rho, int ncols, const int *leaves,
                      double *lpr_out, double *grad)
{
    int k = m->k, n = tr->n, nl = tr->nl;
    double *Pflat = (double *)malloc(sizeof(double) * (size_t)(n - 1) * k * k);
    double *dP = (double *)malloc(sizeof(double) * (size_t)(n - 1) * k * k);
    const double **Ps = (const double **)malloc(sizeof(double *) * (n - 1));
    int st = ORC_OK;
    for (int i = 0; i < n - 1 && st == ORC_OK; i++) {
        Ps[i] = Pflat + (size_t)i * k * k;
        st = orc_pt(m, rho * tr->branch[i], Pflat + (size_t)i * k * k);
        if (st == ORC_OK) st = orc_dpt_dt(m, rho * tr->branch[i], dP + (size_t)i * k * k);
    }
    if (st != ORC_OK) { free(Pflat); free(dP); free((void *)Ps); return st; }
    double *alpha = (double *)malloc(sizeof(double) * (size_t)n * k);
    double *beta = (double *)malloc(sizeof(double) * (size_t)n * k);
    double *inter = (double *)malloc(sizeof(double) * k);
    for (int i = 0; i < n - 1; i++) grad[i] = 0.0;
    double lpr = 0.0;
    for (int c = 0; c < ncols; c++) {
        const int *lv = leaves + (size_t)c * nl;
        double z = column_inside(k, tr, Ps, m->prior, lv, alpha, NULL);
        lpr += log(z);
        for (int a = 0; a < k; a++) beta[(size_t)(n - 1) * k + a] = m->prior[a];
        for (int i = n - 2; i >= 0; i--) {
            int p = tr->parent[i];
            int s = (tr->lchild[p] == i) ? tr->rchild[p] : tr->lchild[p];
            const double *ps = Ps[s], *pi_ = Ps[i], *dpi = dP + (size_t)i * k * k;
            for (int a = 0; a < k; a++) {
                double d = 0.0;
                for (int b = 0; b < k; b++) d += ps[a * k + b] * alpha[(size_t)s * k + b];
                inter[a] = beta[(size_t)p * k + a] * d;
            }
            double g = 0.0;
            for (int b = 0; b < k; b++) {
                double acc = 0.0, dacc = 0.0;
                for (int a = 0; a < k; a++) {
                    acc += inter[a] * pi_[a * k + b];
                    dacc += inter[a] * dpi[a * k + b];
                }
                beta[(size_t)i * k + b] = acc;
                g += dacc * alpha[(size_t)i * k + b];
            }
            grad[i] += g / z;
        }
    }
    free(alpha);
    free(beta);
    free(inter);
    free(Pflat);
    free(dP);
    free((void *)Ps);
    *lpr_out = lpr;
    return ORC_OK;
}

/* Expected substitution counts of every branch summed over the columns of a
 * region: add_branch_posteriors (PhyloLik.ml:140-174) per column and branch, as
 * PhyloEM.collect_sufficient_statistics accumulates them (PhyloEM.ml:14-20):
 *   counts[i][a][b] += beta_p[a] (P_s alpha_s)[a] P_i[a][b] alpha_i[b] / z
 * (rows with beta_p[a] = 0 skipped, columns with z = 0 add nothing).
 * counts: [n-1][k][k], zeroed here.  lpr_out: sum of log z. */
int orc_branch_counts(const orc_model *m, const orc_tree *tr, double rho, int ncols, const int *leaves,
                      double *lpr_out, double *counts)
{
    int k = m->k, n = tr->n, nl = tr->nl;
    double *Pflat = (double *)malloc(sizeof(double) * (size_t)(n - 1) * k * k);
    const double **Ps = (const double **)malloc(sizeof(double *) * (n - 1));
    int st = ORC_OK;
    for (int i = 0; i < n - 1 && st == ORC_OK; i++) {
        Ps[i] = Pflat + (size_t)i * k * k;
        st = orc_pt(m, rho * tr->branch[i], Pflat + (size_t)i * k * k);
    }
    if (st != ORC_OK) { free(Pflat); free((void *)Ps); return st; }
    double *alpha = (double *)malloc(sizeof(double) * (size_t)n * k);
    double *beta = (double *)malloc(sizeof(double) * (size_t)n * k);
    double *inter = (double *)malloc(sizeof(double) * k);
    memset(counts, 0, sizeof(double) * (size_t)(n - 1) * k * k);
    double lpr = 0.0;
    for (int c = 0; c < ncols; c++) {
        const int *lv = leaves + (size_t)c * nl;
        double z = column_inside(k, tr, Ps, m->prior, lv, alpha, NULL);
        lpr += log(z);
        if (!(z > 0.0)) continue;
        for (int a = 0; a < k; a++) beta[(size_t)(n - 1) * k + a] = m->prior[a];
        for (int i = n - 2; i >= 0; i--) {
            int p = tr->parent[i];
            int s = (tr->lchild[p] == i) ? tr->rchild[p] : tr->lchild[p];
            const double *ps = Ps[s], *pi_ = Ps[i];
            for (int a = 0; a < k; a++) {
                double d = 0.0;
                for (int b = 0; b < k; b++) d += ps[a * k + b] * alpha[(size_t)s * k + b];
                inter[a] = beta[(size_t)p * k + a] * d;
            }
            for (int b = 0; b < k; b++) {
                double acc = 0.0;
                for (int a = 0; a < k; a++) acc += inter[a] * pi_[a * k + b];
                beta[(size_t)i * k + b] = acc;
            }
            double *ci = counts + (size_t)i * k * k;
            for (int a = 0; a < k; a++) {
                if (!(inter[a] > 0.0)) continue;
                for (int b = 0; b < k; b++) ci[a * k + b] += inter[a] * pi_[a * k + b] * alpha[(size_t)i * k + b] / z;
            }
        }
    }
    free(alpha);
    free(beta);
    free(inter);
    free(Pflat);
    free((void *)Ps);
    *lpr_out = lpr;
    return ORC_OK;
}

/* Expected log-likelihood of sufficient statistics (PhyloEM.ell, PhyloEM.ml:22-73):
 * branches_ell = sum_i sum_{ab: counts > 0} counts[i][a][b] log P_i[a][b] at t_i = rho b_i,
 * prior_ell = sum_a (sum_b counts[lc][a][b]) log prior[a] (lc = the root's left child,
 * terms with a positive row sum). */
int orc_ell(const orc_model *m, const orc_tree *tr, double rho, const double *counts, double *ell_out)
{
    int k = m->k, n = tr->n;
    double *P = (double *)malloc(sizeof(double) * (size_t)k * k);
    double tot = 0.0;
    int st = ORC_OK;
    for (int i = 0; i < n - 1 && st == ORC_OK; i++) {
        st = orc_pt(m, rho * tr->branch[i], P);
        const double *ci = counts + (size_t)i * k * k;
        for (int a = 0; a < k && st == ORC_OK; a++)
            for (int b = 0; b < k; b++)
                if (ci[a * k + b] > 0.0) tot += ci[a * k + b] * log(P[a * k + b]);
    }
    free(P);
    if (st != ORC_OK) return st;
    const double *cl = counts + (size_t)tr->lchild[n - 1] * k * k;
    for (int a = 0; a < k; a++) {
        double r = 0.0;
        for (int b = 0; b < k; b++) r += cl[a * k + b];
        if (r > 0.0) tot += r * log(m->prior[a]);
    }
    *ell_out = tot;
    return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* SplitMix64: the oracle's stand-in for OCaml's Random in find_init. */
static uint64_t splitmix64(uint64_t *s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
static double uniform01(uint64_t *s) { return (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }

typedef struct {
    const orc_model *m;
    const orc_tree *tr;
    int ncols;
    const int *leaves;
    int evals;
    int status;
    double last_elpr;
} objective_ctx;

/* the objective: lpr at rho (NaN and a status on failure) */
static double objective(objective_ctx *c, double rho)
{
    double lpr = NAN, elpr = NAN;
    int st = orc_lpr_leaves(c->m, c->tr, rho, c->ncols, c->leaves, &lpr, &elpr);
    c->evals++;
    if (st != ORC_OK) {
        if (c->status == ORC_OK) c->status = st;
        return NAN;
    }
    c->last_elpr = elpr;
    return lpr;
}

/* Bounded minimiser state: bracket [lo,hi], best point x, second-best w,
 * previous second-best v, and the two remembered step lengths. */
typedef struct {
    double lo, hi, flo, fhi;
    double x, fx, w, fw, v, fv;
    double d_keep, e_keep;
} orc_brent;

#define ORC_GOLDEN 0.3819660
#define ORC_SQRT_EPS 1.4901161193847656e-08

/* Next trial abscissa: a parabolic step through (x,w,v) when it is well
 * inside the bracket and shorter than half the remembered step, otherwise a
 * golden-section step into the larger side.  GSL keeps the two remembered
 * steps in swapped slots from one iteration to the next; that is reproduced
 * because it changes which step length gates the parabola. */
static double brent_propose(orc_brent *b)
{
    double z = b->x, fz = b->fx;
    double d = b->e_keep, e = b->d_keep;
    double tol = ORC_SQRT_EPS * fabs(z);
    double mid = 0.5 * (b->lo + b->hi);
    double left = z - b->lo, right = b->hi - z;
    double p = 0.0, q = 0.0, r = 0.0;
    if (fabs(e) > tol) {
        r = (z - b->w) * (fz - b->fv);
        q = (z - b->v) * (fz - b->fw);
        p = (z - b->v) * q - (z - b->w) * r;
        q = 2.0 * (q - r);
        if (q > 0.0) p = -p; else q = -q;
        r = e;
        e = d;
    }
    if (fabs(p) < fabs(0.5 * q * r) && p < q * left && p < q * right) {
        d = p / q;
        double u = z + d;
        if ((u - b->lo) < 2.0 * tol || (b->hi - u) < 2.0 * tol) d = (z < mid) ? tol : -tol;
    } else {
        e = (z < mid) ? (b->hi - z) : -(z - b->lo);
        d = ORC_GOLDEN * e;
    }
    double u = (fabs(d) >= tol) ? z + d : z + ((d > 0.0) ? tol : -tol);
    b->e_keep = e;
    b->d_keep = d;
    return u;
}

static void brent_accept(orc_brent *b, double u, double fu)
{
    if (fu <= b->fx) {
        if (u < b->x) { b->hi = b->x; b->fhi = b->fx; }
        else { b->lo = b->x; b->flo = b->fx; }
        b->v = b->w; b->fv = b->fw;
        b->w = b->x; b->fw = b->fx;
        b->x = u; b->fx = fu;
    } else {
        if (u < b->x) { b->lo = u; b->flo = fu; }
        else { b->hi = u; b->fhi = fu; }
        if (fu <= b->fw || b->w == b->x) {
            b->v = b->w; b->fv = b->fw;
            b->w = u; b->fw = fu;
        } else if (fu <= b->fv || b->v == b->x || b->v == b->w) {
            b->v = u; b->fv = fu;
        }
    }
}

/* Fit.find_init with logspace=true (Fit.ml:27-48). */
static double find_init(objective_ctx *c, double init, double lo, double hi, int maxtries)
{
    double width = log(hi) - log(lo);
    double flo = objective(c, lo);
    double fhi = objective(c, hi);
    double x = init;
    double fx = objective(c, init);
    int i = 0;
    uint64_t seed = 0;
    while (i < maxtries && (fx <= flo || fx <= fhi)) {
        x = exp(log(lo) + uniform01(&seed) * width);
        fx = objective(c, x);
        i++;
    }
    if (i == maxtries) x = (flo > fhi) ? lo : hi;
    return x;
}

/* maximize_lpr (PhyloCSFModel.ml:84-99) over rho in [lo,hi].  Returns the
 * maximiser in *rho and f(rho) in *lpr / *elpr. */
static int maximize_lpr(objective_ctx *c, double init, double lo, double hi, double accuracy,
                        double *rho, double *lpr, double *elpr)
{
    double good = find_init(c, init, lo, hi, 250);
    if (c->status != ORC_OK) return c->status;
    double x = good;
    if (lo < good && good < hi) {
        orc_brent b;
        /* fminimizer_set: the minimised function is -lpr */
        b.flo = -objective(c, lo);
        b.fhi = -objective(c, hi);
        b.fx = -objective(c, good);
        if (c->status != ORC_OK) return c->status;
        b.lo = lo; b.hi = hi; b.x = good;
        if (!(b.fx < b.flo && b.fx < b.fhi)) return ORC_EBRACKET;
        b.v = b.w = lo + ORC_GOLDEN * (hi - lo);
        b.fv = b.fw = -objective(c, b.v);
        b.d_keep = b.e_keep = 0.0;
        if (c->status != ORC_OK) return c->status;
        for (int it = 0; it < 1000; it++) {
            double u = brent_propose(&b);
            double fu = -objective(c, u);
            if (c->status != ORC_OK) return c->status;
            brent_accept(&b, u, fu);
            if (!((b.hi - b.lo) / b.x > accuracy)) break;
        }
        x = b.x;
    }
    double f = objective(c, x);
    if (c->status != ORC_OK) return c->status;
    *rho = x;
    *lpr = f;
    *elpr = c->last_elpr;
    return ORC_OK;
}

static double decibans(double x) { return 10.0 * x / log(10.0); }

/* PhyloCSFModel.score (PhyloCSFModel.ml:113-146).  strategy 0 = FixedLik (rho=1),
 * 1 = MaxLik (rho in [0.01,10], init 1, accuracy 0.01). */
int orc_score_region(const orc_model *mc, const orc_model *mn, const orc_tree *tr, int strategy, int ncols,
                     const int *leaves, orc_result *out)
{
    memset(out, 0, sizeof(*out));
    objective_ctx cc = {mc, tr, ncols, leaves, 0, ORC_OK, NAN};
    objective_ctx cn = {mn, tr, ncols, leaves, 0, ORC_OK, NAN};
    int st;
    if (strategy == 0) {
        out->rho_c = out->rho_n = 1.0;
        st = orc_lpr_leaves(mc, tr, 1.0, ncols, leaves, &out->lpr_c, &out->elpr_c);
        if (st == ORC_OK) st = orc_lpr_leaves(mn, tr, 1.0, ncols, leaves, &out->lpr_n, &out->elpr_n);
        cc.evals = 1;
        cn.evals = 1;
    } else {
        st = maximize_lpr(&cc, 1.0, 1e-2, 10.0, 0.01, &out->rho_c, &out->lpr_c, &out->elpr_c);
        if (st == ORC_OK) st = maximize_lpr(&cn, 1.0, 1e-2, 10.0, 0.01, &out->rho_n, &out->lpr_n, &out->elpr_n);
    }
    out->status = st;
    out->evals = cc.evals + cn.evals;
    out->score = decibans(out->lpr_c - out->lpr_n);
    out->anc = decibans(out->elpr_c - out->elpr_n);
    return st;
}

/* Score many regions; regions are independent. */
int orc_score_batch(const orc_model *mc, const orc_model *mn, const orc_tree *tr, int strategy, int nregions,
                    const int64_t *col_offsets, const int *leaves, orc_result *out)
{
    int worst = ORC_OK;
    for (int r = 0; r < nregions; r++) {
        int64_t c0 = col_offsets[r], c1 = col_offsets[r + 1];
        int st = orc_score_region(mc, mn, tr, strategy, (int)(c1 - c0), leaves + (size_t)c0 * tr->nl, out + r);
        if (st != ORC_OK) worst = st;
    }
    return worst;
}
