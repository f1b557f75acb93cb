/*
 * phylocsf_host.h -- native host-side input helpers of the GB300 PhyloCSF engine.
 *
 * These replace the reference's host-side parsing and packing that feed the
 * likelihood engine (paths relative to the mlin/PhyloCSF source tree).  They
 * run on the CPU and need no GPU.  Errors: a PCSF_* status, message via
 * pcsf_last_error(NULL).
 */
#ifndef PHYLOCSF_HOST_H
#define PHYLOCSF_HOST_H

#include <stdint.h>

#include "phylocsf_engine.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ORF search modes (src/PhyloCSF.ml:15,39) */
#define PCSF_ORF_ASIS 0
#define PCSF_ORF_ATGSTOP 1
#define PCSF_ORF_STOPSTOP 2
#define PCSF_ORF_STOPSTOP3 3
#define PCSF_ORF_TOFIRSTSTOP 4
#define PCSF_ORF_FROMLASTSTOP 5
#define PCSF_ORF_TOORFROMSTOP 6

/* Read an ECM parameter file: S 64x64 (row-major, symmetric, S[0][0]=0) and pi.
 * Replaces ECM.import_parameters (src/ECM.ml:18-72). */
int pcsf_read_ecm(const char *path, double *S, double *pi);

/* Parse a Newick tree into CamlPaml T order (lib/CamlPaml/NewickLexer.mll,
 * NewickParser.mly, T.of_newick T.ml:57-112).  Outputs up to max_nodes nodes:
 * parent[n], branch[n] (NaN where absent), labels[n*label_stride] (each
 * NUL-terminated).  *n_leaves receives the leaf count (n = 2*n_leaves-1). */
int pcsf_parse_newick(const char *text, int32_t max_nodes, int32_t *n_leaves, int32_t *parent, double *branch,
                      char *labels, int32_t label_stride);

/* Candidate regions of an alignment's reference row (candidate_regions and
 * find_orfs, src/PhyloCSF.ml:134-217), in the reference's order.  frames is 1,
 * 3 or 6.  Writes up to cap entries (rc flag, lo, hi; coordinates on the
 * reverse-complemented row when rc is 1) and the total count to *count. */
int pcsf_candidate_regions(const char *ref, int64_t len, int32_t frames, int32_t orf_mode, int32_t min_codons,
                           int32_t cap, int32_t *rc, int64_t *lo, int64_t *hi, int32_t *count);

/* Pack regions of an alignment into the engine's leaf layout (pleaves,
 * src/PhyloCSF.ml:219-246).  rows_fwd / rows_rc: n_rows aligned rows (forward
 * and reverse-complemented) of length len; leaf_rows[l] is the alignment row of
 * tree leaf l or -1 when that species is absent.  Region r uses rows_rc when
 * rc[r] != 0 and covers codons starting at lo[r], lo[r]+3, ... while pos+2 <=
 * hi[r].  col_offsets[n_regions+1] is always written; leaves
 * ([total][n_leaves], PCSF_MARGINALIZE for non-ACGT codons and absent species)
 * only when non-NULL. */
int pcsf_pack_regions(int32_t n_leaves, const int32_t *leaf_rows, int32_t n_rows, const char *const *rows_fwd,
                      const char *const *rows_rc, int64_t len, int32_t n_regions, const int32_t *rc,
                      const int64_t *lo, const int64_t *hi, int64_t *col_offsets, uint8_t *leaves);

/* Per nucleotide column of an alignment, the total branch length of the smallest
 * subtree spanning the species present in that column (not '-', '.' or 'N'),
 * without the root branch: Newick.subtree + Newick.total_length
 * (lib/CamlPaml/Newick.ml:34-61) as the branch length score takes them per column
 * (src/PhyloCSF.ml:252-262).  A branch above node v belongs to it exactly when some
 * but not all of the present species lie below v.  leaf_rows[l]: the row of tree
 * leaf l or -1 when absent; rows: [n_rows] strings of length len; out: [len].
 * The score of columns lo..hi is sum(out[lo..hi]) / (total tree length x (hi-lo+1)). */
int pcsf_bls_columns(int32_t n_leaves, const int32_t *parent, const double *branch, const int32_t *leaf_rows,
                     int32_t n_rows, const char *const *rows, int64_t len, double *out);

/* Simulate codon columns along the tree (PhyloModel.simulate,
 * lib/CamlPaml/PhyloModel.ml:38-54: root ~ prior, each child ~ the P row of its
 * parent's state) for synthetic workloads.  P: [n_models][2*n_leaves-2][64][64]
 * row-major substitution matrices, prior: [n_models][64].  Region r
 * (columns [col_offsets[r], col_offsets[r+1])) is drawn from model
 * region_model[r].  When reject_stop_leaf0 is set a column whose leaf 0 is a
 * stop codon is redrawn (testSim.ml:52-65).  Each leaf codon of region r is
 * then replaced by PCSF_MARGINALIZE with probability gap_frac[r*n_leaves+l]
 * (gap_frac may be NULL).  The random stream is keyed by (seed, column), so the
 * output does not depend on n_threads.  leaves: [total][n_leaves]. */
int pcsf_simulate(int32_t n_leaves, const int32_t *parent, int32_t n_models, const double *P, const double *prior,
                  int32_t n_regions, const int64_t *col_offsets, const int32_t *region_model, const double *gap_frac,
                  int32_t reject_stop_leaf0, uint64_t seed, int32_t n_threads, uint8_t *leaves);

#ifdef __cplusplus
}
#endif
#endif /* PHYLOCSF_HOST_H */
