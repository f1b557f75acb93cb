"""The CPU oracle against the reference's own known answers (no GPU).

Pins (paths relative to the mlin/PhyloCSF tree, read into tests/golden by
make_fixtures.py):
  - PhyloLik 2-state known-answer cases ........ lib/CamlPaml/test.ml:8-54
  - BEAGLE TinyTest JC69 log-likelihood ........ lib/CamlPaml/test.ml:56-99
  - end-to-end PhyloCSF scores ................. src/test.ml:27-59
"""
import math

import numpy as np
import pytest

from oracle import oracle as O
from tests import helpers as H


@pytest.fixture(autouse=True, scope="module")
def _sparse():
    O.set_sparse_leaves(True)     # bit-identical to the dense loop, faster
    yield
    O.set_sparse_leaves(False)


# ---------------------------------------------------------------- 2-state
SM0 = np.array([[0.8, 0.2], [0.25, 0.75]])
SM1 = np.array([[0.9, 0.1], [0.85, 0.15]])
PRIOR2 = np.array([0.6, 0.4])


@pytest.mark.parametrize("lvs", [(a, b, c) for a in (0, 1) for b in (0, 1) for c in (0, 1)])
def test_phylolik_two_state(lvs):
    # "(A,(B,C))": leaves 0,1,2; node 3 = (B,C); root 4.  P matrices as test.ml:12-16
    tree = O.tree_of_newick(O.parse_newick("(A,(B,C))"))
    Ps = np.stack([SM0, SM1, SM1, SM1])
    alf = [np.array([1.0 if lvs[i] == s else 0.0 for s in (0, 1)]) for i in range(3)]
    a3 = (SM1 @ alf[1]) * (SM1 @ alf[2])
    a4 = (SM0 @ alf[0]) * (SM1 @ a3)
    z = PRIOR2 @ a4
    zo, post_root = O.column_likelihood(tree, Ps, PRIOR2, list(lvs))
    assert zo == pytest.approx(z, abs=1e-3)
    assert np.allclose(post_root, PRIOR2 * a4 / z, atol=1e-3)
    b3 = ((PRIOR2 * (SM0 @ alf[0])) @ SM1)
    zp, post = O.column_posteriors(tree, Ps, PRIOR2, list(lvs))
    assert np.allclose(post[4], PRIOR2 * a4 / z, atol=1e-3)
    assert np.allclose(post[3], b3 * a3 / z, atol=1e-3)
    # posteriors are distributions
    assert post[3].sum() == pytest.approx(1.0, abs=1e-12)


# ---------------------------------------------------------------- BEAGLE
def _beagle_leaves(b, tree):
    seqs = b["seqs"]
    order = [seqs[tree.labels[i]] for i in range(tree.nl)]
    L = len(order[0])
    return np.array([["ACGT".index(s[i]) if s[i] in "ACGT" else -1 for s in order] for i in range(L)], np.int32)


def test_beagle_tinytest():
    b = H.beagle()
    tree = O.tree_of_newick(O.parse_newick(b["tree"]))
    Q = np.full((4, 4), 1.0)
    np.fill_diagonal(Q, -3.0)
    Q /= 3.0                                  # Q.Diag.scale (of_Q JC) (1/3), test.ml:64-70
    m = O.OModel(Q, np.full(4, 0.25))
    lpr, _ = O.lpr_leaves(m, O.OTree(tree), 1.0, _beagle_leaves(b, tree))
    assert abs(lpr - b["logL"]) <= b["eps"]
    # reversible, equilibrium 1/4 each (test.ml:72-73)
    assert np.allclose(np.sort(m.lam)[-1], 0.0, atol=1e-12)


# ---------------------------------------------------------------- end-to-end
def _oracle_run(params, fa, flags, strategy=O.MLE, regions=None):
    mc, mn, ot, tree = H.oracle_models(params)
    ex = H.examples()[fa]
    f = H.parse_flags(flags)
    sp, aln = ex["species"], ex["rows"]
    if f["remove_ref_gaps"]:
        aln = O.remove_ref_gaps(aln)
    aln = [s.replace("u", "t").replace("U", "T") for s in aln]
    rc = [O.revcomp(s) for s in aln]
    rows = O.leaf_rows_for(tree, sp)
    regs = regions if regions is not None else O.candidate_regions(aln[0], f["frames"], f["orf"])
    out = []
    for (isrc, lo, hi) in regs:
        r = O.score_region(mc, mn, ot, strategy, O.pleaves(rc if isrc else aln, rows, lo, hi))
        assert r.status == 0
        out.append((r.score, r.anc, isrc, lo, hi))
    return out, regs


@pytest.mark.parametrize("idx", [0, 1])
def test_pinned_scores_mle(idx):
    p = H.pins()[idx]
    out, _ = _oracle_run(p["params"], p["file"], p["flags"])
    (score, anc, _, _, _), = out
    (s_lo, s_hi), (a_lo, a_hi) = p["windows"]
    assert s_lo < score < s_hi
    assert a_lo < anc < a_hi


def test_pinned_six_frames():
    p = H.pins()[2]
    out, _ = _oracle_run(p["params"], p["file"], p["flags"])
    best = max(out)
    (s_lo, s_hi), = p["windows"]
    assert s_lo < best[0] < s_hi
    assert [best[3], best[4]] == p["ints"]
    assert (not best[2]) == (p["strand"] == "+")


def test_pinned_mrna_orf_region():
    """ATGStop / 3 frames / removeRefGaps: the pinned region is a candidate and scores in its window.
    (Scoring every candidate region is left to the GPU test; the oracle scores the pinned one.)"""
    p = H.pins()[3]
    f = H.parse_flags(p["flags"])
    ex = H.examples()[p["file"]]
    aln = O.remove_ref_gaps(ex["rows"])
    regs = O.candidate_regions(aln[0], f["frames"], f["orf"])
    lo, hi = p["ints"]
    assert (False, lo, hi) in regs
    out, _ = _oracle_run(p["params"], p["file"], p["flags"], regions=[(False, lo, hi)])
    (s_lo, s_hi), = p["windows"]
    assert s_lo < out[0][0] < s_hi


def test_oracle_fixed_scores_stable():
    """Fixed-strategy (rho = 1) oracle values recorded in the fixtures."""
    for fa, rec in H.oracle_fixed().items():
        mc, mn, ot, tree = H.oracle_models(rec["params"])
        ex = H.examples()[fa]
        lv = O.pleaves(ex["rows"], O.leaf_rows_for(tree, ex["species"]), 0, len(ex["rows"][0]) - 1)
        r = O.score_region(mc, mn, ot, O.FIXED, lv)
        assert r.score == pytest.approx(rec["score"], abs=1e-9)
        assert r.anc == pytest.approx(rec["anc"], abs=1e-9)


def test_dense_and_sparse_leaves_bit_identical():
    mc, mn, ot, tree = H.oracle_models("12flies")
    ex = H.examples()["tal-AA.fa"]
    lv = O.pleaves(ex["rows"], O.leaf_rows_for(tree, ex["species"]), 0, len(ex["rows"][0]) - 1)
    O.set_sparse_leaves(False)
    a = O.lpr_leaves(mc, ot, 0.7, lv)
    O.set_sparse_leaves(True)
    b = O.lpr_leaves(mc, ot, 0.7, lv)
    assert a == b


def test_decibans():
    assert O.decibans(math.log(10.0)) == pytest.approx(10.0)
