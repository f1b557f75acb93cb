"""Branch length score (src/PhyloCSF.ml:252-262) against a direct restatement of
Newick.subtree + Newick.total_length (lib/CamlPaml/Newick.ml:34-61) per column."""
import numpy as np

from oracle import oracle as O
from phylocsf_gb300 import driver as D
from phylocsf_gb300 import engine as E
from tests import helpers as H


def _subtree(node, keep):
    if not node.children:
        return node if (node.label == "" or keep(node.label)) else None
    if not (node.label == "" or keep(node.label)):
        return None
    kids = [k for k in (_subtree(c, keep) for c in node.children) if k is not None]
    if not kids:
        return None
    if len(kids) == 1:
        k = kids[0]
        bl = None if node.branch is None or k.branch is None else node.branch + k.branch
        return O.NewickNode(k.children, k.label, bl)
    return O.NewickNode(kids, node.label, node.branch)


def _total(node, count_root=False):
    def tl(x):
        return (x.branch if x.branch is not None else 0.0) + sum(tl(c) for c in x.children)
    return tl(node) if count_root else sum(tl(c) for c in node.children)


def test_bls_matches_newick_subtree_restatement():
    tree, *_ = H.fixture_params("29mammals")
    nt = O.NewickNode([], "", None)
    # rebuild a Newick tree from the T arrays (children in order)
    def mk(i):
        if i < tree.nl:
            return O.NewickNode([], tree.labels[i], float(tree.branch[i]))
        return O.NewickNode([mk(tree.lchild[i]), mk(tree.rchild[i])], "", float(tree.branch[i]) if i < tree.n - 1 else None)
    nt = mk(tree.n - 1)
    ex = H.examples()["ALDH2.exon5.fa"]
    sp, aln = ex["species"], ex["rows"]
    rows = O.leaf_rows_for(tree, sp)
    which = {s: i for i, s in enumerate(sp)}
    lo, hi = 3, 60
    tot = 0.0
    for i in range(lo, hi + 1):
        st = _subtree(nt, lambda s: s in which and aln[which[s]][i] not in "-.N")
        tot += _total(st) if st is not None else 0.0
    want = tot / (_total(nt) * (hi - lo + 1))
    et = E.Tree(tree.parent, tree.branch, tree.labels)
    assert abs(D.bls(et, aln, rows, lo, hi) - want) < 1e-12


def test_bls_prefix_sums_match_restatement_on_many_windows():
    """The per-column spanning-subtree lengths (native pcsf_bls_columns) and the prefix-sum
    windows against the per-column Newick.subtree restatement, on both strands of an example with
    extra random gaps, for 40 random windows."""
    tree, *_ = H.fixture_params("29mammals")

    def mk(i):
        if i < tree.nl:
            return O.NewickNode([], tree.labels[i], float(tree.branch[i]))
        return O.NewickNode([mk(tree.lchild[i]), mk(tree.rchild[i])], "", float(tree.branch[i]) if i < tree.n - 1 else None)
    nt = mk(tree.n - 1)
    ex = H.examples()["ALDH2.exon5.fa"]
    sp = ex["species"]
    rng = np.random.default_rng(5)
    aln = ["".join(c if rng.random() > 0.15 else rng.choice(list("-.N")) for c in r) for r in ex["rows"]]
    rows = O.leaf_rows_for(tree, sp)
    which = {s: i for i, s in enumerate(sp)}
    et = E.Tree(tree.parent, tree.branch, tree.labels)
    comp = str.maketrans("ACGTacgt", "TGCAtgca")
    for strand in (aln, [r.translate(comp)[::-1] for r in aln]):
        per_col = D.bls_columns(et, strand, rows)
        L = len(strand[0])
        for i in range(0, L, 7):
            st = _subtree(nt, lambda s: s in which and strand[which[s]][i] not in "-.N")
            assert abs(per_col[i] - (_total(st) if st is not None else 0.0)) < 1e-12
        b = D.BLS(et, strand, rows)
        for _ in range(20):
            lo = int(rng.integers(0, L - 1))
            hi = int(rng.integers(lo, L))
            want = sum(_total(s) if s is not None else 0.0 for s in
                       (_subtree(nt, lambda x, i=i: x in which and strand[which[x]][i] not in "-.N")
                        for i in range(lo, hi + 1))) / (_total(nt) * (hi - lo + 1))
            assert abs(b(lo, hi) - want) < 1e-12
