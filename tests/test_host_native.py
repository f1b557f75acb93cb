"""Native library surface without a GPU: symbols, host helpers vs the oracle's restatements."""
import ctypes
import os
import re

import numpy as np
import pytest

import phylocsf_gb300 as P
from phylocsf_gb300 import engine as E
from phylocsf_gb300 import synth
from oracle import oracle as O
from tests import helpers as H

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names += re.findall(r"\b(pcsf_[a-z0-9_]+)\s*\(", txt)
    return sorted(set(names))


def test_library_loads_and_exports_every_declared_symbol():
    lib = P.load_library()
    decl = declared_functions()
    assert len(decl) >= 18
    for name in decl:
        assert hasattr(lib, name), name
        assert name in E.SIGNATURES, "no ctypes signature for " + name


def test_engine_without_gpu_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    tree, Sc, pic, Sn, pin = H.fixture_params("12flies")
    t = P.Tree(tree.parent, tree.branch, tree.labels)
    with pytest.raises(P.EngineError) as ei:
        P.Engine(t, Sc, pic, Sn, pin)
    assert ei.value.status == 2          # PCSF_ECUDA: no CPU fallback


def test_newick_parser_matches_oracle(reference_dir):
    for name in ("12flies", "29mammals", "58mammals", "100vertebrates", "120mammals"):
        path = os.path.join(reference_dir, "PhyloCSF_Parameters", name + ".nh")
        t = P.Tree.load(path)
        o = O.load_tree(path)
        assert np.array_equal(t.parent, o.parent)
        nb = o.n - 1
        assert np.array_equal(t.branch[:nb], o.branch[:nb])
        assert t.labels[: t.nl] == o.labels[: o.nl]


def test_newick_edge_cases():
    t = P.Tree.from_newick("((a:1,b:2):3,c:4);")
    assert list(t.parent) == [3, 3, 4, 4, -1]
    assert t.labels[:3] == ["a", "b", "c"] and np.isnan(t.branch[4])
    with pytest.raises(P.EngineError):
        P.Tree.from_newick("(a,b,c);")          # not bifurcating
    with pytest.raises(P.EngineError):
        P.Tree.from_newick("((a,b);")           # syntax
    # a digits-only token lexes as a branch length (NewickLexer.mll rule order)
    with pytest.raises(P.EngineError):
        P.Tree.from_newick("(123,b);")


def test_ecm_reader_matches_oracle(reference_dir):
    for name in ("12flies_coding", "29mammals_noncoding", "100vertebrates_coding"):
        path = os.path.join(reference_dir, "PhyloCSF_Parameters", name + ".ECM")
        S, pi = P.read_ecm(path)
        So, pio = O.read_ecm(path)
        assert np.array_equal(S, So) and np.array_equal(pi, pio)
        assert np.array_equal(S, S.T) and S[0, 0] == 0.0


def _write_ecm(path, S, pi):
    """An ECM file in the layout ECM.import_parameters reads (src/ECM.ml:18-72): 63 rows of the
    strict lower triangle, a blank line, the 64 frequencies, two free lines, 64 codons on lines
    67-70 in index order."""
    codons = [O.codon_of_index(i) for i in range(64)]
    lines = [" ".join(repr(float(S[i, j])) for j in range(i)) for i in range(1, 64)]
    lines += ["", " ".join(repr(float(x)) for x in pi), "", ""]
    lines += [" ".join(codons[16 * k:16 * k + 16]) for k in range(4)]
    path.write_text("\n".join(lines) + "\n")


def _newick_of(tree):
    """Newick text of an oracle tree (left child first; branch lengths in repr, so they parse
    back exactly)."""
    def rec(i):
        if tree.lchild[i] < 0:
            body = tree.labels[i]
        else:
            body = "(" + rec(tree.lchild[i]) + "," + rec(tree.rchild[i]) + ")"
        return body + (":" + repr(float(tree.branch[i])) if tree.parent[i] >= 0 else "")
    return rec(len(tree.parent) - 1) + ";"


@pytest.mark.parametrize("name", ["12flies", "58mammals", "120mammals"])
def test_readers_round_trip_shipped_parameters(tmp_path, name):
    """The native ECM reader and Newick parser read back, bit for bit, files written from the
    parameter sets shipped with the package, and agree with the oracle's readers."""
    ps = synth.load_params(name)
    for m, (S, pi) in enumerate(((ps.S_c, ps.pi_c), (ps.S_n, ps.pi_n))):
        path = tmp_path / ("%s_%d.ECM" % (name, m))
        _write_ecm(path, S, pi)
        Sr, pir = P.read_ecm(str(path))
        So, pio = O.read_ecm(str(path))
        assert np.array_equal(Sr, S) and np.array_equal(pir, pi)
        assert np.array_equal(So, S) and np.array_equal(pio, pi)
    txt = _newick_of(H.fixture_params(name)[0])
    t = P.Tree.from_newick(txt)
    o = O.tree_of_newick(O.parse_newick(txt))
    nb = ps.tree.n - 1
    assert np.array_equal(t.parent, ps.tree.parent) and np.array_equal(o.parent, ps.tree.parent)
    assert np.array_equal(t.branch[:nb], ps.tree.branch[:nb]) and np.array_equal(o.branch[:nb], ps.tree.branch[:nb])
    assert t.labels[:t.nl] == ps.tree.labels[:t.nl] == o.labels[:o.nl]


def test_ecm_reader_rejects_bad_codon_order_written(tmp_path):
    ps = synth.load_params("12flies")
    path = tmp_path / "bad.ECM"
    _write_ecm(path, ps.S_c, ps.pi_c)
    lines = path.read_text().split("\n")
    lines[67] = lines[67].replace("AAA AAC", "AAC AAA")
    path.write_text("\n".join(lines))
    with pytest.raises(P.EngineError, match="codon order"):
        P.read_ecm(str(path))


def test_ecm_reader_rejects_bad_codon_order(tmp_path, reference_dir):
    src = os.path.join(reference_dir, "PhyloCSF_Parameters", "12flies_coding.ECM")
    lines = open(src).read().split("\n")
    lines[67] = lines[67].replace("AAA AAC", "AAC AAA")
    bad = tmp_path / "bad.ECM"
    bad.write_text("\n".join(lines))
    with pytest.raises(P.EngineError, match="codon order"):
        P.read_ecm(str(bad))


@pytest.mark.parametrize("frames", [1, 3, 6])
@pytest.mark.parametrize("mode", ["AsIs", "ATGStop", "StopStop", "StopStop3", "ToFirstStop", "FromLastStop",
                                  "ToOrFromStop"])
def test_candidate_regions_match_oracle(frames, mode):
    rng = np.random.default_rng(frames * 7 + len(mode))
    for trial in range(20):
        L = int(rng.integers(3, 400))
        dna = "".join(rng.choice(list("ACGTacgtN"), size=L, p=[.22, .22, .22, .22, .02, .02, .02, .02, .04]))
        mc = int(rng.integers(1, 30))
        assert P.candidate_regions(dna, frames, mode, mc) == O.candidate_regions(dna, frames, mode, mc)


def test_candidate_regions_examples():
    for fa, ex in H.examples().items():
        ref = O.remove_ref_gaps(ex["rows"])[0]
        for frames in (1, 3, 6):
            for mode in ("AsIs", "ATGStop", "StopStop3"):
                assert P.candidate_regions(ref, frames, mode) == O.candidate_regions(ref, frames, mode)


def test_pack_regions_matches_pleaves():
    ex = H.examples()["ALDH2.exon5.fa"]
    tree, *_ = H.fixture_params("29mammals")
    rows = O.leaf_rows_for(tree, ex["species"])
    aln = ex["rows"]
    rc = [O.revcomp(s) for s in aln]
    regs = O.candidate_regions(aln[0], 6, "AsIs")
    offs, leaves = P.pack_regions(tree.nl, rows, aln, rc, regs)
    for i, (isrc, lo, hi) in enumerate(regs):
        ref = O.pleaves(rc if isrc else aln, rows, lo, hi)
        got = H.u8_to_oracle(leaves[offs[i]:offs[i + 1]])
        assert np.array_equal(got, ref)


def test_simulate_deterministic_and_thread_independent():
    ps = synth.load_params("12flies")
    lengths = np.array([17, 0, 300, 5])
    models = np.array([0, 1, 1, 0])
    gf = np.full((4, ps.tree.nl), 0.1)
    o1, a = synth.simulate(ps, lengths, models, gf, seed=3, threads=1)
    o2, b = synth.simulate(ps, lengths, models, gf, seed=3, threads=4)
    assert np.array_equal(a, b) and np.array_equal(o1, o2)
    assert a.max() <= 64
    assert not np.isin(a[:, 0], [48, 50, 56]).any()          # no stop codon in leaf 0
    gaps = (a == 64).mean()
    assert 0.05 < gaps < 0.15


def test_simulated_composition_tracks_model():
    """Root-to-leaf simulation: leaf codon frequencies are close to pi (the chain is stationary)."""
    ps = synth.load_params("12flies")
    o, a = synth.simulate(ps, np.array([20000]), np.array([1]), None, seed=1, reject_stop_leaf0=False)
    freq = np.bincount(a[:, 5], minlength=64) / a.shape[0]
    assert np.abs(freq - ps.pi_n).max() < 0.01
