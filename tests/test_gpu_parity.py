"""GPU parity: the CUDA engine (through the C-ABI) against the FP64 CPU oracle.

Tolerances (stated per test):
  - FP64 engine: P(t) entries within 1e-12, lpr within 1e-9 relative, scores
    within 1e-6 dB (same Brent iterates as the oracle).
  - FP32 engines (FP32 contractions on P-I, FP64 eigensystem / exp / sums,
    P(t) corrected around an FP64 grid): P(t) entries within 2e-6.
    fp32c (compensated summation) and fp32b (blocked compensation):
    |d lpr| within max(2.3e-4 nats (= 1e-3 dB),
    5e-9 |lpr|) per model on regions up to 3000 codons for rho in [0.1, 10]
    (the relative term only matters far from the optimum, e.g. rho = 10), fixed-strategy
    |d score| <= 1e-3 dB, mle |d score| <= 1e-3 dB for every region.  fp32 (plain
    summation) carries a downward bias of ~0.3 ulp per contraction; its lpr tolerance
    is 4e-3 nats.
  - The float-float kernel (returned values of long regions): lpr within 1e-12
    relative of the FP64 engine.
"""
import numpy as np
import pytest

import phylocsf_gb300 as P
from phylocsf_gb300 import driver as D
from phylocsf_gb300 import synth
from oracle import oracle as O
from tests import helpers as H

pytestmark = pytest.mark.gpu

DB_PER_NAT = 10.0 / np.log(10.0)


@pytest.fixture(scope="module", autouse=True)
def _oracle_fast():
    O.set_sparse_leaves(True)


_ENGINES = {}


def engine(name, prec):
    key = (name, prec)
    if key not in _ENGINES:
        ps = synth.load_params(name)
        _ENGINES[key] = P.Engine(ps.tree, ps.S_c, ps.pi_c, ps.S_n, ps.pi_n, precision=prec)
    return _ENGINES[key]


PRECS = ["fp64", "fp32c", "fp32b", "fp32"]
PRECS_MLE = ["fp64", "fp32c", "fp32b"]     # plain fp32 is a precision-study mode (biased sums), not an MLE path


@pytest.mark.parametrize("prec", PRECS)
def test_pt_matches_oracle(prec):
    e = engine("58mammals", prec)
    mc, mn, ot, tree = H.oracle_models("58mammals")
    ts = np.array([0.0, 1e-4, 0.00655, 0.05, 0.3, 1.0, 4.0, 25.0])
    tol = 1e-12 if prec == "fp64" else 2e-6
    assert e.precision == prec
    for m, om in ((0, mc), (1, mn)):
        Pg, st = e.pt(m, ts)
        assert (st == 0).all()
        for i, t in enumerate(ts):
            Po = om.pt(t)
            assert np.abs(Pg[i] - Po).max() <= tol, (m, t, np.abs(Pg[i] - Po).max())
            assert np.allclose(Pg[i].sum(1), 1.0, atol=tol * 64)
            assert (Pg[i] >= 0).all()


@pytest.mark.parametrize("name", ["12flies", "29mammals", "58mammals", "100vertebrates", "120mammals"])
def test_eigensystem_matches_oracle(name):
    """k_jacobi (FP64 cyclic Jacobi on the GPU) against the oracle's Jacobi on the CPU, for both
    models of every parameter set: eigenvalues within 1e-12, U orthonormal within 1e-12, and
    D^-1/2 U diag(lam) U^T D^1/2 reproducing Q within 1e-12."""
    e = engine(name, "fp64")
    mc, mn, ot, tree = H.oracle_models(name)
    for m, om in ((0, mc), (1, mn)):
        U, lam = e.eigensystem(m)
        assert np.allclose(np.sort(lam), np.sort(om.lam), atol=1e-12)
        assert np.allclose(U.T @ U, np.eye(64), atol=1e-12)
        sq = np.sqrt(om.pi)
        Qr = (U * lam) @ U.T * sq[None, :] / sq[:, None]
        assert np.abs(Qr - om.Q).max() <= 1e-12


@pytest.mark.parametrize("name", ["58mammals", "100vertebrates"])
def test_search_pt_matches_oracle(name):
    """k_pform_tc, the tensor-core P(t) of the search (TF32 hi/lo products around the FP32 grid),
    against the oracle's FP64 P(t): entries within 2e-6, rows summing to 1 within 1e-6, no negative
    entries, over t from 0 to the longest branch at rho = 9.9."""
    e = engine(name, "tf32x3")
    mc, mn, ot, tree = H.oracle_models(name)
    bmax = tree.branch[: tree.n - 1].max()
    # t = 0, below the FP32 grid (Taylor), on and between grid points, up to rho = 9.9 on the longest branch
    ts = np.array([0.0, 4e-6, 1e-5, 3e-4, 0.00655, 0.05, 0.3, 1.0, 0.5 * bmax, 3.3 * bmax, 9.9 * bmax])
    for m, om in ((0, mc), (1, mn)):
        Pg, st = e.pt_search(m, ts)
        assert (st == 0).all()
        for i, t in enumerate(ts):
            Po = om.pt(t)
            assert np.abs(Pg[i] - Po).max() <= 2e-6, (m, t, np.abs(Pg[i] - Po).max())
            assert np.allclose(Pg[i].sum(1), 1.0, atol=1e-6)
            assert (Pg[i] >= 0).all()


def _synthetic(name, lengths, seed, gaps=(0.05, 0.4), missing=0.2):
    ps = synth.load_params(name)
    rng = np.random.default_rng(seed)
    lengths = np.asarray(lengths, np.int64)
    models = (np.arange(len(lengths)) % 2).astype(np.int32)
    gf = synth.gap_fractions(rng, len(lengths), ps.tree.nl, gaps[0], gaps[1], missing)
    return synth.simulate(ps, lengths, models, gf, seed)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("name,lengths", [("12flies", [300, 1, 64, 65, 129, 0, 7]),
                                          ("58mammals", [50, 333, 1000, 3000])])
def test_lpr_matches_oracle(prec, name, lengths):
    e = engine(name, prec)
    mc, mn, ot, tree = H.oracle_models(name)
    offs, leaves = _synthetic(name, lengths, seed=11)
    b = e.batch(offs, leaves)
    for model, om in ((0, mc), (1, mn)):
        for rho in (0.1, 0.37, 1.0, 3.3, 10.0):
            lpr, elpr, st = e.lpr(b, model, rho)
            assert (st == 0).all()
            for r in range(len(lengths)):
                lv = H.u8_to_oracle(leaves[offs[r]:offs[r + 1]])
                lo, eo = O.lpr_leaves(om, ot, rho, lv)
                if prec == "fp64":
                    assert lpr[r] == pytest.approx(lo, rel=1e-9, abs=1e-9)
                    assert elpr[r] == pytest.approx(eo, rel=1e-9, abs=1e-9)
                else:
                    tol = max(2.3e-4, 5e-9 * abs(lo)) if prec in ("fp32c", "fp32b") else 4e-3
                    assert abs(lpr[r] - lo) <= tol, (r, rho, lpr[r] - lo)
                    assert abs(elpr[r] - eo) <= tol, (r, rho, elpr[r] - eo)


@pytest.mark.parametrize("prec", PRECS)
def test_fixed_scores_match_oracle_fixtures(prec):
    for fa, rec in H.oracle_fixed().items():
        e = engine(rec["params"], prec)
        ex = H.examples()[fa]
        res = D.process_alignment(e, _mfa(ex), D.Options(strategy=P.FIXED, anc_comp=True))
        r = res.best.result
        tol = 1e-6 if prec == "fp64" else 1e-3 if prec in ("fp32c", "fp32b") else 4e-3
        assert abs(r["score"] - rec["score"]) <= tol
        assert abs(r["anc_comp_score"] - rec["anc"]) <= tol


def _mfa(ex):
    return "\n".join(">%s\n%s" % (s, r) for s, r in zip(ex["species"], ex["rows"])) + "\n"


@pytest.mark.parametrize("prec", PRECS_MLE)
@pytest.mark.parametrize("idx", [0, 1, 2, 3])
def test_reference_pins_through_gpu(prec, idx):
    """src/test.ml:27-59 through the GPU driver path (mle)."""
    p = H.pins()[idx]
    f = H.parse_flags(p["flags"])
    e = engine(p["params"], prec)
    ex = H.examples()[p["file"]]
    opts = D.Options(strategy=P.MLE, frames=f["frames"], orf_mode=f["orf"], remove_ref_gaps=f["remove_ref_gaps"],
                     anc_comp=True, aa=f["aa"])
    res = D.process_alignment(e, _mfa(ex), opts, fn=p["file"])
    best = res.best
    wins = p["windows"]
    assert wins[0][0] < best.result["score"] < wins[0][1], best.result["score"]
    if len(wins) > 1:
        assert wins[1][0] < best.result["anc_comp_score"] < wins[1][1]
    if p["ints"]:
        assert [best.lo, best.hi] == p["ints"]
    if p["strand"]:
        assert (not best.rc) == (p["strand"] == "+")
    if f["aa"]:
        assert res.lines[-1].split("\t")[-1].startswith("MLRAALTTVRRGPRLSRLLSAAA")


def test_mle_fp64_follows_oracle_iterates():
    e = engine("29mammals", "fp64")
    mc, mn, ot, tree = H.oracle_models("29mammals")
    offs, leaves = _synthetic("29mammals", [40, 120, 200, 75, 1], seed=5)
    res = e.score_batch(offs, leaves, P.MLE)
    for r in range(len(offs) - 1):
        lv = H.u8_to_oracle(leaves[offs[r]:offs[r + 1]])
        o = O.score_region(mc, mn, ot, O.MLE, lv)
        g = res[r]
        assert g["status"] == 0 and o.status == 0
        assert abs(g["score"] - o.score) <= 1e-6
        assert abs(g["anc_comp_score"] - o.anc) <= 1e-6
        assert g["rho_c"] == pytest.approx(o.rho_c, rel=1e-9)
        assert g["rho_n"] == pytest.approx(o.rho_n, rel=1e-9)


@pytest.mark.parametrize("prec", ["fp32c", "fp32b"])
def test_mle_fp32_close_to_fp64(prec):
    """The compensated FP32 paths against the FP64 path on mle scores (Brent included): |d score| <= 1e-3 dB
    for every region."""
    offs, leaves = _synthetic("58mammals", list(np.random.default_rng(2).integers(50, 3000, size=64)), seed=2)
    a = engine("58mammals", "fp64").score_batch(offs, leaves, P.MLE)
    b = engine("58mammals", prec).score_batch(offs, leaves, P.MLE)
    assert (a["status"] == 0).all() and (b["status"] == 0).all()
    d = np.abs(a["score"] - b["score"])
    assert d.max() <= 1e-3, np.sort(d)[-8:]


@pytest.mark.parametrize("name", ["12flies", "58mammals", "100vertebrates", "120mammals"])
@pytest.mark.parametrize("prec", ["fp32b", "tf32x3b"])
def test_float_float_kernel_matches_fp64(name, prec):
    """The float-float kernel (every region forced onto it) against the FP64 engine at fixed rho:
    lpr and elpr within 1e-12 relative (measured: below 1e-15)."""
    e = engine(name, prec)
    if not e.exact_available:
        pytest.skip("tree does not fit the float-float kernel")
    e64 = engine(name, "fp64")
    offs, leaves = _synthetic(name, [1, 31, 32, 33, 300, 1000], seed=23)
    b, b64 = e.batch(offs, leaves), e64.batch(offs, leaves)
    e.set_exact_threshold(0)
    try:
        for model in (0, 1):
            for rho in (0.05, 1.0, 4.0):
                l, el, st = e.lpr(b, model, rho)
                l64, el64, st64 = e64.lpr(b64, model, rho)
                assert (st == 0).all() and (st64 == 0).all()
                assert np.all(np.abs(l - l64) <= 1e-12 * np.abs(l64) + 1e-12), (model, rho, l - l64)
                assert np.all(np.abs(el - el64) <= 1e-12 * np.abs(el64) + 1e-12), (model, rho, el - el64)
    finally:
        e.set_exact_threshold(150000)


@pytest.mark.parametrize("prec", PRECS)
def test_beagle_tinytest_embedded(prec):
    """lib/CamlPaml/test.ml:56-99 with the 4-state JC69 model embedded in the 64 codon states
    (states 4..63 have no rate and a negligible root prior)."""
    b = H.beagle()
    tree = P.Tree.from_newick(b["tree"])
    Q = np.zeros((64, 64))
    Q[:4, :4] = 1.0 / 3.0
    np.fill_diagonal(Q[:4, :4], -1.0)
    eq = np.ones(64)
    eq[:4] = 0.25
    prior = np.full(64, 1e-300)
    prior[:4] = 0.25
    e = P.Engine.from_q(tree, Q, eq, prior, Q, eq, prior, precision=prec)
    seqs = b["seqs"]
    order = [seqs[tree.labels[i]] for i in range(tree.nl)]
    L = len(order[0])
    lv = np.array([[("ACGT".index(s[i]) if s[i] in "ACGT" else 64) for s in order] for i in range(L)], np.uint8)
    bt = e.batch(np.array([0, L], np.int64), lv)
    lpr, _, st = e.lpr(bt, 0, 1.0)
    assert st[0] == 0
    assert abs(lpr[0] - b["logL"]) <= b["eps"]


@pytest.mark.parametrize("prec", PRECS_MLE)
def test_edge_cases(prec):
    e = engine("12flies", prec)
    mc, mn, ot, tree = H.oracle_models("12flies")
    nl = tree.nl
    cols = [np.full((0, nl), 64, np.uint8),                   # empty region
            np.full((5, nl), 64, np.uint8),                   # all marginalised
            np.array([[0] * nl], np.uint8),                   # one column, all AAA
            np.tile(np.arange(nl, dtype=np.uint8) + 40, (64, 1))]   # exactly one tile
    offs = np.zeros(len(cols) + 1, np.int64)
    offs[1:] = np.cumsum([c.shape[0] for c in cols])
    leaves = np.concatenate(cols)
    res = e.score_batch(offs, leaves, P.MLE)
    assert (res["status"] == 0).all()
    assert res[0]["score"] == 0.0 and res[0]["rho_c"] == 10.0       # find_init exhausts its tries
    for r in range(1, len(cols)):
        lv = H.u8_to_oracle(cols[r])
        o = O.score_region(mc, mn, ot, O.MLE, lv)
        assert abs(res[r]["score"] - o.score) <= (1e-6 if prec == "fp64" else 2e-3)
    with pytest.raises(P.EngineError):
        e.batch(np.array([0, 1], np.int64), np.full((1, nl), 65, np.uint8))     # invalid leaf code
    with pytest.raises(P.EngineError):
        e.batch(np.array([0, 2, 1], np.int64), np.zeros((2, nl), np.uint8))     # decreasing offsets


def test_deterministic():
    e = engine("58mammals", "fp32c")
    offs, leaves = _synthetic("58mammals", [500, 70, 1200], seed=9)
    a = e.score_batch(offs, leaves, P.MLE)
    b = e.score_batch(offs, leaves, P.MLE)
    assert a.tobytes() == b.tobytes()


def test_region_order_invariance():
    e = engine("58mammals", "fp32c")
    offs, leaves = _synthetic("58mammals", [300, 80, 700, 64], seed=4)
    a = e.score_batch(offs, leaves, P.FIXED)
    perm = [2, 0, 3, 1]
    parts = [leaves[offs[i]:offs[i + 1]] for i in perm]
    offs2 = np.zeros(5, np.int64)
    offs2[1:] = np.cumsum([p.shape[0] for p in parts])
    b = e.score_batch(offs2, np.concatenate(parts), P.FIXED)
    assert np.array_equal(a["score"][perm], b["score"])


def test_stats_count_kernels():
    e = engine("12flies", "fp32c")
    e.reset_stats()
    offs, leaves = _synthetic("12flies", [100, 200], seed=1)
    e.score_batch(offs, leaves, P.FIXED)
    s = e.stats()
    assert s["kernel_launches"] >= 3 and s["evaluations"] == 4
    assert s["column_branches"] == 300 * 2 * (2 * 12 - 2)


@pytest.mark.parametrize("name,prec", [("58mammals", "fp32b"), ("120mammals", "tf32x3b")])
def test_autotune_keeps_values(name, prec):
    """pcsf_engine_autotune picks one of the FP32 kernel's column tiles by timing and reports it;
    the per-column arithmetic does not depend on the tile, so lpr changes only by the order of the
    FP64 tile sums (<= 1e-12 relative)."""
    ps = synth.load_params(name)
    e = P.Engine(ps.tree, ps.S_c, ps.pi_c, ps.S_n, ps.pi_n, precision=prec)
    offs, leaves = _synthetic(name, [30, 64, 65, 400, 900], seed=13)
    b = e.batch(offs, leaves)
    before = [e.lpr(b, m, 0.7)[0] for m in (0, 1)]
    tile = e.autotune(b)
    assert tile in (32, 64)
    assert e.stats()["simt_tile"] == tile
    after = [e.lpr(b, m, 0.7)[0] for m in (0, 1)]
    for x, y in zip(before, after):
        np.testing.assert_allclose(y, x, rtol=1e-12, atol=0)
    e.close()


def test_batch_outlives_engine():
    """A batch destroyed after its engine (an explicit close of the engine while batches are
    still referenced): the batch's destroy reads only its own fields, and calls through a closed
    engine fail with an error instead of touching freed memory."""
    ps = synth.load_params("12flies")
    e = P.Engine(ps.tree, ps.S_c, ps.pi_c, ps.S_n, ps.pi_n, precision="fp32b")
    offs, leaves = _synthetic("12flies", [40, 7], seed=2)
    batches = [e.batch(offs, leaves) for _ in range(3)]
    assert np.isfinite(e.lpr(batches[0], 0, 1.0)[0]).all()
    e.close()
    with pytest.raises(P.EngineError):
        e.lpr(batches[1], 0, 1.0)
    for b in batches:
        b.close()
