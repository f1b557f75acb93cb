"""OmegaModel test on the GPU (pcsf_omega_score) against the oracle restatement (oracle/omega.py).

Tolerances: FP64 engine |d score| <= 1e-6 dB, and kappa / rho within 2 %
relative.  The engine builds each Omega Q and its eigensystem on the GPU, so
its likelihoods agree with the oracle's to ~1e-13 relative, not bit for bit; a
Brent probe sqrt(eps)*|x| from the best point can then compare the other way,
after which the coordinate ascent ends at another point inside its stopping
rule (bracket width <= 1 % of the parameter) while the score, flat at the
optimum, still agrees.  Compensated-FP32 engine |d score| <= 1e-2 dB (its P(t)
is formed in FP64; the pruning is FP32).
"""
import numpy as np
import pytest

import phylocsf_gb300 as P
from phylocsf_gb300 import synth
from oracle import oracle as O
from oracle import omega as W
from tests import helpers as H

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _fast():
    O.set_sparse_leaves(True)


def _regions(name, lengths, seed):
    ps = synth.load_params(name)
    rng = np.random.default_rng(seed)
    gf = synth.gap_fractions(rng, len(lengths), ps.tree.nl, 0.05, 0.3, 0.1)
    return ps, *synth.simulate(ps, np.asarray(lengths), (np.arange(len(lengths)) % 2).astype(np.int32), gf, seed)


@pytest.mark.parametrize("prec", ["fp64", "fp32c"])
def test_omega_matches_oracle(prec):
    ps, offs, leaves = _regions("12flies", [30, 45, 0], seed=13)
    tree, *_ = H.fixture_params("12flies")
    e = P.Engine.for_tree(ps.tree, precision=prec)
    res = e.omega_score(e.batch(offs, leaves), 0.2, 0.01)
    for r in range(len(offs) - 1):
        lv = H.u8_to_oracle(leaves[offs[r]:offs[r + 1]])
        sc, l0, l1, q0, r0, q1, r1, _ = W.score(tree, lv)
        g = res[r]
        assert g["status"] == 0
        if prec == "fp64":
            assert abs(g["score"] - sc) <= 1e-6, (r, g["score"], sc)
            assert g["kappa_h0"] == pytest.approx(q0[0], rel=2e-2)
            assert g["rho_h0"] == pytest.approx(r0, rel=2e-2)
            assert g["kappa_h1"] == pytest.approx(q1[0], rel=2e-2)
            assert g["rho_h1"] == pytest.approx(r1, rel=2e-2)
            assert g["lpr_h0"] == pytest.approx(l0, rel=1e-9)
            assert g["lpr_h1"] == pytest.approx(l1, rel=1e-9)
        else:
            assert abs(g["score"] - sc) <= 1e-2, (r, g["score"], sc)


def test_omega_reference_example():
    """The tal-AA example on 12flies: the GPU and the oracle agree on the omega test."""
    tree, *_ = H.fixture_params("12flies")
    ps = synth.load_params("12flies")
    ex = H.examples()["tal-AA.fa"]
    lv = O.pleaves(ex["rows"], O.leaf_rows_for(tree, ex["species"]), 0, len(ex["rows"][0]) - 1)
    e = P.Engine.for_tree(ps.tree, precision="fp64")
    g = e.omega_score(e.batch(np.array([0, lv.shape[0]], np.int64), H.oracle_leaves_to_u8(lv)))[0]
    sc = W.score(tree, lv)[0]
    assert g["status"] == 0 and abs(g["score"] - sc) <= 1e-6


@pytest.mark.parametrize("name", ["12flies", "29mammals"])
def test_omega_grad_matches_finite_differences(name):
    """d lpr / d {kappa, omega, rho} from pcsf_omega_grad (adjoint + eigenbasis derivative of exp(tQ))
    against central differences with h = 1e-5 of the FP64 engine's own lpr and of the oracle's:
    within 1e-5 relative + 2e-4 absolute (the differences carry ~1e-12 relative evaluation noise over
    2h); lpr itself within 1e-9 relative of the oracle."""
    ps, offs, leaves = _regions(name, [40, 120], seed=29)
    tree, *_ = H.fixture_params(name)
    e = P.Engine.for_tree(ps.tree, precision="fp64")
    b = e.batch(offs, leaves)
    kappa, omega, rho, sigma, h = 2.5, 0.3, 0.8, 1.0, 1e-5
    g = e.omega_grad(b, kappa, omega, rho, sigma)
    assert (g["status"] == 0).all()

    def lpr_at(k, o, r):
        return e.omega_grad(b, k, o, r, sigma, branches=False)["lpr"]

    fd = {"d_kappa": (lpr_at(kappa + h, omega, rho) - lpr_at(kappa - h, omega, rho)) / (2 * h),
          "d_omega": (lpr_at(kappa, omega + h, rho) - lpr_at(kappa, omega - h, rho)) / (2 * h),
          "d_rho": (lpr_at(kappa, omega, rho + h) - lpr_at(kappa, omega, rho - h)) / (2 * h)}
    for k, v in fd.items():
        assert np.all(np.abs(g[k] - v) <= 1e-5 * np.abs(v) + 2e-4), (k, g[k], v)
    assert np.allclose(g["d_branch"] @ tree.branch[: tree.n - 1], g["d_rho"], rtol=1e-12, atol=1e-12)
    for r in range(len(offs) - 1):
        lv = H.u8_to_oracle(leaves[offs[r]:offs[r + 1]])
        obj = W._Objective(O.OTree(tree), np.ascontiguousarray(lv, np.int32))
        q = [kappa, omega, sigma] + list(W.f3x4_from_leaves(lv))
        assert g["lpr"][r] == pytest.approx(obj.lpr(q, rho), rel=1e-9)
        for k, idx in (("d_kappa", 0), ("d_omega", 1)):
            qp, qm = list(q), list(q)
            qp[idx] += h
            qm[idx] -= h
            ofd = (obj.lpr(qp, rho) - obj.lpr(qm, rho)) / (2 * h)
            assert abs(g[k][r] - ofd) <= 1e-5 * abs(ofd) + 2e-4, (k, r, g[k][r], ofd)


def test_omega_grad_fp32_close_to_fp64():
    ps, offs, leaves = _regions("29mammals", [150, 60], seed=31)
    g64 = P.Engine.for_tree(ps.tree, precision="fp64")
    g32 = P.Engine.for_tree(ps.tree, precision="fp32c")
    a = g64.omega_grad(g64.batch(offs, leaves), 2.0, 0.5, 1.2, 0.01)
    c = g32.omega_grad(g32.batch(offs, leaves), 2.0, 0.5, 1.2, 0.01)
    for k in ("d_kappa", "d_omega", "d_rho"):
        assert np.all(np.abs(c[k] - a[k]) <= 1e-3 * np.abs(a[k]) + 1e-2), (k, c[k], a[k])


def test_gradient_map_beside_brent():
    """The gradient MAP (omega_fit.gradient_map: batched projected BFGS on pcsf_omega_grad) reaches
    at least the objective of the reference's Brent coordinate ascent (the H0 fit of
    pcsf_omega_score, which stops at a 1 % bracket) on every region, and lands next to it."""
    from phylocsf_gb300 import omega_fit
    ps, offs, leaves = _regions("29mammals", [200, 350, 600, 80, 450, 260], seed=37)
    e = P.Engine.for_tree(ps.tree, precision="fp64")
    b = e.batch(offs, leaves)
    brent = e.omega_score(b)
    gm = omega_fit.gradient_map(e, b, omega=1.0, sigma=1.0)
    assert (gm["status"] == 0).all()
    # kr_map reports lpr + log p(kappa) from its last (kappa) step; add log p(rho) for the joint objective
    brent_f = brent["lpr_h0"] + omega_fit.log_prior_rho(brent["rho_h0"])
    gap = gm["objective"] - brent_f
    print("gradient MAP - Brent objective:", gap, "evaluations:", gm["evals"], "Brent evals:", brent["evals"])
    assert np.all(gap >= -1e-6 * np.abs(brent_f) - 1e-6), gap
    assert np.all(gap <= 0.5), gap
    assert np.allclose(gm["rho"], brent["rho_h0"], rtol=0.05)
    assert np.allclose(gm["kappa"], brent["kappa_h0"], rtol=0.05)


# ---------------------------------------------------------------- the differentiation configuration
# OmegaModel on the 100vertebrates tree, alignments simulated under the OmegaModel's own Q at
# kappa = 2.5, sigma = 1, uniform F3x4 and omega log-uniform in [0.05, 2] (synth.workload_100vertebrates_omega).

def _omega_wl(lengths, seed):
    return synth.workload_100vertebrates_omega(seed=seed, lengths=np.asarray(lengths))


def test_omega_grad_100vertebrates_finite_differences():
    """d lpr / d {kappa, omega, rho} and d lpr / d t for a leaf branch, an internal branch and a root
    branch, by pcsf_omega_grad (FP64 engine) against central differences with h = 1e-5 of the engine's
    own lpr; per region omega (the value it was simulated at).  Within 1e-5 relative + 2e-3 absolute
    (lpr here is ~1e5 nats, so the differences carry ~1e-6 of rounding over 2h)."""
    wl = _omega_wl([200, 450, 800], seed=3)
    tree = wl.tree
    e = P.Engine.for_tree(tree, precision="fp64")
    b = e.batch(wl.col_offsets, wl.leaves)
    kappa, omega, rho, sigma, h = 2.2, wl.omega.copy(), 1.0, 1.0, 1e-5
    g = e.omega_grad(b, kappa, omega, rho, sigma)
    assert (g["status"] == 0).all()

    def lpr_at(eng, bb, k, o, r):
        return eng.omega_grad(bb, k, o, r, sigma, branches=False)["lpr"]

    fd = {"d_kappa": (lpr_at(e, b, kappa + h, omega, rho) - lpr_at(e, b, kappa - h, omega, rho)) / (2 * h),
          "d_omega": (lpr_at(e, b, kappa, omega + h, rho) - lpr_at(e, b, kappa, omega - h, rho)) / (2 * h),
          "d_rho": (lpr_at(e, b, kappa, omega, rho + h) - lpr_at(e, b, kappa, omega, rho - h)) / (2 * h)}
    for k, v in fd.items():
        assert np.all(np.abs(g[k] - v) <= 1e-5 * np.abs(v) + 2e-3), (k, g[k], v)
    for br in (0, tree.nl + 3, tree.n - 2):
        vals = []
        for sgn in (1, -1):
            bl = tree.branch.copy()
            bl[br] += sgn * h
            t2 = P.Tree(tree.parent, bl, tree.labels)
            e2 = P.Engine.for_tree(t2, precision="fp64")
            vals.append(lpr_at(e2, e2.batch(wl.col_offsets, wl.leaves), kappa, omega, rho))
            e2.close()
        fdb = (vals[0] - vals[1]) / (2 * h)
        assert np.all(np.abs(g["d_branch"][:, br] - fdb) <= 1e-5 * np.abs(fdb) + 2e-3), (br, g["d_branch"][:, br], fdb)
    e.close()


def test_omega_grad_100vertebrates_fp32_close_to_fp64():
    """The configuration's arithmetic (FP32 with compensated sums, P(t) and its eigenbasis
    derivative in FP64) against the FP64 engine: every gradient entry within 1e-3 relative + 1e-2."""
    wl = _omega_wl([300, 900, 1500, 250], seed=5)
    a = P.Engine.for_tree(wl.tree, precision="fp64")
    c = P.Engine.for_tree(wl.tree, precision="fp32c")
    ga = a.omega_grad(a.batch(wl.col_offsets, wl.leaves), 2.5, wl.omega, 1.1, 1.0)
    gc = c.omega_grad(c.batch(wl.col_offsets, wl.leaves), 2.5, wl.omega, 1.1, 1.0)
    for k in ("d_kappa", "d_omega", "d_rho", "d_branch"):
        assert np.all(np.abs(gc[k] - ga[k]) <= 1e-3 * np.abs(ga[k]) + 1e-2), k
    np.testing.assert_allclose(gc["lpr"], ga["lpr"], rtol=1e-7)
    a.close()
    c.close()


def test_gradient_map_100vertebrates_beside_brent_and_omega_mle():
    """On 100vertebrates: (a) the gradient MAP of (rho, kappa) at omega = 1 reaches at least the
    objective of the reference's Brent coordinate ascent (the H0 fit of pcsf_omega_score) on every
    region and lands next to it; (b) with omega free, the gradient fit of (rho, kappa, omega) ends
    with a vanishing projected gradient and recovers the omega each 1,500-codon alignment was
    simulated at (within a factor 1.35)."""
    from phylocsf_gb300 import omega_fit
    wl = _omega_wl([250, 600, 1500, 1500, 1500, 400], seed=7)
    e = P.Engine.for_tree(wl.tree, precision="fp64")
    b = e.batch(wl.col_offsets, wl.leaves)
    brent = e.omega_score(b)
    gm = omega_fit.gradient_map(e, b, omega=1.0, sigma=1.0)
    assert (gm["status"] == 0).all()
    brent_f = brent["lpr_h0"] + omega_fit.log_prior_rho(brent["rho_h0"])
    gap = gm["objective"] - brent_f
    print("100vertebrates gradient MAP - Brent objective:", gap, "evaluations:", gm["evals"], "Brent:", brent["evals"])
    assert np.all(gap >= -1e-6 * np.abs(brent_f) - 1e-6), gap
    assert np.allclose(gm["rho"], brent["rho_h0"], rtol=0.05)
    assert np.allclose(gm["kappa"], brent["kappa_h0"], rtol=0.05)
    fo = omega_fit.gradient_map(e, b, sigma=1.0, fit_omega=True, iters=60)
    print("omega MLE:", fo["omega"], "simulated at:", wl.omega)
    assert (fo["status"] == 0).all()
    assert np.all(np.abs(fo["gradient"]).max(axis=1) <= 1e-3 * np.maximum(1.0, np.abs(fo["objective"])))
    assert np.all(fo["objective"] >= gm["objective"] - 1e-6 * np.abs(gm["objective"]))
    long = np.diff(wl.col_offsets) >= 1500
    assert np.all(np.abs(np.log(fo["omega"][long] / wl.omega[long])) <= np.log(1.35)), (fo["omega"], wl.omega)
    e.close()
