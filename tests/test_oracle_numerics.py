"""Internal consistency of the CPU oracle (no GPU): eigensystem, P(t), gradient."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import helpers as H


def test_q_assembly_matches_numpy():
    tree, Sc, pic, Sn, pin = H.fixture_params("12flies")
    Q = O.build_q(Sc, pic)
    R = Sc * pic[None, :]
    np.fill_diagonal(R, 0.0)
    np.fill_diagonal(R, -R.sum(1))
    R = R / (-(pic * np.diag(R)).sum())
    assert np.allclose(Q, R, rtol=1e-13, atol=1e-15)
    assert np.allclose(Q.sum(1), 0.0, atol=1e-13)
    assert (pic * -np.diag(Q)).sum() == pytest.approx(1.0, abs=1e-13)


@pytest.mark.parametrize("name", ["12flies", "58mammals"])
def test_jacobi_eigensystem(name):
    tree, Sc, pic, Sn, pin = H.fixture_params(name)
    for S, pi in ((Sc, pic), (Sn, pin)):
        m = O.OModel.from_ecm(S, pi)
        sq = np.sqrt(pi)
        A = sq[:, None] * m.Q / sq[None, :]
        A = 0.5 * (A + A.T)
        assert np.allclose(m.U.T @ m.U, np.eye(64), atol=1e-12)
        assert np.allclose(m.U @ np.diag(m.lam) @ m.U.T, A, atol=1e-12)
        assert np.allclose(np.sort(m.lam), np.sort(np.linalg.eigvalsh(A)), atol=1e-11)


def test_pt_properties_and_scipy_expm():
    scipy_linalg = pytest.importorskip("scipy.linalg")
    tree, Sc, pic, Sn, pin = H.fixture_params("12flies")
    m = O.OModel.from_ecm(Sc, pic)
    for t in (0.0, 0.01, 0.3, 2.5, 8.0):
        P = m.pt(t)
        assert np.all(P >= 0)
        assert np.allclose(P.sum(1), 1.0, atol=1e-12)
        assert np.allclose(P, scipy_linalg.expm(m.Q * t), atol=1e-10)
    with pytest.raises(RuntimeError):
        m.pt(-1.0)


def test_gradient_matches_finite_differences():
    mc, mn, ot, tree = H.oracle_models("12flies")
    ex = H.examples()["tal-AA.fa"]
    lv = O.pleaves(ex["rows"], O.leaf_rows_for(tree, ex["species"]), 0, len(ex["rows"][0]) - 1)
    rho = 0.8
    lpr, g = O.grad_branches(mc, ot, rho, lv)
    assert lpr == pytest.approx(O.lpr_leaves(mc, ot, rho, lv)[0], abs=1e-10)
    h = 1e-5
    base = tree.branch[: tree.n - 1].copy()
    for i in (0, 5, 13, tree.n - 2):
        bp = base.copy()
        bm = base.copy()
        bp[i] += h / rho
        bm[i] -= h / rho
        fp = O.lpr_leaves(mc, O.OTree(tree, bp), rho, lv)[0]
        fm = O.lpr_leaves(mc, O.OTree(tree, bm), rho, lv)[0]
        assert g[i] == pytest.approx((fp - fm) / (2 * h), rel=1e-5, abs=1e-6)
    # d lpr / d rho = sum_i b_i d lpr / d t_i
    fp = O.lpr_leaves(mc, ot, rho + h, lv)[0]
    fm = O.lpr_leaves(mc, ot, rho - h, lv)[0]
    assert float(base @ g) == pytest.approx((fp - fm) / (2 * h), rel=1e-6)


def test_brent_result_is_a_local_maximum():
    mc, mn, ot, tree = H.oracle_models("12flies")
    ex = H.examples()["tal-AA.fa"]
    lv = O.pleaves(ex["rows"], O.leaf_rows_for(tree, ex["species"]), 0, len(ex["rows"][0]) - 1)
    r = O.score_region(mc, mn, ot, O.MLE, lv)
    for m, rho in ((mc, r.rho_c), (mn, r.rho_n)):
        f0 = O.lpr_leaves(m, ot, rho, lv)[0]
        # the stopping rule leaves the maximiser within 1% relative bracket width
        assert f0 >= O.lpr_leaves(m, ot, rho * 1.02, lv)[0] - 1e-3
        assert f0 >= O.lpr_leaves(m, ot, rho / 1.02, lv)[0] - 1e-3


def test_empty_region_mle():
    """An empty region: f == 0 everywhere, find_init exhausts its tries and returns hi (Fit.ml:36-47)."""
    mc, mn, ot, tree = H.oracle_models("12flies")
    r = O.score_region(mc, mn, ot, O.MLE, np.zeros((0, tree.nl), np.int32))
    assert r.status == 0 and r.score == 0.0 and r.rho_c == 10.0 and r.rho_n == 10.0


def test_oracle_branch_counts_identities():
    """The oracle's sufficient statistics (PhyloEM.ml:14-20): every branch's expected counts sum to
    the number of columns, the counts' ELL is at most lpr (Gibbs: ELL - lpr = -entropy of the
    hidden states <= 0), and at fixed counts d ELL / d rho = d lpr / d rho (Fisher identity)."""
    from phylocsf_gb300 import synth
    mc, mn, ot, tree = H.oracle_models("12flies")
    ps = synth.load_params("12flies")
    offs, lv = synth.simulate(ps, np.array([60]), np.array([0], np.int32), np.full((1, 12), 0.2), 3)
    x = H.u8_to_oracle(lv)
    rho = 0.8
    lpr, c = O.branch_counts(mc, ot, rho, x)
    assert lpr == pytest.approx(O.lpr_leaves(mc, ot, rho, x)[0], rel=1e-12)
    np.testing.assert_allclose(c.sum(axis=(1, 2)), 60.0, rtol=1e-12)
    assert (c >= 0).all()
    assert O.ell(mc, ot, rho, c) <= lpr
    h = 1e-6
    dell = (O.ell(mc, ot, rho + h, c) - O.ell(mc, ot, rho - h, c)) / (2 * h)
    dlpr = (O.lpr_leaves(mc, ot, rho + h, x)[0] - O.lpr_leaves(mc, ot, rho - h, x)[0]) / (2 * h)
    assert dell == pytest.approx(dlpr, rel=1e-6)
