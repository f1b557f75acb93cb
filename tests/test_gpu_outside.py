"""Outside-pass statistics on the GPU against the FP64 oracle: expected substitution counts of
every branch (PhyloEM sufficient statistics, lib/CamlPaml/PhyloEM.ml:14-20 over
PhyloLik.add_branch_posteriors, PhyloLik.ml:140-174), their expected log-likelihood
(PhyloEM.ell, PhyloEM.ml:22-73) and node posteriors (PhyloLik.node_posterior, PhyloLik.ml:127-138).

Tolerances: FP64 engine -- counts within 1e-9 relative + 1e-9 x columns, ELL and lpr within 1e-9
relative, posteriors within 1e-10; FP32 engines (compensated FP32 arithmetic) -- counts within
2e-5 relative + 2e-5 x columns, posteriors within 2e-5.
"""
import numpy as np
import pytest

import phylocsf_gb300 as P
from phylocsf_gb300 import synth
from oracle import oracle as O
from tests import helpers as H

pytestmark = pytest.mark.gpu

_E = {}


def engine(name, prec):
    if (name, prec) not in _E:
        ps = synth.load_params(name)
        _E[(name, prec)] = P.Engine(ps.tree, ps.S_c, ps.pi_c, ps.S_n, ps.pi_n, precision=prec)
    return _E[(name, prec)]


def _data(name, lengths, seed):
    ps = synth.load_params(name)
    rng = np.random.default_rng(seed)
    gf = synth.gap_fractions(rng, len(lengths), ps.tree.nl, 0.05, 0.4, 0.2)
    return synth.simulate(ps, np.asarray(lengths), (np.arange(len(lengths)) % 2).astype(np.int32), gf, seed)


@pytest.fixture(scope="module", autouse=True)
def _fast():
    O.set_sparse_leaves(True)


CASES = [("12flies", "fp64"), ("12flies", "fp32b"), ("58mammals", "fp64"), ("58mammals", "tf32x3b"),
         ("120mammals", "fp32b")]


@pytest.mark.parametrize("name,prec", CASES)
def test_branch_counts_and_ell_match_oracle(name, prec):
    e = engine(name, prec)
    mc, mn, ot, tree = H.oracle_models(name)
    lengths = [1, 31, 32, 33, 150] if name != "120mammals" else [40, 65]
    offs, leaves = _data(name, lengths, seed=29)
    b = e.batch(offs, leaves)
    fp64 = prec == "fp64"
    rt = 1e-9 if fp64 else 2e-5
    for model, om in ((0, mc), (1, mn)):
        rho = np.linspace(0.4, 2.5, len(lengths))
        counts, lpr, st = e.branch_counts(b, model, rho)
        assert (st == 0).all()
        ref_lpr, _, _ = e.lpr(b, model, rho)
        np.testing.assert_allclose(lpr, ref_lpr, rtol=1e-9 if fp64 else 1e-6, atol=1e-9)
        for r, L in enumerate(lengths):
            lv = H.u8_to_oracle(leaves[offs[r]:offs[r + 1]])
            olpr, oc = O.branch_counts(om, ot, rho[r], lv)
            assert abs(lpr[r] - olpr) <= (1e-9 if fp64 else 2e-6) * abs(olpr) + 1e-9
            np.testing.assert_allclose(counts[r], oc, rtol=rt, atol=rt * L, err_msg="region %d" % r)
            # every branch's expected counts sum to the number of columns
            np.testing.assert_allclose(counts[r].sum(axis=(1, 2)), L, rtol=1e-9 if fp64 else 1e-5)
            ell = e.ell(model, rho[r], counts[r])
            oell = O.ell(om, ot, rho[r], oc)
            assert abs(ell - oell) <= (1e-9 if fp64 else 2e-5) * abs(oell) + 1e-9, (ell, oell)


def test_ell_fisher_identity():
    """At fixed sufficient statistics, d ELL / d rho equals d lpr / d rho (PhyloEM.ml:140-182):
    central difference of pcsf_ell (h = 1e-5) against the adjoint's d lpr / d rho."""
    e = engine("58mammals", "fp64")
    offs, leaves = _data("58mammals", [120, 300], seed=31)
    b = e.batch(offs, leaves)
    for rho in (0.6, 1.7):
        counts, lpr, st = e.branch_counts(b, 0, rho)
        _, _, drho, _ = e.grad(b, 0, rho, branches=False)
        for r in range(2):
            h = 1e-5
            fd = (e.ell(0, rho + h, counts[r]) - e.ell(0, rho - h, counts[r])) / (2 * h)
            assert fd == pytest.approx(drho[r], rel=1e-6, abs=1e-6)


@pytest.mark.parametrize("name,prec", [("12flies", "fp64"), ("12flies", "tf32x3b"), ("58mammals", "fp64"),
                                       ("58mammals", "fp32b")])
def test_node_posteriors_match_oracle(name, prec):
    e = engine(name, prec)
    mc, mn, ot, tree = H.oracle_models(name)
    offs, leaves = _data(name, [37, 1, 70], seed=41)
    b = e.batch(offs, leaves)
    n = tree.n
    nodes = np.arange(n) if name == "12flies" else np.array([n - 1, n - 2, 0, 3, tree.nl, (n + tree.nl) // 2])
    rho = np.array([0.8, 1.3, 2.2])
    post, st = e.node_posteriors(b, 1, rho, nodes)
    assert (st == 0).all()
    tol = 1e-10 if prec == "fp64" else 2e-5
    for r in range(len(offs) - 1):
        Ps = np.stack([mn.pt(rho[r] * ot.branch[i]) for i in range(n - 1)])
        lv = H.u8_to_oracle(leaves[offs[r]:offs[r + 1]])
        for col in range(offs[r], offs[r + 1]):
            z, op = O.column_posteriors(tree, Ps, mn.prior, lv[col - offs[r]])
            np.testing.assert_allclose(post[:, col, :], op[nodes], rtol=0, atol=tol, err_msg="column %d" % col)
    # internal nodes' posteriors are distributions
    internal = [k for k, v in enumerate(nodes) if v >= tree.nl]
    np.testing.assert_allclose(post[internal].sum(axis=2), 1.0, atol=1e-9 if prec == "fp64" else 2e-5)
