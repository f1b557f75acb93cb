"""GPU adjoint gradient (pcsf_grad) against the oracle's outside pass and finite differences.

Tolerances: FP64 engine, per-branch d lpr / d t within 1e-7 relative (abs
floor 1e-8) of the oracle (the oracle differentiates P(t) = exp(tQ)
analytically, the kernel applies dP/dt = Q P to P after the clamp /
renormalise row rule); FP32 (compensated or blocked) per entry within 1e-4
relative plus 2e-6 per column of the region.  d lpr / d rho against a central difference of the
FP64 engine's lpr with h = 1e-5: within 1e-6 relative.
"""
import numpy as np
import pytest

import phylocsf_gb300 as P
from phylocsf_gb300 import synth
from oracle import oracle as O
from tests import helpers as H

pytestmark = pytest.mark.gpu

_E = {}
_G = {}     # oracle gradients, shared by the precisions


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


@pytest.mark.parametrize("prec", ["fp64", "fp32c", "fp32b"])
@pytest.mark.parametrize("name", ["12flies", "29mammals", "58mammals", "100vertebrates"])
def test_branch_gradient_matches_oracle(prec, name):
    e = engine(name, prec)
    mc, mn, ot, tree = H.oracle_models(name)
    lengths = [90, 1, 200, 0] if name in ("12flies", "29mammals") else [90, 1, 333, 0, 700, 64]
    offs, leaves = _data(name, lengths, seed=21)
    b = e.batch(offs, leaves)
    for model, om in ((0, mc), (1, mn)):
        for rho in (0.3, 1.0, 2.5):
            lpr, db, drho, st = e.grad(b, model, rho)
            assert (st == 0).all()
            for r in range(len(offs) - 1):
                lv = H.u8_to_oracle(leaves[offs[r]:offs[r + 1]])
                key = (name, model, rho, r)
                if key not in _G:
                    _G[key] = O.grad_branches(om, ot, rho, lv)
                lo, go = _G[key]
                if lv.shape[0] == 0:
                    assert np.all(db[r] == 0.0) and lpr[r] == 0.0
                    continue
                if prec == "fp64":
                    assert lpr[r] == pytest.approx(lo, rel=1e-9)
                    err = np.abs(db[r] - go) - (1e-7 * np.abs(go) + 1e-8)
                    k = int(np.argmax(err))
                    assert err[k] <= 0, (model, rho, r, k, db[r][k], go[k], tree.branch[k])
                else:
                    # per entry: 1e-4 relative plus 2e-6 per column (the FP32 rounding of each
                    # column's term), so near-zero entries are held to an absolute bound
                    err = np.abs(db[r] - go) - (1e-4 * np.abs(go) + 2e-6 * lv.shape[0])
                    k = int(np.argmax(err))
                    assert err[k] <= 0, (model, rho, r, k, db[r][k], go[k])
                assert drho[r] == pytest.approx(float(tree.branch[: tree.n - 1] @ db[r]), rel=1e-12, abs=1e-12)


def test_rho_gradient_matches_central_difference():
    e = engine("58mammals", "fp64")
    offs, leaves = _data("58mammals", [150, 700], seed=3)
    b = e.batch(offs, leaves)
    h = 1e-5
    for model in (0, 1):
        for rho in (0.5, 1.0, 3.0):
            _, _, drho, st = e.grad(b, model, rho)
            fp = e.lpr(b, model, rho + h)[0]
            fm = e.lpr(b, model, rho - h)[0]
            fd = (fp - fm) / (2 * h)
            assert np.allclose(drho, fd, rtol=1e-6, atol=1e-6), (drho, fd)


def test_gradient_zero_at_mle():
    """At the fitted rho the derivative in rho is close to zero (relative to its scale)."""
    e = engine("29mammals", "fp64")
    offs, leaves = _data("29mammals", [400], seed=8)
    res = e.score_batch(offs, leaves, P.MLE)
    b = e.batch(offs, leaves)
    _, _, d1, _ = e.grad(b, 0, res[0]["rho_c"])
    _, _, d2, _ = e.grad(b, 0, res[0]["rho_c"] * 1.2)
    assert abs(d1[0]) < 0.05 * abs(d2[0])


@pytest.mark.parametrize("prec", ["fp64", "fp32b"])
@pytest.mark.parametrize("name", ["12flies", "100vertebrates"])
def test_recomputed_leaf_partials_identical(name, prec):
    """The adjoint with leaf children's partials recomputed in the outside pass (a third less
    scratch per CTA) gives bit-identical lpr, branch gradients and d / d rho, and reports the
    smaller scratch."""
    ps = synth.load_params(name)
    e = P.Engine(ps.tree, ps.S_c, ps.pi_c, ps.S_n, ps.pi_n, precision=prec)
    offs, leaves = _data(name, [90, 1, 333, 0, 700], seed=31)
    b = e.batch(offs, leaves)
    stored = e.grad_scratch_bytes()
    ref = [e.grad(b, m, rho) for m in (0, 1) for rho in (0.3, 2.5)]
    e.set_grad_recompute(True)
    assert e.grad_scratch_bytes() < 0.7 * stored
    got = [e.grad(b, m, rho) for m in (0, 1) for rho in (0.3, 2.5)]
    for x, y in zip(ref, got):
        for u, v in zip(x, y):
            assert u.tobytes() == v.tobytes()
