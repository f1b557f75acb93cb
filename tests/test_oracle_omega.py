"""The OmegaModel restatement (oracle/omega.py) on its own terms (no GPU)."""
import math

import numpy as np
import pytest

from oracle import oracle as O
from oracle import omega as W
from tests import helpers as H


def test_omega_q_structure():
    q = [2.5, 0.3, 0.5] + [1.1, 0.9, 1.3, 0.8, 1.2, 1.0, 1.05, 0.95, 1.2]
    Q, pi = W.omega_q(q)
    assert np.allclose(Q.sum(1), 0.0, atol=1e-13)
    assert -(pi * np.diag(Q)).sum() == pytest.approx(1.0, rel=1e-12)          # mean rate 1 under pi
    F = pi[:, None] * Q
    assert np.allclose(F, F.T, atol=1e-15)                                     # reversible
    # only single-nucleotide changes; AAA->AAG (K->K, transition A->G) vs AAA->AAC (K->N, transversion)
    assert Q[0, 2] / pi[2] == pytest.approx(2.5 * Q[0, 1] / pi[1] / 0.3, rel=1e-12)
    assert Q[0, 5] == 0.0                                                      # AAA->ACC: two changes
    # stop codons: no omega on a change into a stop (TAC -> TAA, a transversion at position 3)
    taa, tac = 48, 49
    assert Q[tac, taa] / pi[taa] == pytest.approx(Q[0, 1] / pi[1] / 0.3, rel=1e-12)


def test_f3x4_counts():
    lv = np.array([[0, 63, -1], [16, 48, 5]], np.int32)
    f = W.f3x4_from_leaves(lv)
    # position 1 nucleotides: A(0), T(63), C(16), T(48), A(5) -> counts A 3, C 2, G 1, T 3
    assert f[:3] == pytest.approx([3 / 3, 2 / 3, 1 / 3])


def test_priors():
    assert W.lpr_rho(1.0) == pytest.approx(math.log(1.0 / (math.pi * 0.5)) - math.log(0.5 + math.atan(2.0) / math.pi))
    k = 2.5
    x = k - 1.0
    assert W.lpr_kappa(k) == pytest.approx(6 * math.log(x) - x / 0.25 - math.lgamma(7.0) - 7 * math.log(0.25), abs=1e-12)


def test_omega_score_small():
    O.set_sparse_leaves(True)
    tree, *_ = H.fixture_params("12flies")
    ex = H.examples()["tal-AA.fa"]
    lv = O.pleaves(ex["rows"], O.leaf_rows_for(tree, ex["species"]), 0, 47)
    sc, l0, l1, q0, r0, q1, r1, evals = W.score(tree, lv)
    assert math.isfinite(sc) and 1.0 <= q0[0] <= 10.0 and 0.001 <= r0 <= 10.0
    assert q1[1] == 0.2 and q1[2] == 0.01
    assert evals > 20


def test_package_omega_rate_matrix_matches_oracle():
    """The synthetic-data module's OmegaModel rate matrix (used to simulate the differentiation
    workload) against the oracle's restatement of src/OmegaModel.ml:21-80, on uniform and skewed
    F3x4 frequencies and both sigma settings."""
    from phylocsf_gb300 import synth
    from oracle import omega as W
    for q in ([2.5, 0.3, 1.0] + [1.0] * 9, [1.7, 1.4, 0.01, 0.8, 1.2, 1.1, 0.9, 1.0, 1.3, 0.7, 1.5, 1.05]):
        Q, pi = W.omega_q(q)
        Q2, pi2 = synth.omega_rate_matrix(q[0], q[1], q[2], np.array(q[3:]))
        assert np.abs(Q - Q2).max() <= 1e-14 and np.abs(pi - pi2).max() <= 1e-15
