"""The OmegaModel restatement (oracle/omega.py) pinned piece by piece to the reference's
formulas (src/OmegaModel.ml, lines cited per test; no GPU).  The reference ships no
OmegaModel output, so the assembled score (kr_map and the H1-H0 LLR) is pinned only
through these pieces and the oracle's own Brent, not to a value the reference computed."""
import math

import numpy as np
import pytest

from oracle import oracle as O
from oracle import omega as W
from tests import helpers as H


def test_omega_q_structure():
    """src/OmegaModel.ml:42-74 (q_p14n): only codons one nucleotide apart exchange; the rate is
    pi_j x kappa for a transition (A<->G, C<->T) x omega for a non-synonymous change; a change into
    or out of a stop codon carries no omega; the diagonal makes rows sum to 0.  :76-80 (q_scale):
    mean rate 1 under pi.  Reversible with respect to pi."""
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


def test_omega_pi_f3x4():
    """src/OmegaModel.ml:21-40 (pi_exprs): a codon's frequency is the product over its three
    positions of (that position's A, C or G parameter, or 1 for T) / (A + C + G + 1), divided by
    1 - (1 - sigma) x (the three stop codons' undamped mass)."""
    f = [1.1, 0.9, 1.3, 0.8, 1.2, 1.0, 1.05, 0.95, 1.2]
    sigma = 0.3
    pi = W.omega_pi([2.0, 0.5, sigma] + f)
    rel = np.ones((3, 4))
    rel[:, :3] = np.reshape(f, (3, 3))
    pos = rel / rel.sum(1, keepdims=True)
    und = np.array([pos[0][i // 16] * pos[1][(i // 4) % 4] * pos[2][i % 4] for i in range(64)])
    stop_mass = und[48] + und[50] + und[56]
    np.testing.assert_allclose(pi, und / (1.0 - (1.0 - sigma) * stop_mass), rtol=1e-14)


def test_new_instance_defaults():
    """src/OmegaModel.ml:95-99 (new_instance): kappa = omega = sigma = 1 and all nine F3x4
    parameters 1, i.e. uniform codon frequencies and every single-nucleotide change at the same
    rate."""
    Q, pi = W.omega_q([1.0, 1.0, 1.0] + [1.0] * 9)
    np.testing.assert_allclose(pi, np.full(64, 1.0 / 64), rtol=1e-14)
    off = Q[~np.eye(64, dtype=bool)]
    rates = off[off > 0]
    assert len(rates) == 64 * 9 and np.allclose(rates, rates[0], rtol=1e-14)


def test_f3x4_counts():
    """src/OmegaModel.ml:102-134 (update_f3x4): per codon position, counts of A, C, G, T over the
    Certain leaves only (marginalised leaves skipped), each count starting at 1; the parameters are
    count(A, C or G) / count(T) per position."""
    lv = np.array([[0, 63, -1], [16, 48, 5]], np.int32)
    f = W.f3x4_from_leaves(lv)
    # codons AAA(0) TTT(63) CAA(16) TAA(48) ACC(5 = 16*0 + 4*1 + 1); the -1 leaf is skipped
    # position 1: A 2 (AAA, ACC), C 1, G 0, T 2 -> with the pseudocount 1: 3, 2, 1, 3
    # position 2: A 3 (AAA, CAA, TAA), C 1 (ACC), G 0, T 1 -> 4, 2, 1, 2
    # position 3: the same as position 2 -> 4, 2, 1, 2
    np.testing.assert_allclose(f, [3 / 3, 2 / 3, 1 / 3, 4 / 2, 2 / 2, 1 / 2, 4 / 2, 2 / 2, 1 / 2], rtol=1e-15)


def test_priors():
    """src/OmegaModel.ml:146-156 (half_cauchy_lpdf ~mode:1 ~scale:0.5 for rho: log of
    1 / (pi scale (1 + ((x - mode)/scale)^2)) minus log (1 - cdf(0 - mode)), cdf(y) = atan(y/scale)/pi
    + 1/2) and :157 (lpr_kappa: log Gamma density with a = 7, b = 0.25 at kappa - 1 + epsilon_float)."""
    for x in (0.01, 1.0, 3.7):
        want = math.log(1.0 / (math.pi * 0.5 * (1.0 + ((x - 1.0) / 0.5) ** 2))) - \
            math.log(1.0 - (math.atan(-1.0 / 0.5) / math.pi + 0.5))
        assert W.lpr_rho(x) == pytest.approx(want, rel=1e-14)
    assert W.lpr_rho(1.0) == pytest.approx(math.log(1.0 / (math.pi * 0.5)) - math.log(0.5 + math.atan(2.0) / math.pi))
    for k in (1.0, 2.5, 9.0):
        x = k - 1.0 + 2.220446049250313e-16
        want = 6 * math.log(x) - x / 0.25 - math.lgamma(7.0) - 7 * math.log(0.25)
        assert W.lpr_kappa(k) == pytest.approx(want, abs=1e-12)


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
