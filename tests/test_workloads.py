"""The synthetic benchmark workloads have the shapes of the configurations they stand in for
(there is no public benchmark: seeded synthetic inputs with the stated sizes, length and gap
distributions and model mixes).  Checked on the specs alone (no simulation).  No GPU."""
import numpy as np

from phylocsf_gb300 import synth


def _lengths(spec):
    return np.diff(spec.col_offsets)


def test_58mammals_mle_shape():
    """10,000 alignments, half coding / half noncoding, lengths log-uniform 50-3,000 codons
    (mean ~720, ~7.2 M columns), per-species gaps U(5 %, 40 %), 0-20 % of species missing."""
    s = synth.spec_58mammals_mle()
    L = _lengths(s)
    assert len(L) == 10000 and L.min() >= 50 and L.max() <= 3000
    assert 650 < L.mean() < 790 and 6.5e6 < L.sum() < 7.9e6
    assert abs(np.mean(np.log(L)) - 0.5 * (np.log(50) + np.log(3000))) < 0.05   # log-uniform
    assert (s.models == 0).sum() == 5000
    g = s.gap_frac
    present = g[g < 1.0]
    assert present.min() >= 0.05 and present.max() <= 0.40
    missing = (g >= 1.0).mean(axis=1)
    assert missing.max() <= 0.21 and 0.05 < missing.mean() < 0.15
    assert (g[:, 0] < 1.0).all()                # the reference row is never missing


def test_100vertebrates_mle_shape():
    """Lengths log-uniform 30-10,000 codons (mean ~1,716), coding : noncoding = 1 : 3, 5-40 % gaps."""
    s = synth.spec_100vertebrates_mle()
    L = _lengths(s)
    assert len(L) == 20000 and L.min() >= 30 and L.max() <= 10000
    assert 1550 < L.mean() < 1880
    assert 0.23 < (s.models == 0).mean() < 0.27
    assert s.gap_frac.min() >= 0.05 and s.gap_frac.max() <= 0.40


def test_120mammals_fixed_shape():
    """2 M columns in alignments of log-uniform 100-5,000 codons, coding : noncoding 1 : 1, rho = 1."""
    s = synth.spec_120mammals_fixed()
    L = _lengths(s)
    assert L.sum() == 2_000_000
    assert L.max() <= 5000 and (L[:-1] >= 100).all()
    assert abs((s.models == 0).mean() - 0.5) < 0.01
    assert s.strategy == synth.E.FIXED


def test_12flies_fixed_shape():
    """One alignment of 300 codons, noncoding model, 10 % gaps per species, fixed rho."""
    s = synth.spec_12flies_fixed()
    assert list(_lengths(s)) == [300] and list(s.models) == [1]
    assert np.allclose(s.gap_frac, 0.10) and s.strategy == synth.E.FIXED


def test_specs_are_seeded():
    a, b = synth.spec_58mammals_mle(200, seed=3), synth.spec_58mammals_mle(200, seed=3)
    c = synth.spec_58mammals_mle(200, seed=4)
    assert (a.col_offsets == b.col_offsets).all() and (a.gap_frac == b.gap_frac).all()
    assert not (a.col_offsets == c.col_offsets).all()
