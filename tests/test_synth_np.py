"""The numpy restatement of the column simulator (oracle/synth_np.py) against the engine
library's pcsf_simulate: identical leaf codes for any subset of regions (the benchmark's CPU
arm builds its sample of regions with the restatement, without the product library)."""
import numpy as np
import pytest

from phylocsf_gb300 import synth
from oracle import synth_np


@pytest.mark.parametrize("name,lengths,reject", [("12flies", [300, 0, 17, 64], True),
                                                 ("58mammals", [50, 129, 3, 400], True),
                                                 ("58mammals", [80, 9], False)])
def test_numpy_simulator_matches_native(name, lengths, reject):
    ps = synth.load_params(name)
    rng = np.random.default_rng(3)
    models = (np.arange(len(lengths)) % 2).astype(np.int32)
    gf = synth.gap_fractions(rng, len(lengths), ps.tree.nl, 0.05, 0.4, 0.2)
    offs, lv = synth.simulate(ps, np.array(lengths), models, gf, seed=7, reject_stop_leaf0=reject)
    P, prior = synth.simulation_inputs(ps)
    sub = [3, 0, 2] if len(lengths) > 3 else [1, 0]
    got = synth_np.simulate_regions(ps.tree.parent, P, prior, offs, models, gf, 7, sub, reject_stop_leaf0=reject)
    want = np.concatenate([lv[offs[r]:offs[r + 1]] for r in sub])
    assert got.shape == want.shape and np.array_equal(got, want)


def test_workload_spec_regions_match_realized_workload():
    spec = synth.spec_58mammals_mle(n_regions=40, seed=0)
    wl = synth.realize(spec)
    assert np.array_equal(wl.col_offsets, spec.col_offsets)
    P, prior = synth.simulation_inputs(spec.params)
    sub = [39, 5, 12]
    got = synth_np.simulate_regions(spec.params.tree.parent, P, prior, spec.col_offsets, spec.models, spec.gap_frac,
                                    spec.seed, sub)
    want = np.concatenate([wl.leaves[wl.col_offsets[r]:wl.col_offsets[r + 1]] for r in sub])
    assert np.array_equal(got, want)


def test_nucleotide_rows_round_trip_through_native_packing():
    """Simulated codon columns written out as nucleotide rows and packed back by the native
    region packer (pleaves' path) give the same leaf codes in frame 0 of the forward strand;
    the six AsIs frames of an alignment cover its whole length."""
    from phylocsf_gb300 import engine as E
    ps = synth.load_params("12flies")
    rng = np.random.default_rng(4)
    gf = synth.gap_fractions(rng, 1, ps.tree.nl, 0.1, 0.3, 0.0)
    offs, codes = synth.simulate(ps, np.array([90]), np.array([0], np.int32), gf, seed=2)
    rows = synth.nucleotide_rows(codes)
    assert all(len(r) == 270 for r in rows) and "-" not in rows[0]
    comp = str.maketrans("ACGTN-", "TGCAN-")
    rc_rows = [r.translate(comp)[::-1] for r in rows]
    regs = E.candidate_regions(rows[0], 6, "AsIs", 25)
    assert len(regs) == 6 and sorted(r[0] for r in regs) == [False] * 3 + [True] * 3
    o, lv = E.pack_regions(ps.tree.nl, list(range(ps.tree.nl)), rows, rc_rows, regs)
    k = [i for i, r in enumerate(regs) if not r[0] and r[1] == 0][0]
    assert np.array_equal(lv[o[k]:o[k + 1]], codes)
