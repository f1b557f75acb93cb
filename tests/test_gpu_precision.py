"""Precision of the split-precision contractions on the 120mammals workload (238 branches,
2 M codon columns in alignments of 100-5000 codons, rho = 1), against the FP64 GPU path
(itself within 1e-9 relative of the FP64 oracle, test_gpu_parity.py).

Per alignment: relative logL error of each model and |d score| of the fixed-strategy
score.  Bounds (the measured values are printed):
  - tensor cores, TF32 single product (tf32_direct): relative logL error <= 2e-3;
  - tensor cores, TF32 hi/lo x3 (tf32x3_direct): relative logL error <= 2e-6;
  - tensor cores, 3xBF16 split x = h + m + l with the six products that reach FP32
    accuracy (bf16x3_direct): relative logL error <= 2e-6;
  - returned values of the tensor-core engines (tf32x3b, bf16x3b: compensated SIMT and
    float-float kernels) and the compensated FP32 engines: |d score| <= 1e-3 dB for every
    alignment.
"""
import numpy as np
import pytest

import phylocsf_gb300 as P
from phylocsf_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def workload():
    return synth.workload_120mammals_fixed(total_cols=2_000_000, seed=0)


@pytest.fixture(scope="module")
def reference(workload):
    ps = workload.params
    e = P.Engine(ps.tree, ps.S_c, ps.pi_c, ps.S_n, ps.pi_n, precision="fp64")
    b = e.batch(workload.col_offsets, workload.leaves)
    out = (e.lpr(b, 0, 1.0)[0], e.lpr(b, 1, 1.0)[0])
    e.close()
    return out


def _lprs(workload, prec):
    ps = workload.params
    e = P.Engine(ps.tree, ps.S_c, ps.pi_c, ps.S_n, ps.pi_n, precision=prec)
    b = e.batch(workload.col_offsets, workload.leaves)
    out = (e.lpr(b, 0, 1.0)[0], e.lpr(b, 1, 1.0)[0])
    e.close()
    return out


@pytest.mark.parametrize("prec,rel_bound,db_bound", [("tf32_direct", 2e-3, None), ("tf32x3_direct", 2e-6, None),
                                                     ("bf16x3_direct", 2e-6, None),
                                                     ("tf32x3b", None, 1e-3), ("bf16x3b", None, 1e-3),
                                                     ("fp32b", None, 1e-3), ("fp32c", None, 1e-3)])
def test_120mammals_precision(workload, reference, prec, rel_bound, db_bound):
    c64, n64 = reference
    c, n = _lprs(workload, prec)
    rel = np.maximum(np.abs(c - c64) / np.abs(c64), np.abs(n - n64) / np.abs(n64))
    ddb = np.abs(10.0 * ((c - n) - (c64 - n64)) / np.log(10.0))
    print("%s: %d alignments, relative logL error max %.3e median %.3e; |d score| max %.3e dB median %.3e dB"
          % (prec, len(c), rel.max(), np.median(rel), ddb.max(), np.median(ddb)))
    if rel_bound is not None:
        assert rel.max() <= rel_bound
    if db_bound is not None:
        assert ddb.max() <= db_bound


@pytest.mark.parametrize("prec", ["fp32b", "tf32x3b"])
def test_long_regions_fixed_rho(prec):
    """Returned values on long 100vertebrates regions (2,000 / 5,000 / 10,000 codons) at fixed rho,
    against FP64.  Regions at or past the engine's threshold (columns x (n_leaves - 2) >= 150,000,
    1,531 codons here) take their values from the float-float kernel: |d score| <= 1e-6 dB
    (measured ~1e-10).  Regions just below it (1,530 codons) stay on the compensated FP32 kernel,
    whose error grows roughly linearly with length (measured max 3.0e-4 / 8.8e-4 / 1.6e-3 dB at
    2,000 / 5,000 / 10,000 codons without the float-float kernel): <= 5e-4 dB."""
    ps = synth.load_params("100vertebrates")
    rng = np.random.default_rng(11)
    lengths = np.array([2000] * 4 + [5000] * 4 + [10000] * 2 + [1530] * 8)
    models = (rng.random(len(lengths)) >= 0.25).astype(np.int32)
    gf = synth.gap_fractions(rng, len(lengths), ps.tree.nl, 0.05, 0.40, 0.0)
    offs, lv = synth.simulate(ps, lengths, models, gf, 5)
    e64 = P.Engine(ps.tree, ps.S_c, ps.pi_c, ps.S_n, ps.pi_n, precision="fp64")
    e = P.Engine(ps.tree, ps.S_c, ps.pi_c, ps.S_n, ps.pi_n, precision=prec)
    b64, b = e64.batch(offs, lv), e.batch(offs, lv)
    for rho in (1.0, 3.0):
        c0, n0 = e64.lpr(b64, 0, rho)[0], e64.lpr(b64, 1, rho)[0]
        c, n = e.lpr(b, 0, rho)[0], e.lpr(b, 1, rho)[0]
        ddb = np.abs(10.0 * ((c - n) - (c0 - n0)) / np.log(10.0))
        print("%s rho %.1f: float-float regions max %.2e dB; 1,530-codon regions (FP32 kernel) max %.2e dB"
              % (prec, rho, ddb[:10].max(), ddb[10:].max()))
        assert ddb[:10].max() <= 1e-6
        assert ddb[10:].max() <= 5e-4
    e.close()
    e64.close()
