"""pcsf_lpr_noalloc: the allocation-free likelihood entry point, through the C-ABI.

It is for callers that cannot call cudaMalloc when they need a likelihood
(they own all device memory through their own pool, or run where the
allocator's implicit synchronisation is not allowed).  The test hands it
caller-owned device buffers and checks its results against pcsf_lpr, the
allocating entry point, on two calls in a row (the second call reuses the
static scratch area the first one left behind).  Tolerance: the one the GPU
parity tests use for the engine's own results, 1e-9 relative.

This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

import phylocsf_gb300 as P
from phylocsf_gb300 import synth

pytestmark = pytest.mark.gpu


def _data(name, lengths, seed):
    ps = synth.load_params(name)
    rng = np.random.default_rng(seed)
    gf = synth.gap_fractions(rng, len(lengths), ps.tree.nl, 0.05, 0.4, 0.2)
    offs, lv = synth.simulate(ps, np.asarray(lengths), (np.arange(len(lengths)) % 2).astype(np.int32), gf, seed)
    return ps, offs, lv


@pytest.mark.parametrize("prec", ["fp64", "fp32c"])
def test_noalloc_matches_allocating_entry_point(prec):
    torch = pytest.importorskip("torch")
    ps, offs, leaves = _data("58mammals", [64, 1, 333, 0, 1000, 129], seed=17)
    e = P.Engine(ps.tree, ps.S_c, ps.pi_c, ps.S_n, ps.pi_n, precision=prec)
    lib = P.load_library()
    n = len(offs) - 1
    b = e.batch(offs, leaves)
    d_leaves = torch.from_numpy(leaves).to("cuda")
    d_lpr = torch.empty(n, dtype=torch.float64, device="cuda")
    d_elpr = torch.empty(n, dtype=torch.float64, device="cuda")
    offs_c = np.ascontiguousarray(offs, np.int64)
    for call, (model, rho) in enumerate([(0, 1.0), (1, 0.37)]):
        ref_lpr, ref_elpr, st = e.lpr(b, model, rho)
        assert (st == 0).all()
        d_lpr.fill_(float("nan"))
        d_elpr.fill_(float("nan"))
        torch.cuda.synchronize()
        rc = lib.pcsf_lpr_noalloc(e.handle, model, rho, n, offs_c.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                  ctypes.c_void_p(d_leaves.data_ptr()), ctypes.c_void_p(d_lpr.data_ptr()),
                                  ctypes.c_void_p(d_elpr.data_ptr()))
        assert rc == 0, lib.pcsf_last_error(e.handle)
        got_lpr = d_lpr.cpu().numpy()
        got_elpr = d_elpr.cpu().numpy()
        np.testing.assert_allclose(got_lpr, ref_lpr, rtol=1e-9, atol=1e-9, err_msg="call %d" % call)
        np.testing.assert_allclose(got_elpr, ref_elpr, rtol=1e-9, atol=1e-9, err_msg="call %d" % call)
    # a batch beyond the fixed capacity is refused, before any device work
    big = np.arange(40000, dtype=np.int64)
    rc = lib.pcsf_lpr_noalloc(e.handle, 0, 1.0, len(big) - 1, big.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                              ctypes.c_void_p(d_leaves.data_ptr()), ctypes.c_void_p(d_lpr.data_ptr()), None)
    assert rc == 10      # PCSF_ERANGE
    b.close()
    e.close()
