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

PCSF_EINVAL, PCSF_ERANGE = 1, 10


def _data(name, lengths, seed):
    ps = synth.load_params(name)
    rng = np.random.default_rng(seed)
    gf = synth.gap_fractions(rng, len(lengths), ps.tree.nl, 0.05, 0.4, 0.2)
    offs, lv = synth.simulate(ps, np.asarray(lengths), (np.arange(len(lengths)) % 2).astype(np.int32), gf, seed)
    return ps, offs, lv


def _call(lib, e, model, rho, offs, d_leaves, d_lpr, d_elpr):
    n = len(offs) - 1
    offs_c = np.ascontiguousarray(offs, np.int64)
    return lib.pcsf_lpr_noalloc(e.handle, model, rho, n, offs_c.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                None if d_leaves is None else ctypes.c_void_p(d_leaves.data_ptr()),
                                ctypes.c_void_p(d_lpr.data_ptr()),
                                None if d_elpr is None else ctypes.c_void_p(d_elpr.data_ptr()))


CASES = [("58mammals", "fp64", [64, 1, 333, 0, 1000, 129]),
         ("58mammals", "fp32c", [64, 1, 333, 0, 1000, 129]),
         ("58mammals", "tf32x3b", [64, 1, 333, 0, 1000, 129]),
         ("58mammals", "fp32b_pt64", [200, 31, 700]),
         ("120mammals", "tf32x3b", [500, 33, 1200])]      # five-slot tree: 32-column SIMT tiles


@pytest.mark.parametrize("name,prec,lengths", CASES)
def test_noalloc_matches_allocating_entry_point(name, prec, lengths):
    torch = pytest.importorskip("torch")
    ps, offs, leaves = _data(name, lengths, seed=17)
    e = P.Engine(ps.tree, ps.S_c, ps.pi_c, ps.S_n, ps.pi_n, precision=prec)
    lib = P.load_library()
    n = len(offs) - 1
    b = e.batch(offs, leaves)
    d_leaves = torch.from_numpy(leaves).to("cuda")
    d_lpr = torch.empty(n, dtype=torch.float64, device="cuda")
    d_elpr = torch.empty(n, dtype=torch.float64, device="cuda")
    for call, (model, rho, with_elpr) in enumerate([(0, 1.0, True), (1, 0.37, False)]):
        ref_lpr, ref_elpr, st = e.lpr(b, model, rho)
        assert (st == 0).all()
        d_lpr.fill_(float("nan"))
        d_elpr.fill_(float("nan"))
        torch.cuda.synchronize()
        rc = _call(lib, e, model, rho, offs, d_leaves, d_lpr, d_elpr if with_elpr else None)
        assert rc == 0, lib.pcsf_last_error(e.handle)
        np.testing.assert_allclose(d_lpr.cpu().numpy(), ref_lpr, rtol=1e-9, atol=1e-9, err_msg="call %d" % call)
        if with_elpr:
            np.testing.assert_allclose(d_elpr.cpu().numpy(), ref_elpr, rtol=1e-9, atol=1e-9, err_msg="call %d" % call)
        else:
            assert np.isnan(d_elpr.cpu().numpy()).all()       # untouched
    b.close()
    e.close()


def test_noalloc_refusals():
    torch = pytest.importorskip("torch")
    ps, offs, leaves = _data("12flies", [40, 7], seed=3)
    e = P.Engine(ps.tree, ps.S_c, ps.pi_c, ps.S_n, ps.pi_n, precision="fp32b")
    lib = P.load_library()
    d_lpr = torch.empty(2, dtype=torch.float64, device="cuda")
    # a leaf code above PCSF_MARGINALIZE is refused, as pcsf_batch_create refuses it
    bad = leaves.copy()
    bad[45, 3] = 65
    rc = _call(lib, e, 0, 1.0, offs, torch.from_numpy(bad).to("cuda"), d_lpr, None)
    assert rc == PCSF_EINVAL
    assert b"leaf code" in lib.pcsf_last_error(e.handle)
    # no leaves for a batch with columns
    assert _call(lib, e, 0, 1.0, offs, None, d_lpr, None) == PCSF_EINVAL
    # a batch beyond the fixed capacity is refused, before any device work
    d_leaves = torch.from_numpy(leaves).to("cuda")
    big = np.arange(40000, dtype=np.int64)
    assert _call(lib, e, 0, 1.0, big, d_leaves, d_lpr, None) == PCSF_ERANGE
    # after the refusals the entry point still gives pcsf_lpr's values
    b = e.batch(offs, leaves)
    ref, _, _ = e.lpr(b, 1, 2.5)
    assert _call(lib, e, 1, 2.5, offs, d_leaves, d_lpr, None) == 0
    np.testing.assert_allclose(d_lpr.cpu().numpy(), ref, rtol=1e-9, atol=1e-9)
    b.close()
    e.close()
