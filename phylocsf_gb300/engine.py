"""ctypes binding of the engine's C-ABI (include/phylocsf_engine.h, phylocsf_host.h).

The Python surface mirrors the reference's model interface
(src/PhyloCSFModel.ml): :func:`make` builds the coding/noncoding pair,
:meth:`Engine.score` is ``PhyloCSFModel.score`` over many regions at once and
:meth:`Engine.lpr` is ``lpr_leaves``.  There is no CPU fallback: without the
compiled library or a GB300 every call raises.
"""
from __future__ import annotations

import ctypes
import os
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import _build

PCSF_OK = 0
STATUS_NAMES = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of memory",
                4: "CamlPaml.Q.substition_matrix: expm(tQ) entry < -tol",
                5: "CamlPaml.Q.substitution matrix: row sum of expm(tQ) differs from 1",
                6: "Assert_failure: renormalised diagonal of expm(tQ) not in (0,1]",
                7: "Gsl.Error: endpoints do not enclose a minimum",
                8: "eigensolver did not converge",
                9: "CamlPaml.P14n.instantiate_q: Q scale evaluated to a non-positive value",
                10: "capacity exceeded"}
FIXED, MLE = 0, 1
PREC = {"fp64": 0, "fp32": 1, "tf32x3": 2, "bf16x3": 3, "tf32": 4,
        "fp32c": 1 | (1 << 16),      # FP32 contractions with compensated summation
        "fp32b": 1 | (1 << 18),      # FP32 contractions with blocked compensation
        "tf32x3b": 2 | (1 << 18),    # tensor-core search, blocked-compensation returned values
        "bf16x3b": 3 | (1 << 18),    # BF16-split tensor-core search, blocked-compensation returned values
        "tf32x3_direct": 2 | (1 << 17), "tf32_direct": 4 | (1 << 17),   # lpr straight from the tensor cores
        "bf16x3_direct": 3 | (1 << 17),
        "fp32b_pt64": 1 | (1 << 18) | (1 << 19)}   # FP64-formed P(t) stored in FP32 (accuracy studies)
MARGINALIZE = 64
ORF_MODES = {"asis": 0, "atgstop": 1, "stopstop": 2, "stopstop3": 3, "tofirststop": 4,
             "fromlaststop": 5, "toorfromstop": 6}


class EngineError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__("%s (status %d)" % (msg, status))
        self.status = status


class _Tree(ctypes.Structure):
    _fields_ = [("n_leaves", ctypes.c_int32), ("parent", ctypes.POINTER(ctypes.c_int32)),
                ("branch", ctypes.POINTER(ctypes.c_double))]


class Result(ctypes.Structure):
    _fields_ = [("score", ctypes.c_double), ("anc_comp_score", ctypes.c_double),
                ("rho_c", ctypes.c_double), ("rho_n", ctypes.c_double),
                ("lpr_c", ctypes.c_double), ("lpr_n", ctypes.c_double),
                ("elpr_c", ctypes.c_double), ("elpr_n", ctypes.c_double),
                ("status", ctypes.c_int32), ("evals", ctypes.c_int32)]


RESULT_DTYPE = np.dtype([("score", "f8"), ("anc_comp_score", "f8"), ("rho_c", "f8"), ("rho_n", "f8"),
                         ("lpr_c", "f8"), ("lpr_n", "f8"), ("elpr_c", "f8"), ("elpr_n", "f8"),
                         ("status", "i4"), ("evals", "i4")])
assert RESULT_DTYPE.itemsize == ctypes.sizeof(Result)


class OmegaResult(ctypes.Structure):
    _fields_ = [("score", ctypes.c_double), ("lpr_h0", ctypes.c_double), ("lpr_h1", ctypes.c_double),
                ("rho_h0", ctypes.c_double), ("kappa_h0", ctypes.c_double), ("rho_h1", ctypes.c_double),
                ("kappa_h1", ctypes.c_double), ("status", ctypes.c_int32), ("evals", ctypes.c_int32)]


OMEGA_DTYPE = np.dtype([("score", "f8"), ("lpr_h0", "f8"), ("lpr_h1", "f8"), ("rho_h0", "f8"), ("kappa_h0", "f8"),
                        ("rho_h1", "f8"), ("kappa_h1", "f8"), ("status", "i4"), ("evals", "i4")])
assert OMEGA_DTYPE.itemsize == ctypes.sizeof(OmegaResult)


class Stats(ctypes.Structure):
    _fields_ = [("kernel_launches", ctypes.c_int64), ("evaluations", ctypes.c_int64),
                ("column_branches", ctypes.c_int64), ("rounds", ctypes.c_int64),
                ("prune_ms", ctypes.c_double), ("pform_ms", ctypes.c_double), ("other_ms", ctypes.c_double),
                ("prune_launches", ctypes.c_int64), ("pform_launches", ctypes.c_int64),
                ("kind_launches", ctypes.c_int64 * 5), ("kind_columns", ctypes.c_int64 * 5),
                ("kind_ms", ctypes.c_double * 5),
                ("prune_grid", ctypes.c_int32), ("tc_grid", ctypes.c_int32), ("simt_tile", ctypes.c_int32),
                ("tc_shape", ctypes.c_int32)]


# Every entry point declared in include/*.h, with its ctypes signature.
_D = ctypes.POINTER(ctypes.c_double)
_I32 = ctypes.POINTER(ctypes.c_int32)
_I64 = ctypes.POINTER(ctypes.c_int64)
_U8 = ctypes.POINTER(ctypes.c_uint8)
_VP = ctypes.c_void_p
SIGNATURES = {
    "pcsf_engine_create": ([ctypes.POINTER(_Tree), _D, _D, _D, _D, ctypes.c_int32, ctypes.POINTER(_VP)], ctypes.c_int),
    "pcsf_engine_create_q": ([ctypes.POINTER(_Tree), _D, _D, _D, _D, _D, _D, ctypes.c_int32, ctypes.POINTER(_VP)],
                             ctypes.c_int),
    "pcsf_engine_create_tree": ([ctypes.POINTER(_Tree), ctypes.c_int32, ctypes.POINTER(_VP)], ctypes.c_int),
    "pcsf_omega_score": ([_VP, _VP, ctypes.c_double, ctypes.c_double, ctypes.POINTER(OmegaResult)], ctypes.c_int),
    "pcsf_omega_grad": ([_VP, _VP, _D, _D, ctypes.c_double, _D, _D, _D, _D, _D, _D, _I32], ctypes.c_int),
    "pcsf_engine_destroy": ([_VP], None),
    "pcsf_last_error": ([_VP], ctypes.c_char_p),
    "pcsf_engine_get_stats": ([_VP, ctypes.POINTER(Stats)], ctypes.c_int),
    "pcsf_engine_reset_stats": ([_VP], ctypes.c_int),
    "pcsf_engine_stream": ([_VP, ctypes.POINTER(_VP)], ctypes.c_int),
    "pcsf_engine_eigensystem": ([_VP, ctypes.c_int32, _D, _D], ctypes.c_int),
    "pcsf_engine_pt": ([_VP, ctypes.c_int32, ctypes.c_int32, _D, _D, _I32], ctypes.c_int),
    "pcsf_batch_create": ([_VP, ctypes.c_int32, _I64, _U8, ctypes.POINTER(_VP)], ctypes.c_int),
    "pcsf_batch_destroy": ([_VP], None),
    "pcsf_score": ([_VP, _VP, ctypes.c_int32, ctypes.POINTER(Result)], ctypes.c_int),
    "pcsf_score_batch": ([_VP, ctypes.c_int32, _I64, _U8, ctypes.c_int32, ctypes.POINTER(Result)], ctypes.c_int),
    "pcsf_lpr": ([_VP, _VP, ctypes.c_int32, _D, _D, _D, _I32], ctypes.c_int),
    "pcsf_grad": ([_VP, _VP, ctypes.c_int32, _D, _D, _D, _D, _I32], ctypes.c_int),
    "pcsf_read_ecm": ([ctypes.c_char_p, _D, _D], ctypes.c_int),
    "pcsf_parse_newick": ([ctypes.c_char_p, ctypes.c_int32, _I32, _I32, _D, ctypes.c_char_p, ctypes.c_int32],
                          ctypes.c_int),
    "pcsf_candidate_regions": ([ctypes.c_char_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                ctypes.c_int32, _I32, _I64, _I64, _I32], ctypes.c_int),
    "pcsf_pack_regions": ([ctypes.c_int32, _I32, ctypes.c_int32, ctypes.POINTER(ctypes.c_char_p),
                           ctypes.POINTER(ctypes.c_char_p), ctypes.c_int64, ctypes.c_int32, _I32, _I64, _I64, _I64,
                           _U8], ctypes.c_int),
    "pcsf_engine_set_exact_threshold": ([_VP, ctypes.c_int64], ctypes.c_int),
    "pcsf_engine_exact_available": ([_VP], ctypes.c_int),
    "pcsf_engine_autotune": ([_VP, _VP, _I32], ctypes.c_int),
    "pcsf_engine_set_tc_shape": ([_VP, ctypes.c_int32], ctypes.c_int),
    "pcsf_engine_set_grad_recompute": ([_VP, ctypes.c_int32], ctypes.c_int),
    "pcsf_engine_set_derivative_mode": ([_VP, ctypes.c_int32], ctypes.c_int),
    "pcsf_engine_grad_scratch_bytes": ([_VP, ctypes.c_int32], ctypes.c_int64),
    "pcsf_engine_tc_shape_times": ([_VP, _D, ctypes.c_int32], ctypes.c_int),
    "pcsf_engine_pt_search": ([_VP, ctypes.c_int32, ctypes.c_int32, _D, _D, _I32], ctypes.c_int),
    "pcsf_branch_counts": ([_VP, _VP, ctypes.c_int32, _D, _D, _D, _I32], ctypes.c_int),
    "pcsf_ell": ([_VP, ctypes.c_int32, ctypes.c_double, _D, _D], ctypes.c_int),
    "pcsf_node_posteriors": ([_VP, _VP, ctypes.c_int32, _D, ctypes.c_int32, _I32, _D, _I32], ctypes.c_int),
    "pcsf_lpr_noalloc": ([_VP, ctypes.c_int32, ctypes.c_double, ctypes.c_int32, _I64, ctypes.c_void_p, ctypes.c_void_p,
                          ctypes.c_void_p], ctypes.c_int),
    "pcsf_bls_columns": ([ctypes.c_int32, _I32, _D, _I32, ctypes.c_int32, ctypes.POINTER(ctypes.c_char_p),
                          ctypes.c_int64, _D], ctypes.c_int),
    "pcsf_simulate": ([ctypes.c_int32, _I32, ctypes.c_int32, _D, _D, ctypes.c_int32, _I64, _I32, _D, ctypes.c_int32,
                       ctypes.c_uint64, ctypes.c_int32, _U8], ctypes.c_int),
}

_LIB = None


def library_path() -> str:
    return _build.LIB


def load_library(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load the in-tree library; raise if it is missing (no fallback exists)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError("phylocsf_gb300: native library %s is missing; run __graft_entry__.build()" % path)
        _build.build()
    lib = ctypes.CDLL(path)
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _LIB = lib
    return lib


def _p(a: np.ndarray, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


def _err(lib, handle=None) -> str:
    m = lib.pcsf_last_error(handle)
    return m.decode() if m else ""


def _check(rc: int, handle=None):
    if rc != PCSF_OK:
        lib = load_library()
        raise EngineError(rc, _err(lib, handle) or STATUS_NAMES.get(rc, "error"))


# --------------------------------------------------------------------------
# host helpers


class Tree:
    """A tree in CamlPaml T order (leaves left to right, internal nodes post-order)."""

    def __init__(self, parent: np.ndarray, branch: np.ndarray, labels: List[str]):
        self.parent = np.ascontiguousarray(parent, np.int32)
        self.branch = np.ascontiguousarray(branch, np.float64)   # [n] (root entry unused)
        self.labels = labels
        self.n = len(self.parent)
        self.nl = (self.n + 1) // 2

    @classmethod
    def from_newick(cls, text: str) -> "Tree":
        lib = load_library()
        cap = 4096
        nl = ctypes.c_int32()
        parent = np.zeros(cap, np.int32)
        branch = np.zeros(cap)
        stride = 128
        labels = ctypes.create_string_buffer(cap * stride)
        _check(lib.pcsf_parse_newick(text.encode(), cap, ctypes.byref(nl), _p(parent, ctypes.c_int32),
                                     _p(branch, ctypes.c_double), labels, stride))
        n = 2 * nl.value - 1
        raw = labels.raw
        labs = [raw[i * stride:(i + 1) * stride].split(b"\0", 1)[0].decode() for i in range(n)]
        return cls(parent[:n].copy(), branch[:n].copy(), labs)

    @classmethod
    def load(cls, path: str) -> "Tree":
        with open(path) as f:
            return cls.from_newick(f.read())

    def scaled(self, factor: float) -> "Tree":
        b = self.branch.copy()
        b[: self.n - 1] *= factor
        return Tree(self.parent.copy(), b, list(self.labels))

    def c_struct(self) -> Tuple[_Tree, tuple]:
        keep = (self.parent, np.ascontiguousarray(self.branch[: self.n - 1], np.float64))
        return _Tree(self.nl, _p(keep[0], ctypes.c_int32), _p(keep[1], ctypes.c_double)), keep


def read_ecm(path: str) -> Tuple[np.ndarray, np.ndarray]:
    """ECM.import_parameters (src/ECM.ml:18-72) through the native reader."""
    lib = load_library()
    S = np.zeros((64, 64))
    pi = np.zeros(64)
    _check(lib.pcsf_read_ecm(path.encode(), _p(S, ctypes.c_double), _p(pi, ctypes.c_double)))
    return S, pi


def candidate_regions(ref: str, frames: int = 1, orf_mode: str = "AsIs", min_codons: int = 25):
    lib = load_library()
    mode = ORF_MODES[orf_mode.lower()]
    cnt = ctypes.c_int32()
    n = len(ref)
    _check(lib.pcsf_candidate_regions(ref.encode(), n, frames, mode, min_codons, 0, None, None, None,
                                      ctypes.byref(cnt)))
    k = cnt.value
    rc = np.zeros(max(k, 1), np.int32)
    lo = np.zeros(max(k, 1), np.int64)
    hi = np.zeros(max(k, 1), np.int64)
    _check(lib.pcsf_candidate_regions(ref.encode(), n, frames, mode, min_codons, k, _p(rc, ctypes.c_int32),
                                      _p(lo, ctypes.c_int64), _p(hi, ctypes.c_int64), ctypes.byref(cnt)))
    return [(bool(rc[i]), int(lo[i]), int(hi[i])) for i in range(k)]


def pack_regions(nl: int, leaf_rows: Sequence[Optional[int]], rows_fwd: Sequence[str], rows_rc: Sequence[str],
                 regions: Sequence[Tuple[bool, int, int]]) -> Tuple[np.ndarray, np.ndarray]:
    """pleaves over many regions: (col_offsets int64[R+1], leaves uint8[total, nl])."""
    lib = load_library()
    lr = np.array([-1 if r is None else r for r in leaf_rows], np.int32)
    fw = (ctypes.c_char_p * len(rows_fwd))(*[s.encode() for s in rows_fwd])
    rv = (ctypes.c_char_p * len(rows_rc))(*[s.encode() for s in rows_rc])
    R = len(regions)
    rc = np.array([1 if r[0] else 0 for r in regions] or [0], np.int32)
    lo = np.array([r[1] for r in regions] or [0], np.int64)
    hi = np.array([r[2] for r in regions] or [0], np.int64)
    offs = np.zeros(R + 1, np.int64)
    L = len(rows_fwd[0])
    _check(lib.pcsf_pack_regions(nl, _p(lr, ctypes.c_int32), len(rows_fwd), fw, rv, L, R, _p(rc, ctypes.c_int32),
                                 _p(lo, ctypes.c_int64), _p(hi, ctypes.c_int64), _p(offs, ctypes.c_int64), None))
    leaves = np.zeros((int(offs[-1]), nl), np.uint8)
    _check(lib.pcsf_pack_regions(nl, _p(lr, ctypes.c_int32), len(rows_fwd), fw, rv, L, R, _p(rc, ctypes.c_int32),
                                 _p(lo, ctypes.c_int64), _p(hi, ctypes.c_int64), _p(offs, ctypes.c_int64),
                                 _p(leaves, ctypes.c_uint8) if leaves.size else None))
    return offs, leaves


# --------------------------------------------------------------------------
# engine


class Batch:
    """Regions resident in device memory (pcsf_batch)."""

    def __init__(self, engine: "Engine", col_offsets: np.ndarray, leaves: np.ndarray):
        self.engine = engine
        lib = engine.lib
        self.col_offsets = np.ascontiguousarray(col_offsets, np.int64)
        self.n_regions = len(self.col_offsets) - 1
        lv = np.ascontiguousarray(leaves, np.uint8)
        if lv.ndim != 2 or lv.shape[1] != engine.nl:
            raise ValueError("leaves must be [total_cols, n_leaves=%d]" % engine.nl)
        self.total_cols = lv.shape[0]
        h = _VP()
        _check(lib.pcsf_batch_create(engine.handle, self.n_regions, _p(self.col_offsets, ctypes.c_int64),
                                     _p(lv, ctypes.c_uint8), ctypes.byref(h)), engine.handle)
        self.handle = h

    def omega_grad(self, batch: Batch, kappa, omega, rho, sigma: float = 1.0, branches: bool = True) -> dict:
        """OmegaModel log-likelihood and its gradient at per-region (kappa, omega, rho): keys lpr,
        d_branch (or None), d_rho, d_kappa, d_omega, status (pcsf_omega_grad)."""
        n = batch.n_regions
        arr = lambda v: np.ascontiguousarray(np.broadcast_to(np.asarray(v, np.float64), (n,)))
        k, o, r = arr(kappa), arr(omega), arr(rho)
        out = {"lpr": np.zeros(n), "d_rho": np.zeros(n), "d_kappa": np.zeros(n), "d_omega": np.zeros(n),
               "status": np.zeros(n, np.int32),
               "d_branch": np.zeros((n, self.tree.n - 1)) if branches else None}
        D = lambda a: _p(a, ctypes.c_double) if a is not None else None
        _check(self.lib.pcsf_omega_grad(self.handle, batch.handle, D(k), D(o), sigma, D(r), D(out["lpr"]),
                                        D(out["d_branch"]), D(out["d_rho"]), D(out["d_kappa"]), D(out["d_omega"]),
                                        _p(out["status"], ctypes.c_int32)), self.handle)
        return out

    def close(self):
        if getattr(self, "handle", None):
            self.engine.lib.pcsf_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Engine:
    """GB300 likelihood engine for one tree and a coding/noncoding model pair."""

    def __init__(self, tree: Tree, S_c=None, pi_c=None, S_n=None, pi_n=None, precision: str = "fp32",
                 Q=None, device: Optional[int] = None):
        self.lib = load_library()
        self.tree = tree
        self.nl = tree.nl
        self.precision = precision
        flags = PREC[precision] | (0 if device is None else (device + 1) << 8)
        ct, keep = tree.c_struct()
        h = _VP()
        if Q == "tree":
            rc = self.lib.pcsf_engine_create_tree(ctypes.byref(ct), flags, ctypes.byref(h))
        elif Q is None:
            arrs = [np.ascontiguousarray(x, np.float64) for x in (S_c, pi_c, S_n, pi_n)]
            rc = self.lib.pcsf_engine_create(ctypes.byref(ct), *[_p(a, ctypes.c_double) for a in arrs], flags,
                                             ctypes.byref(h))
        else:
            arrs = [np.ascontiguousarray(x, np.float64) for x in Q]   # Qc, eqc, priorc, Qn, eqn, priorn
            rc = self.lib.pcsf_engine_create_q(ctypes.byref(ct), *[_p(a, ctypes.c_double) for a in arrs], flags,
                                               ctypes.byref(h))
        _check(rc, None)
        self.handle = h

    @classmethod
    def from_q(cls, tree: Tree, Q_c, eq_c, prior_c, Q_n, eq_n, prior_n, precision: str = "fp32",
               device: Optional[int] = None) -> "Engine":
        return cls(tree, precision=precision, Q=(Q_c, eq_c, prior_c, Q_n, eq_n, prior_n), device=device)

    @classmethod
    def for_tree(cls, tree: Tree, precision: str = "fp64", device: Optional[int] = None) -> "Engine":
        """An engine without fixed models, for the OmegaModel test."""
        return cls(tree, precision=precision, Q="tree", device=device)

    def omega_score(self, batch: Batch, omega_h1: float = 0.2, sigma_h1: float = 0.01) -> np.ndarray:
        """OmegaModel.score (src/OmegaModel.ml:195-219) for every region of the batch."""
        out = np.zeros(batch.n_regions, OMEGA_DTYPE)
        _check(self.lib.pcsf_omega_score(self.handle, batch.handle, omega_h1, sigma_h1,
                                         out.ctypes.data_as(ctypes.POINTER(OmegaResult))), self.handle)
        return out

    def omega_grad(self, batch: Batch, kappa, omega, rho, sigma: float = 1.0, branches: bool = True) -> dict:
        """OmegaModel log-likelihood and its gradient at per-region (kappa, omega, rho): keys lpr,
        d_branch (or None), d_rho, d_kappa, d_omega, status (pcsf_omega_grad)."""
        n = batch.n_regions
        arr = lambda v: np.ascontiguousarray(np.broadcast_to(np.asarray(v, np.float64), (n,)))
        k, o, r = arr(kappa), arr(omega), arr(rho)
        out = {"lpr": np.zeros(n), "d_rho": np.zeros(n), "d_kappa": np.zeros(n), "d_omega": np.zeros(n),
               "status": np.zeros(n, np.int32),
               "d_branch": np.zeros((n, self.tree.n - 1)) if branches else None}
        D = lambda a: _p(a, ctypes.c_double) if a is not None else None
        _check(self.lib.pcsf_omega_grad(self.handle, batch.handle, D(k), D(o), sigma, D(r), D(out["lpr"]),
                                        D(out["d_branch"]), D(out["d_rho"]), D(out["d_kappa"]), D(out["d_omega"]),
                                        _p(out["status"], ctypes.c_int32)), self.handle)
        return out

    def close(self):
        if getattr(self, "handle", None):
            self.lib.pcsf_engine_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- data
    def batch(self, col_offsets, leaves) -> Batch:
        return Batch(self, col_offsets, leaves)

    # ---- PhyloCSFModel.score over many regions
    def score(self, batch: Batch, strategy: int = MLE) -> np.ndarray:
        out = np.zeros(batch.n_regions, RESULT_DTYPE)
        _check(self.lib.pcsf_score(self.handle, batch.handle, strategy,
                                   out.ctypes.data_as(ctypes.POINTER(Result))), self.handle)
        return out

    def score_batch(self, col_offsets, leaves, strategy: int = MLE) -> np.ndarray:
        """One-shot: host buffers in, results out (upload, score, free)."""
        offs = np.ascontiguousarray(col_offsets, np.int64)
        lv = np.ascontiguousarray(leaves, np.uint8)
        out = np.zeros(len(offs) - 1, RESULT_DTYPE)
        _check(self.lib.pcsf_score_batch(self.handle, len(offs) - 1, _p(offs, ctypes.c_int64),
                                         _p(lv, ctypes.c_uint8), strategy,
                                         out.ctypes.data_as(ctypes.POINTER(Result))), self.handle)
        return out

    # ---- lpr_leaves
    def lpr(self, batch: Batch, model: int, rho) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
        r = np.ascontiguousarray(np.broadcast_to(np.asarray(rho, np.float64), (batch.n_regions,)))
        lpr = np.zeros(batch.n_regions)
        elpr = np.zeros(batch.n_regions)
        st = np.zeros(batch.n_regions, np.int32)
        _check(self.lib.pcsf_lpr(self.handle, batch.handle, model, _p(r, ctypes.c_double),
                                 _p(lpr, ctypes.c_double), _p(elpr, ctypes.c_double), _p(st, ctypes.c_int32)),
               self.handle)
        return lpr, elpr, st

    def grad(self, batch: Batch, model: int, rho, branches: bool = True):
        """(lpr, d lpr / d branch or None, d lpr / d rho, status).  branches=False asks for
        d lpr / d rho alone (on a *_direct tensor-core engine: by the tangent pass)."""
        r = np.ascontiguousarray(np.broadcast_to(np.asarray(rho, np.float64), (batch.n_regions,)))
        nbr = self.tree.n - 1
        lpr = np.zeros(batch.n_regions)
        db = np.zeros((batch.n_regions, nbr)) if branches else None
        drho = np.zeros(batch.n_regions)
        st = np.zeros(batch.n_regions, np.int32)
        _check(self.lib.pcsf_grad(self.handle, batch.handle, model, _p(r, ctypes.c_double), _p(lpr, ctypes.c_double),
                                  _p(db, ctypes.c_double) if branches else None, _p(drho, ctypes.c_double),
                                  _p(st, ctypes.c_int32)), self.handle)
        return lpr, db, drho, st

    # ---- outside-pass statistics (PhyloEM sufficient statistics, node posteriors)
    def branch_counts(self, batch: Batch, model: int, rho):
        """(counts [n_regions][n-1][64][64], lpr, status): expected substitution counts of every
        branch summed over each region's columns (PhyloEM.collect_sufficient_statistics)."""
        r = np.ascontiguousarray(np.broadcast_to(np.asarray(rho, np.float64), (batch.n_regions,)))
        nbr = self.tree.n - 1
        counts = np.zeros((batch.n_regions, nbr, 64, 64))
        lpr = np.zeros(batch.n_regions)
        st = np.zeros(batch.n_regions, np.int32)
        _check(self.lib.pcsf_branch_counts(self.handle, batch.handle, model, _p(r, ctypes.c_double),
                                           _p(counts, ctypes.c_double), _p(lpr, ctypes.c_double),
                                           _p(st, ctypes.c_int32)), self.handle)
        return counts, lpr, st

    def ell(self, model: int, rho: float, counts) -> float:
        """PhyloEM.ell of one set of sufficient statistics [n-1][64][64] at tree scale rho."""
        c = np.ascontiguousarray(counts, np.float64)
        out = ctypes.c_double()
        _check(self.lib.pcsf_ell(self.handle, model, float(rho), _p(c, ctypes.c_double), ctypes.byref(out)),
               self.handle)
        return out.value

    def node_posteriors(self, batch: Batch, model: int, rho, nodes):
        """(post [len(nodes)][total_cols][64], status): PhyloLik.node_posterior of the given nodes at
        every column of the batch."""
        r = np.ascontiguousarray(np.broadcast_to(np.asarray(rho, np.float64), (batch.n_regions,)))
        nd = np.ascontiguousarray(nodes, np.int32)
        post = np.zeros((len(nd), batch.total_cols, 64))
        st = np.zeros(batch.n_regions, np.int32)
        _check(self.lib.pcsf_node_posteriors(self.handle, batch.handle, model, _p(r, ctypes.c_double), len(nd),
                                             _p(nd, ctypes.c_int32), _p(post, ctypes.c_double),
                                             _p(st, ctypes.c_int32)), self.handle)
        return post, st

    # ---- model introspection
    def pt(self, model: int, t) -> Tuple[np.ndarray, np.ndarray]:
        tt = np.ascontiguousarray(np.atleast_1d(np.asarray(t, np.float64)))
        P = np.zeros((len(tt), 64, 64))
        st = np.zeros(len(tt), np.int32)
        _check(self.lib.pcsf_engine_pt(self.handle, model, len(tt), _p(tt, ctypes.c_double), _p(P, ctypes.c_double),
                                       _p(st, ctypes.c_int32)), self.handle)
        return P, st

    TC_SHAPES = {0: "alpha kept in registers", 1: "alpha read back"}

    def set_derivative_mode(self, mode: int) -> None:
        """Search derivative of the mle derivative rule: 1 central difference of search values
        (tensor-core default), 0 analytic (tangent pass or adjoint)."""
        _check(self.lib.pcsf_engine_set_derivative_mode(self.handle, mode), self.handle)

    def set_grad_recompute(self, on: bool) -> None:
        """Adjoint: recompute leaf children's partials instead of storing them (identical values)."""
        _check(self.lib.pcsf_engine_set_grad_recompute(self.handle, 1 if on else 0), self.handle)

    def grad_scratch_bytes(self, n_rate_params: int = 0) -> int:
        """Adjoint scratch per CTA under the current setting."""
        v = self.lib.pcsf_engine_grad_scratch_bytes(self.handle, n_rate_params)
        if v < 0:
            raise ValueError("n_rate_params must be 0 or 2")
        return v

    def set_tc_shape(self, shape: int) -> None:
        """Shape of the TF32 tensor-core search kernel (TC_SHAPES; identical values)."""
        _check(self.lib.pcsf_engine_set_tc_shape(self.handle, shape), self.handle)

    def tc_shape_times(self) -> np.ndarray:
        """The autotuner's ms per pass of each search-kernel shape (0 where untimed)."""
        out = np.zeros(len(self.TC_SHAPES))
        _check(self.lib.pcsf_engine_tc_shape_times(self.handle, _p(out, ctypes.c_double), len(out)), self.handle)
        return out

    def pt_search(self, model: int, t) -> Tuple[np.ndarray, np.ndarray]:
        """P(t) as the tensor-core search forms it (TF32 tensor-core engines)."""
        tt = np.ascontiguousarray(t, np.float64)
        P_ = np.zeros((len(tt), 64, 64))
        st = np.zeros(len(tt), np.int32)
        _check(self.lib.pcsf_engine_pt_search(self.handle, model, len(tt), _p(tt, ctypes.c_double),
                                              _p(P_, ctypes.c_double), _p(st, ctypes.c_int32)), self.handle)
        return P_, st

    def eigensystem(self, model: int) -> Tuple[np.ndarray, np.ndarray]:
        U = np.zeros((64, 64))
        lam = np.zeros(64)
        _check(self.lib.pcsf_engine_eigensystem(self.handle, model, _p(U, ctypes.c_double), _p(lam, ctypes.c_double)),
               self.handle)
        return U, lam

    def stats(self) -> dict:
        s = Stats()
        _check(self.lib.pcsf_engine_get_stats(self.handle, ctypes.byref(s)), self.handle)
        out = {}
        for k, _ in Stats._fields_:
            v = getattr(s, k)
            out[k] = list(v) if not isinstance(v, (int, float)) else v
        return out

    def stream_handle(self) -> int:
        """The engine's cudaStream_t as an integer (for event timing on that stream)."""
        h = _VP()
        _check(self.lib.pcsf_engine_stream(self.handle, ctypes.byref(h)), self.handle)
        return int(h.value or 0)

    def reset_stats(self):
        _check(self.lib.pcsf_engine_reset_stats(self.handle), self.handle)

    def set_exact_threshold(self, units: int):
        """Regions with columns x (n_leaves - 2) >= units take their returned values from the
        float-float kernel (0: all regions)."""
        _check(self.lib.pcsf_engine_set_exact_threshold(self.handle, int(units)), self.handle)

    def autotune(self, batch: Batch) -> int:
        """Time the compensated FP32 kernel's column tiles (and, on TF32 tensor-core engines,
        the search kernel's shapes) on a sample of the batch, keep the fastest for this
        engine; returns the chosen tile."""
        t = ctypes.c_int32()
        _check(self.lib.pcsf_engine_autotune(self.handle, batch.handle, ctypes.byref(t)), self.handle)
        return t.value

    @property
    def exact_available(self) -> bool:
        return bool(self.lib.pcsf_engine_exact_available(self.handle))


# --------------------------------------------------------------------------
# PhyloCSFModel-style entry points


def make(s1, pi1, s2, pi2, tree: Tree, precision: str = "fp32") -> Engine:
    """PhyloCSFModel.make (PhyloCSFModel.ml:107-110): coding and noncoding models on one tree."""
    return Engine(tree, s1, pi1, s2, pi2, precision=precision)


def score(strategy: int, model: Engine, leaves: np.ndarray) -> np.void:
    """PhyloCSFModel.score for one region's leaves ([ncols, nl] uint8)."""
    lv = np.ascontiguousarray(leaves, np.uint8).reshape(-1, model.nl)
    return model.score_batch(np.array([0, lv.shape[0]], np.int64), lv, strategy)[0]
