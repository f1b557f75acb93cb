"""Seeded synthetic alignments for the benchmark and parity workloads.

Columns are simulated along the tree as PhyloModel.simulate does
(lib/CamlPaml/PhyloModel.ml:38-54: root ~ prior, child ~ P row of the parent
state) with branch lengths at rho = 1, rejecting a stop codon in leaf 0 as
testSim does (src/testSim.ml:52-65).  Gaps / N and entirely missing species
are then marginalised per region.  The column simulation runs in the native
helper ``pcsf_simulate`` (multithreaded, deterministic per column).
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import engine as E

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
# parameter sets shipped with the package: trees in CamlPaml T order and the coding /
# noncoding ECMs, parsed from PhyloCSF_Parameters by tests/golden/make_fixtures.py
PARAMS_DIR = os.path.join(HERE, "params")


@dataclass
class ParamSet:
    name: str
    tree: E.Tree
    S_c: np.ndarray
    pi_c: np.ndarray
    S_n: np.ndarray
    pi_n: np.ndarray


def load_params(name: str, params_dir: Optional[str] = None) -> ParamSet:
    """A parameter set (tree + coding/noncoding ECMs) shipped with the package."""
    d = np.load(os.path.join(params_dir or PARAMS_DIR, name + ".npz"))

    def full(tri):
        S = np.zeros((64, 64))
        il = np.tril_indices(64, -1)
        S[il] = tri
        return S + S.T

    labels = [str(x) for x in d["labels"]]
    tree = E.Tree(d["parent"].astype(np.int32), d["branch"].astype(np.float64), labels)
    return ParamSet(name, tree, full(d["S_c"]), d["pi_c"].copy(), full(d["S_n"]), d["pi_n"].copy())


def q_matrix(S: np.ndarray, pi: np.ndarray) -> np.ndarray:
    """q_ij = s_ij pi_j, zero row sums, mean rate 1 (PhyloCSFModel.ml:11-30)."""
    Q = S * pi[None, :]
    np.fill_diagonal(Q, 0.0)
    np.fill_diagonal(Q, -Q.sum(1))
    return Q / (-(pi * np.diag(Q)).sum())


def p_matrices(S: np.ndarray, pi: np.ndarray, t: np.ndarray) -> np.ndarray:
    """P(t) for each t (numpy eigh of the symmetrised Q); rows clamped >= 0 and renormalised."""
    Q = q_matrix(S, pi)
    sq = np.sqrt(pi)
    A = sq[:, None] * Q / sq[None, :]
    lam, U = np.linalg.eigh(0.5 * (A + A.T))
    out = np.empty((len(t), 64, 64))
    for i, ti in enumerate(t):
        M = (U * np.exp(lam * ti)) @ U.T
        P = M * sq[None, :] / sq[:, None]
        P = np.maximum(P, 0.0)
        out[i] = P / P.sum(1, keepdims=True)
    return out


def simulate(ps: ParamSet, lengths: np.ndarray, models: np.ndarray, gap_frac: Optional[np.ndarray], seed: int,
             reject_stop_leaf0: bool = True, threads: int = 0, rho: float = 1.0):
    """Simulate regions: returns (col_offsets int64[R+1], leaves uint8[total, nl])."""
    P, prior = simulation_inputs(ps, rho)
    return simulate_with(ps.tree, P, prior, lengths, models, gap_frac, seed, reject_stop_leaf0, threads)


def simulate_with(tree, P: np.ndarray, prior: np.ndarray, lengths: np.ndarray, models: np.ndarray,
                  gap_frac: Optional[np.ndarray], seed: int, reject_stop_leaf0: bool = True, threads: int = 0):
    """Simulate regions from explicit models: P [n_models][nbr][64][64], prior [n_models][64]."""
    lib = E.load_library()
    P = np.ascontiguousarray(P, np.float64)
    prior = np.ascontiguousarray(prior, np.float64)
    offs = np.zeros(len(lengths) + 1, np.int64)
    offs[1:] = np.cumsum(lengths)
    leaves = np.empty((int(offs[-1]), tree.nl), np.uint8)
    models = np.ascontiguousarray(models, np.int32)
    gf = None if gap_frac is None else np.ascontiguousarray(gap_frac, np.float64)
    rc = lib.pcsf_simulate(tree.nl, E._p(tree.parent, ctypes.c_int32), P.shape[0], E._p(P, ctypes.c_double),
                           E._p(prior, ctypes.c_double), len(lengths), E._p(offs, ctypes.c_int64),
                           E._p(models, ctypes.c_int32), None if gf is None else E._p(gf, ctypes.c_double),
                           1 if reject_stop_leaf0 else 0, seed, threads,
                           E._p(leaves, ctypes.c_uint8) if leaves.size else E._p(np.zeros(1, np.uint8), ctypes.c_uint8))
    E._check(rc)
    return offs, leaves


def gap_fractions(rng: np.random.Generator, nreg: int, nl: int, lo: float, hi: float, missing_max: float = 0.0):
    """Per (region, species) gap probability ~ U(lo, hi); a U(0, missing_max)
    fraction of each region's species (never leaf 0, the reference row) is
    missing entirely (probability 1)."""
    gf = rng.uniform(lo, hi, size=(nreg, nl))
    if missing_max > 0:
        for r in range(nreg):
            k = int(round(rng.uniform(0.0, missing_max) * nl))
            if k:
                gone = rng.choice(np.arange(1, nl), size=min(k, nl - 1), replace=False)
                gf[r, gone] = 1.0
    return gf


@dataclass
class WorkloadSpec:
    """A workload before its columns are simulated: region lengths (as column offsets),
    per-region model (0 coding, 1 noncoding), per (region, species) gap probability and
    the simulation seed.  Building it needs numpy only."""
    name: str
    params: ParamSet
    col_offsets: np.ndarray
    models: np.ndarray
    gap_frac: np.ndarray
    seed: int
    strategy: int

    @property
    def n_regions(self) -> int:
        return len(self.col_offsets) - 1

    @property
    def total_cols(self) -> int:
        return int(self.col_offsets[-1])


@dataclass
class Workload:
    name: str
    params: ParamSet
    col_offsets: np.ndarray
    leaves: np.ndarray
    models: np.ndarray
    strategy: int

    @property
    def n_regions(self) -> int:
        return len(self.col_offsets) - 1

    @property
    def total_cols(self) -> int:
        return int(self.col_offsets[-1])


def realize(spec: WorkloadSpec) -> Workload:
    """Simulate the columns of a workload (native, multithreaded; deterministic per column)."""
    lengths = np.diff(spec.col_offsets)
    offs, lv = simulate(spec.params, lengths, spec.models, spec.gap_frac, spec.seed)
    return Workload(spec.name, spec.params, offs, lv, spec.models, spec.strategy)


def simulation_inputs(ps: ParamSet, rho: float = 1.0):
    """What the column simulation draws from: per model the P(t) of every branch at tree
    scale rho, [2][nbr][64][64], and the root priors [2][64]."""
    nbr = ps.tree.n - 1
    t = ps.tree.branch[:nbr] * rho
    P = np.ascontiguousarray(np.stack([p_matrices(ps.S_c, ps.pi_c, t), p_matrices(ps.S_n, ps.pi_n, t)]))
    prior = np.ascontiguousarray(np.stack([ps.pi_c, ps.pi_n]))
    return P, prior


def log_uniform_lengths(rng, n, lo, hi):
    return np.floor(np.exp(rng.uniform(np.log(lo), np.log(hi), size=n))).astype(np.int64).clip(lo, hi)


def _offsets(lengths) -> np.ndarray:
    offs = np.zeros(len(lengths) + 1, np.int64)
    offs[1:] = np.cumsum(lengths)
    return offs


def spec_12flies_fixed(seed: int = 0) -> WorkloadSpec:
    """One alignment of 300 codons on 12flies from the noncoding ECM, 10% gaps per species; fixed."""
    ps = load_params("12flies")
    gf = np.full((1, ps.tree.nl), 0.10)
    return WorkloadSpec("12flies_fixed_1x300", ps, _offsets([300]), np.array([1], np.int32), gf, seed, E.FIXED)


def spec_58mammals_mle(n_regions: int = 10000, seed: int = 0) -> WorkloadSpec:
    """58mammals, mle: half coding / half noncoding, lengths log-uniform 50-3000 codons,
    per-species gap+N fraction U(5%,40%), 0-20% of species entirely missing."""
    ps = load_params("58mammals")
    rng = np.random.default_rng(seed)
    lengths = log_uniform_lengths(rng, n_regions, 50, 3000)
    models = (np.arange(n_regions) % 2).astype(np.int32)    # 0 coding, 1 noncoding
    gf = gap_fractions(rng, n_regions, ps.tree.nl, 0.05, 0.40, 0.20)
    return WorkloadSpec("58mammals_mle_%dregions" % n_regions, ps, _offsets(lengths), models, gf, seed, E.MLE)


def spec_120mammals_fixed(total_cols: int = 2_000_000, seed: int = 0) -> WorkloadSpec:
    """120mammals at rho = 1: alignments log-uniform 100-5000 codons totalling ~total_cols, 1:1 models."""
    ps = load_params("120mammals")
    rng = np.random.default_rng(seed)
    lens = []
    s = 0
    while s < total_cols:
        L = int(log_uniform_lengths(rng, 1, 100, 5000)[0])
        L = min(L, total_cols - s) if total_cols - s >= 100 else L
        lens.append(L)
        s += L
    lengths = np.array(lens, np.int64)
    models = (np.arange(len(lengths)) % 2).astype(np.int32)
    gf = gap_fractions(rng, len(lengths), ps.tree.nl, 0.05, 0.40, 0.0)
    return WorkloadSpec("120mammals_fixed_%dcols" % total_cols, ps, _offsets(lengths), models, gf, seed, E.FIXED)


def spec_100vertebrates_mle(n_regions: int = 20000, seed: int = 0) -> WorkloadSpec:
    """100vertebrates, mle: lengths log-uniform 30-10000 codons, coding:noncoding 1:3, 5-40% gaps."""
    ps = load_params("100vertebrates")
    rng = np.random.default_rng(seed)
    lengths = log_uniform_lengths(rng, n_regions, 30, 10000)
    models = (rng.random(n_regions) >= 0.25).astype(np.int32)
    gf = gap_fractions(rng, n_regions, ps.tree.nl, 0.05, 0.40, 0.0)
    return WorkloadSpec("100vertebrates_mle_%dregions" % n_regions, ps, _offsets(lengths), models, gf, seed, E.MLE)


def workload_12flies_fixed(seed: int = 0) -> Workload:
    return realize(spec_12flies_fixed(seed))


def workload_58mammals_mle(n_regions: int = 10000, seed: int = 0) -> Workload:
    return realize(spec_58mammals_mle(n_regions, seed))


def workload_120mammals_fixed(total_cols: int = 2_000_000, seed: int = 0) -> Workload:
    return realize(spec_120mammals_fixed(total_cols, seed))


def workload_100vertebrates_mle(n_regions: int = 20000, seed: int = 0) -> Workload:
    return realize(spec_100vertebrates_mle(n_regions, seed))


_NT = np.frombuffer(b"ACGT", np.uint8)


def nucleotide_rows(codes: np.ndarray, ref_leaf: int = 0) -> list:
    """Codon-level leaf codes [L][nl] -> nl nucleotide rows of 3L characters: codon
    16 n1 + 4 n2 + n3 as its three bases, a marginalised codon as '---' (as 'NNN' in the
    reference row, which the driver requires ungapped)."""
    L, nl = codes.shape
    c = codes.astype(np.int64)
    nt = np.empty((nl, L, 3), np.uint8)
    ok = c < 64
    for k, sh in enumerate((4, 2, 0)):
        nt[:, :, k] = np.where(ok, _NT[(np.where(ok, c, 0) >> sh) & 3], ord("-")).T
    nt[ref_leaf][~ok[:, ref_leaf]] = ord("N")
    return [nt[l].tobytes().decode() for l in range(nl)]


def workload_100vertebrates_6frame(n_regions: int = 20000, seed: int = 0, min_codons: int = 25) -> Workload:
    """Six-frame scoring on 100vertebrates (the batching configuration): alignments of
    log-uniform 30-10,000 codons simulated from the coding / noncoding ECMs at 1:3 with
    5-40% gaps per species, written out as nucleotide rows; every alignment's candidate
    regions in all six frames (AsIs: each frame's whole length) are enumerated and packed
    by the native pcsf_candidate_regions / pcsf_pack_regions, the MFA driver's path
    (src/PhyloCSF.ml:134-246).  Regions of one alignment are consecutive."""
    ps = load_params("100vertebrates")
    nl = ps.tree.nl
    rng = np.random.default_rng(seed)
    n_aln = max(1, -(-n_regions // 6))
    lengths = log_uniform_lengths(rng, n_aln, 30, 10000)
    models = (rng.random(n_aln) >= 0.25).astype(np.int32)
    gf = gap_fractions(rng, n_aln, nl, 0.05, 0.40, 0.0)
    aoffs, codes = simulate(ps, lengths, models, gf, seed)
    comp = str.maketrans("ACGTN-", "TGCAN-")
    all_offs, all_leaves, region_models = [np.zeros(1, np.int64)], [], []
    base = 0
    for a in range(n_aln):
        rows = nucleotide_rows(codes[aoffs[a]:aoffs[a + 1]])
        rows_rc = [r.translate(comp)[::-1] for r in rows]
        regs = E.candidate_regions(rows[0], 6, "AsIs", min_codons)
        o, lv = E.pack_regions(nl, list(range(nl)), rows, rows_rc, regs)
        all_offs.append(o[1:] + base)
        all_leaves.append(lv)
        region_models.extend([models[a]] * len(regs))
        base += int(o[-1])
    offs = np.concatenate(all_offs)
    leaves = np.concatenate(all_leaves) if all_leaves else np.zeros((0, nl), np.uint8)
    return Workload("100vertebrates_6frame_%dregions" % (len(offs) - 1), ps, offs, leaves,
                    np.array(region_models, np.int32), E.MLE)


# ---------------------------------------------------------------- OmegaModel workloads
_GENETIC_CODE = "KNKNTTTTRSRSIIMIQHQHPPPPRRRRLLLLEDEDAAAAGGGGVVVV*Y*YSSSS*CWCLFLF"
_STOPS = (48, 50, 56)


def omega_rate_matrix(kappa: float, omega: float, sigma: float = 1.0, f3x4: Optional[np.ndarray] = None):
    """(Q, pi) of the OmegaModel's parametric codon model (src/OmegaModel.ml:21-80): F3x4 codon
    frequencies (9 values, each position's A, C, G relative to T; default uniform) with the stop
    codons' mass damped by sigma; q_ij = pi_j x kappa (transitions) x omega (non-synonymous) between
    codons one nucleotide apart; Q scaled to mean rate 1."""
    f = np.ones(9) if f3x4 is None else np.asarray(f3x4, np.float64)
    nuc = np.array([[i // 16, (i // 4) % 4, i % 4] for i in range(64)])
    rel = np.ones((3, 4))
    rel[:, :3] = f.reshape(3, 3)
    pos = rel / rel.sum(axis=1, keepdims=True)
    sc = pos[0][nuc[:, 0]] * pos[1][nuc[:, 1]] * pos[2][nuc[:, 2]]
    pi = sc / (1.0 - (1.0 - sigma) * sc[list(_STOPS)].sum())
    diff = nuc[:, None, :] != nuc[None, :, :]
    one = diff.sum(axis=2) == 1
    a = np.where(diff, nuc[:, None, :], -1).max(axis=2)
    b = np.where(diff, nuc[None, :, :], -1).max(axis=2)
    transition = ((a == 0) & (b == 2)) | ((a == 2) & (b == 0)) | ((a == 1) & (b == 3)) | ((a == 3) & (b == 1))
    aa = np.array(list(_GENETIC_CODE))
    stop = np.isin(np.arange(64), _STOPS)
    nonsyn = (~stop[:, None]) & (~stop[None, :]) & (aa[:, None] != aa[None, :])
    Q = np.where(one, pi[None, :] * np.where(transition, kappa, 1.0) * np.where(nonsyn, omega, 1.0), 0.0)
    np.fill_diagonal(Q, -Q.sum(axis=1))
    return Q / (-(pi * np.diag(Q)).sum()), pi


def p_matrices_q(Q: np.ndarray, pi: np.ndarray, t: np.ndarray) -> np.ndarray:
    """P(t) of a reversible Q for each t (symmetrised eigensystem); rows clamped and renormalised."""
    sq = np.sqrt(pi)
    A = sq[:, None] * Q / sq[None, :]
    lam, U = np.linalg.eigh(0.5 * (A + A.T))
    out = np.empty((len(t), 64, 64))
    for i, ti in enumerate(t):
        M = (U * np.exp(lam * ti)) @ U.T
        P = np.maximum(M * sq[None, :] / sq[:, None], 0.0)
        out[i] = P / P.sum(1, keepdims=True)
    return out


@dataclass
class OmegaWorkload:
    name: str
    tree: E.Tree
    col_offsets: np.ndarray
    leaves: np.ndarray
    omega: np.ndarray        # per region, the omega it was simulated at
    kappa: float
    sigma: float

    @property
    def n_regions(self) -> int:
        return len(self.col_offsets) - 1

    @property
    def total_cols(self) -> int:
        return int(self.col_offsets[-1])


def workload_100vertebrates_omega(n_alignments: int = 2000, seed: int = 0, n_omega: int = 16,
                                  lengths: Optional[np.ndarray] = None) -> OmegaWorkload:
    """The differentiation configuration: alignments of log-uniform 200-2,000 codons on
    100vertebrates simulated under the OmegaModel at kappa = 2.5, sigma = 1, uniform F3x4 and
    omega log-uniform in [0.05, 2] (n_omega levels), with 5-20 % gaps per species."""
    ps = load_params("100vertebrates")
    tree = ps.tree
    rng = np.random.default_rng(seed)
    L = log_uniform_lengths(rng, n_alignments, 200, 2000) if lengths is None else np.asarray(lengths, np.int64)
    levels = np.exp(np.linspace(np.log(0.05), np.log(2.0), n_omega))
    which = rng.integers(0, n_omega, size=len(L)).astype(np.int32)
    gf = gap_fractions(rng, len(L), tree.nl, 0.05, 0.20, 0.0)
    nbr = tree.n - 1
    P = np.empty((n_omega, nbr, 64, 64))
    prior = np.empty((n_omega, 64))
    for k, w in enumerate(levels):
        Q, pi = omega_rate_matrix(2.5, w, 1.0)
        P[k] = p_matrices_q(Q, pi, tree.branch[:nbr])
        prior[k] = pi / pi.sum()
    offs, lv = simulate_with(tree, P, prior, L, which, gf, seed)
    return OmegaWorkload("100vertebrates_omega_%dalignments" % len(L), tree, offs, lv, levels[which], 2.5, 1.0)
