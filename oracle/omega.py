"""OmegaModel (dN/dS) test restated on the CPU -- TEST INFRASTRUCTURE ONLY.

Restates src/OmegaModel.ml (paths relative to the mlin/PhyloCSF tree):
  - F3x4 codon frequencies pi_exprs ........ OmegaModel.ml:21-40
  - parametric codon Q (kappa, omega) ...... OmegaModel.ml:42-74
  - mean-rate scale ........................ OmegaModel.ml:76-80
  - F3x4 counts from the leaves ............ OmegaModel.ml:102-134
  - priors on rho and kappa ................ OmegaModel.ml:146-157
  - kr_map (3 rounds of rho then kappa) .... OmegaModel.ml:160-190
  - H1 vs H0 score ......................... OmegaModel.ml:195-219
The likelihood evaluations use the C oracle (oracle.OModel / lpr_leaves); the
maximisations use the oracle's find_init + Brent through a small Python driver
around orc_lpr_leaves.  The root prior is the model's equilibrium, normalised
(PhyloModel.prior without an explicit prior, PhyloModel.ml:25-29).
"""
from __future__ import annotations

import math
from typing import Sequence, Tuple

import numpy as np

from . import oracle as O

TRANSLATION = "KNKNTTTTRSRSIIMIQHQHPPPPRRRRLLLLEDEDAAAAGGGGVVVV*Y*YSSSS*CWCLFLF"
STOPS = (48, 50, 56)          # TAA TAG TGA


def codon_nucs(i: int) -> Tuple[int, int, int]:
    return i // 16, (i // 4) % 4, i % 4


def omega_pi(q: Sequence[float]) -> np.ndarray:
    """pi_exprs: F3x4 frequencies relative to T per position, stop mass damped by sigma in the denominator."""
    sigma = q[2]

    def sc(i):
        out = 1.0
        for pos, n in enumerate(codon_nucs(i)):
            base = 3 + 3 * pos
            num = 1.0 if n == 3 else q[base + n]
            den = q[base] + (q[base + 1] + (q[base + 2] + 1.0))
            out *= num / den
        return out

    denom = 1.0 - (1.0 - sigma) * (sc(48) + (sc(50) + sc(56)))
    return np.array([sc(i) / denom for i in range(64)])


def omega_q(q: Sequence[float]) -> Tuple[np.ndarray, np.ndarray]:
    """(Q scaled to mean rate 1, pi) for q = [kappa, omega, sigma, 9 frequencies]."""
    kappa, omega = q[0], q[1]
    pi = omega_pi(q)
    Q = np.zeros((64, 64))
    for i in range(64):
        ni = codon_nucs(i)
        for j in range(64):
            if i == j:
                continue
            nj = codon_nucs(j)
            diffs = [(a, b) for a, b in zip(ni, nj) if a != b]
            if len(diffs) != 1:
                continue
            a, b = diffs[0]
            transition = {a, b} in ({0, 2}, {1, 3})          # A<->G, C<->T
            kp = kappa if transition else 1.0
            nonsyn = (i not in STOPS and j not in STOPS) and TRANSLATION[i] != TRANSLATION[j]
            op = omega if nonsyn else 1.0
            Q[i, j] = pi[j] * (kp * op)
    for i in range(64):
        Q[i, i] = -Q[i].sum()
    scale = -(pi * np.diag(Q)).sum()
    return Q / scale, pi


def f3x4_from_leaves(leaves: np.ndarray) -> np.ndarray:
    """update_f3x4: nucleotide counts per codon position (pseudocount 1), relative to T."""
    counts = np.ones((3, 4))
    lv = np.asarray(leaves).ravel()
    lv = lv[(lv >= 0) & (lv < 64)]
    for pos, div in enumerate((16, 4, 1)):
        nuc = (lv // div) % 4
        counts[pos] += np.bincount(nuc, minlength=4)
    f = np.zeros(9)
    for pos in range(3):
        f[3 * pos: 3 * pos + 3] = counts[pos, :3] / counts[pos, 3]
    return f


def lpr_rho(x: float) -> float:
    """half_cauchy_lpdf ~mode:1 ~scale:0.5 (OmegaModel.ml:148-156)."""
    mode, scale = 1.0, 0.5
    numer = 1.0 / (math.pi * scale * (1.0 + ((x - mode) / scale) ** 2.0))
    cdf = math.atan((0.0 - mode) / scale) / math.pi + 0.5
    return math.log(numer) - math.log(1.0 - cdf)


def lpr_kappa(k: float) -> float:
    """log Gamma(a=7, scale b=0.25) density at k - 1 + DBL_EPSILON (OmegaModel.ml:157)."""
    x = k - 1.0 + 2.220446049250313e-16
    a, b = 7.0, 0.25
    if x <= 0:
        return -math.inf
    return (a - 1.0) * math.log(x) - x / b - math.lgamma(a) - a * math.log(b)


class _Objective:
    def __init__(self, otree, leaves):
        self.otree = otree
        self.leaves = leaves
        self.models = {}
        self.evals = 0

    def model(self, q):
        key = tuple(q)
        if key not in self.models:
            Q, pi = omega_q(q)
            self.models[key] = O.OModel(Q, pi, pi / pi.sum())
        return self.models[key]

    def lpr(self, q, rho):
        self.evals += 1
        return O.lpr_leaves(self.model(q), self.otree, rho, self.leaves)[0]


GOLDEN = 0.3819660
SQRT_EPS = 1.4901161193847656e-08


def _uniform(state):
    state[0] = (state[0] + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
    z = state[0]
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
    z = z ^ (z >> 31)
    return (z >> 11) * (1.0 / 9007199254740992.0)


def maximize(f, init, lo, hi, accuracy=0.01, maxtries=250):
    """PhyloCSFModel.maximize_lpr with find_init + Brent (the same steps as phylocsf_oracle.c)."""
    width = math.log(hi) - math.log(lo)
    flo, fhi = f(lo), f(hi)
    x, fx = init, f(init)
    i, st = 0, [0]
    while i < maxtries and (fx <= flo or fx <= fhi):
        x = math.exp(math.log(lo) + _uniform(st) * width)
        fx = f(x)
        i += 1
    if i == maxtries:
        x = lo if flo > fhi else hi
    if not (lo < x < hi):
        return x, f(x)
    blo, bhi, bx = lo, hi, x
    bflo, bfhi, bfx = -f(lo), -f(hi), -f(x)
    if not (bfx < bflo and bfx < bfhi):
        raise RuntimeError("endpoints do not enclose a minimum")
    v = w = blo + GOLDEN * (bhi - blo)
    fv = fw = -f(v)
    d_keep = e_keep = 0.0
    for _ in range(1000):
        z, fz = bx, bfx
        d, e = e_keep, d_keep
        tol = SQRT_EPS * abs(z)
        mid = 0.5 * (blo + bhi)
        left, right = z - blo, bhi - z
        p = q = r = 0.0
        if abs(e) > tol:
            r = (z - w) * (fz - fv)
            q = (z - v) * (fz - fw)
            p = (z - v) * q - (z - w) * r
            q = 2.0 * (q - r)
            if q > 0:
                p = -p
            else:
                q = -q
            r = e
            e = d
        if abs(p) < abs(0.5 * q * r) and p < q * left and p < q * right:
            d = p / q
            u = z + d
            if (u - blo) < 2 * tol or (bhi - u) < 2 * tol:
                d = tol if z < mid else -tol
        else:
            e = (bhi - z) if z < mid else -(z - blo)
            d = GOLDEN * e
        u = z + d if abs(d) >= tol else z + (tol if d > 0 else -tol)
        e_keep, d_keep = e, d
        fu = -f(u)
        if fu <= bfx:
            if u < bx:
                bhi, bfhi = bx, bfx
            else:
                blo, bflo = bx, bfx
            v, fv, w, fw, bx, bfx = w, fw, bx, bfx, u, fu
        else:
            if u < bx:
                blo, bflo = u, fu
            else:
                bhi, bfhi = u, fu
            if fu <= fw or w == bx:
                v, fv, w, fw = w, fw, u, fu
            elif fu <= fv or v == bx or v == w:
                v, fv = u, fu
        if not ((bhi - blo) / bx > accuracy):
            break
    return bx, f(bx)


def kr_map(obj: _Objective, q, rho):
    q = list(q)
    lpr = None
    for _ in range(3):
        rho, _ = maximize(lambda r: lpr_rho(r) + obj.lpr(q, r), rho, 0.001, 10.0)
        qk = list(q)

        def fk(k):
            qk[0] = k
            return lpr_kappa(k) + obj.lpr(qk, rho)

        kappa, lpr = maximize(fk, q[0], 1.0, 10.0)
        q[0] = kappa
    return q, rho, lpr


def score(tree: O.Tree, leaves: np.ndarray, omega_h1: float = 0.2, sigma_h1: float = 0.01):
    """OmegaModel.score: (score in decibans, lpr_H0, lpr_H1, q0, rho0, q1, rho1, evals)."""
    ot = O.OTree(tree)
    obj = _Objective(ot, np.ascontiguousarray(leaves, np.int32))
    q0 = [2.5, 1.0, 1.0] + list(f3x4_from_leaves(leaves))
    q0, rho0, lpr0 = kr_map(obj, q0, 1.0)
    q1 = list(q0)
    q1[1], q1[2] = omega_h1, sigma_h1
    q1, rho1, lpr1 = kr_map(obj, q1, rho0)
    return 10.0 * (lpr1 - lpr0) / math.log(10.0), lpr0, lpr1, q0, rho0, q1, rho1, obj.evals
