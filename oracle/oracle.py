"""CPU oracle for the PhyloCSF likelihood path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
may import this module.  The product package (``phylocsf_gb300``) never imports
it; it is the checker, never the thing measured or shipped.

Two layers:

* pure-Python restatements of the reference's host-side parsing and region
  logic (paths relative to the mlin/PhyloCSF tree):

  - Newick lexer/parser ............ lib/CamlPaml/NewickLexer.mll:1-14, NewickParser.mly:1-25
  - tree numbering (T.of_newick) ... lib/CamlPaml/T.ml:57-112
  - ECM reader ..................... src/ECM.ml:18-72
  - Codon64 index / is ............. lib/CamlPaml/Code.ml:18-30,138-141
  - MFA reader, ref-gap removal .... src/PhyloCSF.ml:83-132
  - find_orfs / candidate_regions .. src/PhyloCSF.ml:134-217
  - pleaves (leaf encoding) ........ src/PhyloCSF.ml:219-246

* ctypes bindings to ``phylocsf_oracle.c`` (the FP64 numeric restatement:
  Q build, eigendecomposition, P(t), dense pruning, find_init + Brent, LLR,
  outside pass, node posteriors, expected branch counts and ELL).
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
from dataclasses import dataclass
from typing import List, Optional, Sequence, Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")
MARGINALIZE = -1

# --------------------------------------------------------------------------
# Build


def build(force: bool = False) -> str:
    """Compile phylocsf_oracle.c with gcc into oracle/_build/liboracle.so."""
    src = os.path.join(HERE, "phylocsf_oracle.c")
    os.makedirs(BUILD_DIR, exist_ok=True)
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        tmp = LIB_PATH + ".tmp%d" % os.getpid()
        subprocess.check_call(["gcc", "-O3", "-fPIC", "-shared", "-o", tmp, src, "-lm"])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


# --------------------------------------------------------------------------
# Newick (NewickLexer.mll / NewickParser.mly) and T.of_newick


@dataclass
class NewickNode:
    children: list
    label: str
    branch: Optional[float]


def _newick_tokens(text: str):
    i, n = 0, len(text)
    digits = set("0123456789.")
    labchars = set("ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789_.")
    while i < n:
        ch = text[i]
        if ch in " \t\r\n;":
            i += 1
        elif ch in "(),:":
            yield ch, None
            i += 1
        elif ch in labchars:
            # longest match; on a tie the BRANCHLEN rule (listed first) wins
            j = i
            while j < n and text[j] in labchars:
                j += 1
            k = i
            while k < n and text[k] in digits:
                k += 1
            if k >= j:
                yield "LEN", float(text[i:k])
                i = k
            else:
                yield "LABEL", text[i:j]
                i = j
        else:
            raise ValueError("Newick: unexpected character %r" % ch)


def parse_newick(text: str) -> NewickNode:
    toks = list(_newick_tokens(text))
    pos = [0]

    def peek():
        return toks[pos[0]][0] if pos[0] < len(toks) else "EOF"

    def take(kind):
        if peek() != kind:
            raise ValueError("Newick: expected %s, got %s" % (kind, peek()))
        t = toks[pos[0]]
        pos[0] += 1
        return t[1]

    def label():
        if peek() == "LABEL":
            lbl = take("LABEL")
            if peek() == ":":
                take(":")
                return lbl, take("LEN")
            return lbl, None
        take(":")
        return "", take("LEN")

    def node():
        if peek() == "(":
            take("(")
            subs = [node()]
            while peek() == ",":
                take(",")
                subs.append(node())
            take(")")
            if peek() in ("LABEL", ":"):
                lbl, bl = label()
                return NewickNode(subs, lbl, bl)
            return NewickNode(subs, "", None)
        lbl, bl = label()
        return NewickNode([], lbl, bl)

    root = node()
    if peek() != "EOF":
        raise ValueError("Newick: trailing tokens")
    return root


@dataclass
class Tree:
    """T.t: leaves 0..nl-1 left to right, internal nodes numbered post-order, root n-1."""
    labels: List[str]
    parent: np.ndarray   # int32 [n], -1 at the root
    lchild: np.ndarray   # int32 [n], -1 at leaves
    rchild: np.ndarray   # int32 [n]
    branch: np.ndarray   # float64 [n] (entry n-1 is the root's, unused)

    @property
    def n(self) -> int:
        return len(self.parent)

    @property
    def nl(self) -> int:
        return (self.n + 1) // 2


def tree_of_newick(nt: NewickNode) -> Tree:
    leaves: List[NewickNode] = []

    def find_leaves(x):
        if not x.children:
            leaves.append(x)
        elif len(x.children) == 2:
            find_leaves(x.children[0])
            find_leaves(x.children[1])
        else:
            raise ValueError("T.of_newick: input is not a rooted, bifurcating tree")

    find_leaves(nt)
    nl = len(leaves)
    n = 2 * nl - 1
    labels = [""] * n
    parent = np.full(n, -1, np.int32)
    lch = np.full(n, -1, np.int32)
    rch = np.full(n, -1, np.int32)
    branch = np.full(n, np.nan)
    leaf_id = {id(x): i for i, x in enumerate(leaves)}
    nxt = [nl - 1]

    def fill(x):
        if not x.children:
            i = leaf_id[id(x)]
        else:
            lc = fill(x.children[0])
            rc = fill(x.children[1])
            nxt[0] += 1
            i = nxt[0]
            parent[lc] = i
            parent[rc] = i
            lch[i] = lc
            rch[i] = rc
        labels[i] = x.label
        branch[i] = x.branch if x.branch is not None else np.nan
        return i

    root = fill(nt)
    assert root == n - 1
    return Tree(labels, parent, lch, rch, branch)


def load_tree(path: str) -> Tree:
    with open(path) as f:
        return tree_of_newick(parse_newick(f.read()))


# --------------------------------------------------------------------------
# Genetic code and ECM reader

DNA_INDEX = {"A": 0, "C": 1, "G": 2, "T": 3, "a": 0, "c": 1, "g": 2, "t": 3}
_COMP = {"A": "T", "G": "C", "C": "G", "T": "A", "a": "t", "g": "c", "c": "g", "t": "a",
         "N": "N", "n": "n", "-": "-"}


def codon_index(n1: str, n2: str, n3: str) -> int:
    return 16 * DNA_INDEX[n1] + 4 * DNA_INDEX[n2] + DNA_INDEX[n3]


def codon_is(n1: str, n2: str, n3: str) -> bool:
    return n1 in DNA_INDEX and n2 in DNA_INDEX and n3 in DNA_INDEX


def codon_of_index(i: int) -> str:
    return "ACGT"[i // 16] + "ACGT"[(i // 4) % 4] + "ACGT"[i % 4]


def revcomp(s: str) -> str:
    try:
        return "".join(_COMP[c] for c in reversed(s))
    except KeyError as e:
        raise ValueError("unrecognized nucleotide %s" % e.args[0])


def read_ecm(path: str) -> Tuple[np.ndarray, np.ndarray]:
    """ECM.import_parameters: S (64x64 symmetric, zero diagonal) and pi (64)."""
    with open(path) as f:
        lines = f.read().split("\n")

    def nums(line):
        return [float(x.strip()) for x in line.split(" ") if x.strip() != ""]

    raw = [nums(lines[i]) for i in range(63)]
    S = np.zeros((64, 64))
    for i in range(64):
        for j in range(64):
            if i > j:
                S[i, j] = raw[i - 1][j]
            elif i < j:
                S[i, j] = raw[j - 1][i]
    if lines[63].strip() != "":
        raise ValueError("ECM.import_parameters")
    pi = np.array(nums(lines[64]))
    codons = []
    for li in (67, 68, 69, 70):
        for s in lines[li].split(" "):
            s = s.strip()
            if s:
                assert len(s) == 3
                codons.append(s)
    if len(codons) != 64 or any(codon_index(*c) != i for i, c in enumerate(codons)):
        raise ValueError("ECM.import_parameters: incorrect codon order")
    return S, pi


def build_q(S: np.ndarray, pi: np.ndarray) -> np.ndarray:
    """Q of PhyloCSFModel.make_q_p14n / qscale, via the C restatement."""
    lib = _lib()
    k = len(pi)
    Q = np.zeros((k, k))
    st = lib.orc_build_q(k, _dp(np.ascontiguousarray(S, np.float64)), _dp(np.ascontiguousarray(pi, np.float64)), _dp(Q))
    if st:
        raise RuntimeError("orc_build_q status %d" % st)
    return Q


# --------------------------------------------------------------------------
# Driver-side restatements (src/PhyloCSF.ml)


def input_mfa(text: str) -> Tuple[List[str], List[str]]:
    lines = text.split("\n")
    species: List[str] = []
    seqs: List[List[str]] = []
    i = 0
    # hdr: skip empty lines, then require '>'
    while i < len(lines) and len(lines[i]) == 0:
        i += 1
    if i >= len(lines):
        raise ValueError("invalid MFA alignment: no header")
    while i < len(lines):
        line = lines[i]
        i += 1
        if len(line) == 0:
            continue
        if line[0] != ">":
            raise ValueError("invalid MFA alignment: bad header")
        hdr = line[1:]
        sp = (hdr[: hdr.index("|")] if "|" in hdr else hdr).strip()
        species.append(sp)
        buf: List[str] = []
        while i < len(lines):
            s = lines[i].strip()
            if len(s) == 0:
                i += 1
                continue
            if s[0] == ">":
                break
            buf.append(s)
            i += 1
        seqs.append(buf)
    out = ["".join(b) for b in seqs]
    if not out or len(out[0]) == 0 or any(s == "" for s in species) or any(len(s) != len(out[0]) for s in out):
        raise ValueError("invalid MFA alignment: empty species name or sequence, or sequence length mismatch")
    return species, out


def remove_ref_gaps(aln: List[str]) -> List[str]:
    keep = [j for j, c in enumerate(aln[0]) if c != "-"]
    return ["".join(row[j] for j in keep) for row in aln]


ORF_MODES = ("AsIs", "ATGStop", "StopStop", "StopStop3", "ToFirstStop", "FromLastStop", "ToOrFromStop")


def find_orfs(dna: str, ofs: int, orf_mode: str, min_codons: int = 25) -> List[Tuple[int, int]]:
    atg = orf_mode == "ATGStop"

    def codon(p):
        return dna[p:p + 3].upper()

    def is_start(p):
        return codon(p) == "ATG"

    def is_stop(p):
        return codon(p) in ("TAA", "TAG", "TGA")

    n = len(dna)
    orfs: List[Tuple[int, int]] = []   # most recent first, as the reference's list
    starts: List[int] = []
    for lo in range(ofs, n - 2):
        if (lo - ofs) % 3 == 0:
            hi = lo + 2
            if (not atg and not starts and not is_stop(lo)) or (atg and is_start(lo)):
                starts.insert(0, lo)
            if hi + 3 < n and is_stop(hi + 1):
                for st in starts:
                    if hi > st + 2:
                        orfs.insert(0, (st, hi))
                starts = []
    if not atg:
        for st in starts:
            rem = n - st
            orfs.insert(0, (st, st + (rem // 3) * 3 - 1))
    if orf_mode == "StopStop3":
        allsub = []
        for (lo, hi) in orfs:
            sub = [(lo, hi)]
            cod = (hi - lo + 1) // 3
            lo2 = lo + (cod // 3) * 3
            if lo2 > lo:
                sub.insert(0, (lo2, hi))
            lo3 = lo + (2 * cod // 3) * 3
            if lo3 > lo2 and lo3 > lo:
                sub.insert(0, (lo3, hi))
            allsub.extend(sub)
        orfs = allsub
    if orf_mode == "ToFirstStop" and orfs:
        first = orfs[-1]
        orfs = [first] if first[0] == ofs else []
    if orf_mode == "FromLastStop" and orfs:
        last = orfs[0]
        orfs = [last] if n - last[1] <= 3 else []
    if orf_mode == "ToOrFromStop" and orfs:
        first = orfs[-1]
        last = orfs[0]
        orfs = [first] if first[0] == ofs else []
        if n - last[1] <= 3 and first != last:
            orfs = [last] + orfs
    out = []
    for (lo, hi) in reversed(orfs):
        assert (hi - lo + 1) % 3 == 0 and (lo - ofs) % 3 == 0
        if (hi - lo + 1) // 3 >= min_codons:
            out.append((lo, hi))
    return out


def candidate_regions(dna: str, frames: int, orf_mode: str = "AsIs", min_codons: int = 25):
    """List of (rc, lo, hi) in the reference's order (PhyloCSF.ml:198-217)."""
    if orf_mode == "AsIs":
        hi = len(dna) - 1
        r = [(False, 0, hi)]
        if frames != 1:
            r += [(False, 1, hi), (False, 2, hi)]
        if frames == 6:
            r += [(True, 0, hi), (True, 1, hi), (True, 2, hi)]
        return r
    groups = [[(False, lo, hi) for lo, hi in find_orfs(dna, 0, orf_mode, min_codons)]]
    if frames != 1:
        groups.append([(False, lo, hi) for lo, hi in find_orfs(dna, 1, orf_mode, min_codons)])
        groups.append([(False, lo, hi) for lo, hi in find_orfs(dna, 2, orf_mode, min_codons)])
    if frames == 6:
        rc = revcomp(dna)
        for o in (0, 1, 2):
            groups.append([(True, lo, hi) for lo, hi in find_orfs(rc, o, orf_mode, min_codons)])
    return [x for g in groups for x in g]


def pleaves(aln: Sequence[str], leaf_rows: Sequence[Optional[int]], lo: int, hi: int) -> np.ndarray:
    """Leaf states per codon column: int32 [ncols, nl]; -1 = Marginalize."""
    cols = []
    pos = lo
    while pos + 2 <= hi:
        row = []
        for r in leaf_rows:
            if r is None:
                row.append(MARGINALIZE)
            else:
                c = aln[r][pos:pos + 3]
                row.append(codon_index(*c) if codon_is(*c) else MARGINALIZE)
        cols.append(row)
        pos += 3
    return np.array(cols, dtype=np.int32).reshape(len(cols), len(leaf_rows))


def leaf_rows_for(tree: Tree, species: List[str]) -> List[Optional[int]]:
    t_species = set(tree.labels[: tree.nl])
    extra = sorted(set(species) - t_species)
    if extra:
        raise ValueError("parameters not available for species: " + " ".join(extra))
    which = {}
    for i, sp in enumerate(species):
        which[sp] = i     # last occurrence wins, as SMap.add over the rows
    return [which.get(tree.labels[i]) for i in range(tree.nl)]


# --------------------------------------------------------------------------
# ctypes layer


class _Tree(ctypes.Structure):
    _fields_ = [("nl", ctypes.c_int), ("n", ctypes.c_int),
                ("lchild", ctypes.POINTER(ctypes.c_int)), ("rchild", ctypes.POINTER(ctypes.c_int)),
                ("parent", ctypes.POINTER(ctypes.c_int)), ("branch", ctypes.POINTER(ctypes.c_double))]


class _Model(ctypes.Structure):
    _fields_ = [("k", ctypes.c_int), ("U", ctypes.POINTER(ctypes.c_double)),
                ("lam", ctypes.POINTER(ctypes.c_double)), ("pi", ctypes.POINTER(ctypes.c_double)),
                ("prior", ctypes.POINTER(ctypes.c_double)), ("tol", ctypes.c_double)]


class Result(ctypes.Structure):
    _fields_ = [("score", ctypes.c_double), ("anc", ctypes.c_double),
                ("rho_c", ctypes.c_double), ("rho_n", ctypes.c_double),
                ("lpr_c", ctypes.c_double), ("lpr_n", ctypes.c_double),
                ("elpr_c", ctypes.c_double), ("elpr_n", ctypes.c_double),
                ("status", ctypes.c_int), ("evals", ctypes.c_int)]


_LIB = None


def _lib():
    global _LIB
    if _LIB is None:
        path = build()
        lib = ctypes.CDLL(path)
        D = ctypes.POINTER(ctypes.c_double)
        I = ctypes.POINTER(ctypes.c_int)
        lib.orc_build_q.argtypes = [ctypes.c_int, D, D, D]
        lib.orc_eigen_reversible.argtypes = [ctypes.c_int, D, D, D, D]
        lib.orc_pt.argtypes = [ctypes.POINTER(_Model), ctypes.c_double, D]
        lib.orc_dpt_dt.argtypes = [ctypes.POINTER(_Model), ctypes.c_double, D]
        lib.orc_column_likelihood.argtypes = [ctypes.c_int, ctypes.POINTER(_Tree), D, D, I, D]
        lib.orc_column_likelihood.restype = ctypes.c_double
        lib.orc_column_posteriors.argtypes = [ctypes.c_int, ctypes.POINTER(_Tree), D, D, I, D]
        lib.orc_column_posteriors.restype = ctypes.c_double
        lib.orc_lpr_leaves.argtypes = [ctypes.POINTER(_Model), ctypes.POINTER(_Tree), ctypes.c_double,
                                       ctypes.c_int, I, D, D]
        lib.orc_grad_branches.argtypes = [ctypes.POINTER(_Model), ctypes.POINTER(_Tree), ctypes.c_double,
                                          ctypes.c_int, I, D, D]
        lib.orc_branch_counts.argtypes = [ctypes.POINTER(_Model), ctypes.POINTER(_Tree), ctypes.c_double,
                                          ctypes.c_int, I, D, D]
        lib.orc_ell.argtypes = [ctypes.POINTER(_Model), ctypes.POINTER(_Tree), ctypes.c_double, D, D]
        lib.orc_score_region.argtypes = [ctypes.POINTER(_Model), ctypes.POINTER(_Model), ctypes.POINTER(_Tree),
                                         ctypes.c_int, ctypes.c_int, I, ctypes.POINTER(Result)]
        lib.orc_score_batch.argtypes = [ctypes.POINTER(_Model), ctypes.POINTER(_Model), ctypes.POINTER(_Tree),
                                        ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int64), I,
                                        ctypes.POINTER(Result)]
        lib.orc_set_sparse_leaves.argtypes = [ctypes.c_int]
        _LIB = lib
    return _LIB


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def set_sparse_leaves(on: bool) -> None:
    _lib().orc_set_sparse_leaves(1 if on else 0)


class OTree:
    """Tree arrays pinned for the C oracle."""

    def __init__(self, tree: Tree, branch: Optional[np.ndarray] = None):
        self.tree = tree
        self.lchild = np.ascontiguousarray(tree.lchild, np.int32)
        self.rchild = np.ascontiguousarray(tree.rchild, np.int32)
        self.parent = np.ascontiguousarray(tree.parent, np.int32)
        b = tree.branch[: tree.n - 1] if branch is None else branch
        self.branch = np.ascontiguousarray(b, np.float64)
        self.c = _Tree(tree.nl, tree.n, _ip(self.lchild), _ip(self.rchild), _ip(self.parent), _dp(self.branch))


class OModel:
    """A reversible model: eigendecomposition of Q (C Jacobi) plus prior."""

    def __init__(self, Q: np.ndarray, pi: np.ndarray, prior: Optional[np.ndarray] = None, tol: float = 1e-6):
        lib = _lib()
        k = len(pi)
        self.k = k
        self.Q = np.ascontiguousarray(Q, np.float64)
        self.pi = np.ascontiguousarray(pi, np.float64)
        self.prior = np.ascontiguousarray(pi if prior is None else prior, np.float64)
        self.U = np.zeros((k, k))
        self.lam = np.zeros(k)
        st = lib.orc_eigen_reversible(k, _dp(self.Q), _dp(self.pi), _dp(self.U), _dp(self.lam))
        if st:
            raise RuntimeError("orc_eigen_reversible status %d" % st)
        self.tol = tol
        self.c = _Model(k, _dp(self.U), _dp(self.lam), _dp(self.pi), _dp(self.prior), tol)

    @classmethod
    def from_ecm(cls, S: np.ndarray, pi: np.ndarray) -> "OModel":
        return cls(build_q(S, pi), pi, pi)

    def pt(self, t: float) -> np.ndarray:
        P = np.zeros((self.k, self.k))
        st = _lib().orc_pt(ctypes.byref(self.c), t, _dp(P))
        if st:
            raise RuntimeError("orc_pt status %d" % st)
        return P

    def dpt_dt(self, t: float) -> np.ndarray:
        P = np.zeros((self.k, self.k))
        _lib().orc_dpt_dt(ctypes.byref(self.c), t, _dp(P))
        return P


def _leaves_c(leaves: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(leaves, np.int32)


def column_likelihood(tree: Tree, Ps: np.ndarray, prior: np.ndarray, leaves: Sequence[int]):
    """(z, root posterior) for one column with explicit P matrices [n-1,k,k]."""
    ot = OTree(tree, np.zeros(tree.n - 1))
    k = len(prior)
    Pf = np.ascontiguousarray(Ps, np.float64)
    pr = np.ascontiguousarray(prior, np.float64)
    lv = _leaves_c(np.asarray(leaves))
    post = np.zeros(k)
    z = _lib().orc_column_likelihood(k, ctypes.byref(ot.c), _dp(Pf), _dp(pr), _ip(lv), _dp(post))
    return z, post


def column_posteriors(tree: Tree, Ps: np.ndarray, prior: np.ndarray, leaves: Sequence[int]):
    ot = OTree(tree, np.zeros(tree.n - 1))
    k = len(prior)
    Pf = np.ascontiguousarray(Ps, np.float64)
    pr = np.ascontiguousarray(prior, np.float64)
    lv = _leaves_c(np.asarray(leaves))
    post = np.zeros((tree.n, k))
    z = _lib().orc_column_posteriors(k, ctypes.byref(ot.c), _dp(Pf), _dp(pr), _ip(lv), _dp(post))
    return z, post


def lpr_leaves(model: OModel, otree: OTree, rho: float, leaves: np.ndarray) -> Tuple[float, float]:
    lv = _leaves_c(leaves)
    lpr = ctypes.c_double()
    elpr = ctypes.c_double()
    st = _lib().orc_lpr_leaves(ctypes.byref(model.c), ctypes.byref(otree.c), rho, lv.shape[0], _ip(lv),
                               ctypes.byref(lpr), ctypes.byref(elpr))
    if st:
        raise RuntimeError("orc_lpr_leaves status %d" % st)
    return lpr.value, elpr.value


def grad_branches(model: OModel, otree: OTree, rho: float, leaves: np.ndarray) -> Tuple[float, np.ndarray]:
    lv = _leaves_c(leaves)
    lpr = ctypes.c_double()
    g = np.zeros(otree.tree.n - 1)
    st = _lib().orc_grad_branches(ctypes.byref(model.c), ctypes.byref(otree.c), rho, lv.shape[0], _ip(lv),
                                  ctypes.byref(lpr), _dp(g))
    if st:
        raise RuntimeError("orc_grad_branches status %d" % st)
    return lpr.value, g


def branch_counts(model: OModel, otree: OTree, rho: float, leaves: np.ndarray) -> Tuple[float, np.ndarray]:
    """(lpr, expected substitution counts [n-1][k][k] summed over the columns)."""
    lv = _leaves_c(leaves)
    lpr = ctypes.c_double()
    c = np.zeros((otree.tree.n - 1, model.k, model.k))
    st = _lib().orc_branch_counts(ctypes.byref(model.c), ctypes.byref(otree.c), rho, lv.shape[0], _ip(lv),
                                  ctypes.byref(lpr), _dp(c))
    if st:
        raise RuntimeError("orc_branch_counts status %d" % st)
    return lpr.value, c


def ell(model: OModel, otree: OTree, rho: float, counts: np.ndarray) -> float:
    """PhyloEM.ell of sufficient statistics counts [n-1][k][k] at tree scale rho."""
    out = ctypes.c_double()
    cc = np.ascontiguousarray(counts, np.float64)
    st = _lib().orc_ell(ctypes.byref(model.c), ctypes.byref(otree.c), rho, _dp(cc), ctypes.byref(out))
    if st:
        raise RuntimeError("orc_ell status %d" % st)
    return out.value


FIXED, MLE = 0, 1


def score_region(mc: OModel, mn: OModel, otree: OTree, strategy: int, leaves: np.ndarray) -> Result:
    lv = _leaves_c(leaves)
    res = Result()
    _lib().orc_score_region(ctypes.byref(mc.c), ctypes.byref(mn.c), ctypes.byref(otree.c), strategy,
                            lv.shape[0], _ip(lv), ctypes.byref(res))
    return res


def score_batch(mc: OModel, mn: OModel, otree: OTree, strategy: int, col_offsets: np.ndarray,
                leaves: np.ndarray) -> List[Result]:
    lv = _leaves_c(leaves)
    offs = np.ascontiguousarray(col_offsets, np.int64)
    nreg = len(offs) - 1
    arr = (Result * max(nreg, 1))()
    _lib().orc_score_batch(ctypes.byref(mc.c), ctypes.byref(mn.c), ctypes.byref(otree.c), strategy, nreg,
                           offs.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), _ip(lv), arr)
    return [arr[i] for i in range(nreg)]


def decibans(x: float) -> float:
    return 10.0 * x / math.log(10.0)
