"""Host-side mirror of the reference driver's per-alignment path.

``process_alignment`` follows src/PhyloCSF.ml:280-389: parse the MFA
(:83-118), optional reference-gap removal (:122-132), U->T, the ungapped
reference check, reverse complements, the species -> leaf mapping
(:293-298), candidate regions (:198-217) and leaf packing (:219-246), then
scores every candidate region in ONE batched engine call (the batching
replacement of ForkMaybe.map, :317) and formats the reference's output line
(:353-376).  Per-region failures become ``exception`` lines, an alignment
that yields no region becomes a ``failure`` line, as in the reference.
"""
from __future__ import annotations

import ctypes

from dataclasses import dataclass, field
from typing import List, Optional, Tuple

import numpy as np

from . import engine as E


class AlignmentError(ValueError):
    pass


def input_mfa(text: str) -> Tuple[List[str], List[str]]:
    lines = text.split("\n")
    i = 0
    while i < len(lines) and len(lines[i]) == 0:
        i += 1
    species: List[str] = []
    rows: List[str] = []
    while i < len(lines):
        line = lines[i]
        i += 1
        if len(line) == 0:
            continue
        if line[0] != ">":
            raise AlignmentError("invalid MFA alignment: bad header")
        hdr = line[1:]
        species.append((hdr.split("|", 1)[0] if "|" in hdr else hdr).strip())
        buf = []
        while i < len(lines):
            s = lines[i].strip()
            if not s:
                i += 1
                continue
            if s[0] == ">":
                break
            buf.append(s)
            i += 1
        rows.append("".join(buf))
    if not rows or not rows[0] or any(not s for s in species) or any(len(r) != len(rows[0]) for r in rows):
        raise AlignmentError("invalid MFA alignment: empty species name or sequence, or sequence length mismatch")
    return species, rows


_COMP = str.maketrans("AGCTagctNn-", "TCGAtcgaNn-")
_VALID = set("AGCTagctNn-")


def revcomp(s: str) -> str:
    bad = set(s) - _VALID
    if bad:
        raise AlignmentError("unrecognized nucleotide %s" % sorted(bad)[0])
    return s.translate(_COMP)[::-1]


_TRANSLATE = ("KNKNTTTTRSRSIIMIQHQHPPPPRRRRLLLLEDEDAAAAGGGGVVVV*Y*YSSSS*CWCLFLF")


def translate(dna: str) -> str:
    out = []
    for i in range(len(dna) // 3):
        c = dna[3 * i:3 * i + 3]
        idx = ["ACGTacgt".find(x) % 4 if x in "ACGTacgt" else -1 for x in c]
        out.append(_TRANSLATE[16 * idx[0] + 4 * idx[1] + idx[2]] if min(idx) >= 0 else "?")
    return "".join(out)


def bls_columns(tree: E.Tree, aln: List[str], leaf_rows: List[Optional[int]]) -> np.ndarray:
    """Per nucleotide column, the total length of the smallest subtree spanning the species
    present there (Newick.subtree + Newick.total_length, lib/CamlPaml/Newick.ml:34-61), computed
    once per alignment by the native helper pcsf_bls_columns."""
    lib = E.load_library()
    L = len(aln[0]) if aln else 0
    out = np.zeros(L)
    rows = (ctypes.c_char_p * max(len(aln), 1))(*[r.encode() for r in aln])
    lr = np.array([-1 if r is None else r for r in leaf_rows], np.int32)
    E._check(lib.pcsf_bls_columns(tree.nl, E._p(tree.parent, ctypes.c_int32), E._p(tree.branch, ctypes.c_double),
                                  E._p(lr, ctypes.c_int32), len(aln), rows, L,
                                  E._p(out, ctypes.c_double) if L else None))
    return out


class BLS:
    """Branch length score of nucleotide columns lo..hi (src/PhyloCSF.ml:252-262): the mean over
    the columns of the spanning-subtree length, over the full tree's length.  The per-column
    lengths are computed once; each region's score is a difference of prefix sums."""

    def __init__(self, tree: E.Tree, aln: List[str], leaf_rows: List[Optional[int]]):
        self.cum = np.concatenate([[0.0], np.cumsum(bls_columns(tree, aln, leaf_rows))])
        self.total = float(tree.branch[: tree.n - 1].sum())

    def __call__(self, lo: int, hi: int) -> float:
        return (self.cum[hi + 1] - self.cum[lo]) / (self.total * (hi - lo + 1))


def bls(tree: E.Tree, aln: List[str], leaf_rows: List[Optional[int]], lo: int, hi: int) -> float:
    """Branch length score of nucleotide columns lo..hi of one alignment (src/PhyloCSF.ml:252-262)."""
    return BLS(tree, aln, leaf_rows)(lo, hi)


@dataclass
class Options:
    strategy: int = E.MLE
    frames: int = 1
    orf_mode: str = "AsIs"
    min_codons: int = 25
    remove_ref_gaps: bool = False
    allow_ref_gaps: bool = False
    anc_comp: bool = False
    all_scores: bool = False
    dna: bool = False
    aa: bool = False
    bls: bool = False


@dataclass
class RegionScore:
    rc: bool
    lo: int
    hi: int
    result: np.void


@dataclass
class AlignmentResult:
    lines: List[str] = field(default_factory=list)
    best: Optional[RegionScore] = None
    regions: List[RegionScore] = field(default_factory=list)


def process_alignment(engine: E.Engine, text: str, opts: Options, fn: str = "") -> AlignmentResult:
    name = fn if fn else "(STDIN)"
    out = AlignmentResult()
    species, aln = input_mfa(text)
    if opts.remove_ref_gaps:
        keep = [j for j, c in enumerate(aln[0]) if c != "-"]
        aln = ["".join(r[j] for j in keep) for r in aln]
    aln = [r.replace("u", "t").replace("U", "T") for r in aln]
    if not opts.allow_ref_gaps and "-" in aln[0]:
        raise AlignmentError("the reference sequence (first alignment row) must be ungapped")
    rc_aln = [revcomp(r) for r in aln]
    tree = engine.tree
    t_species = set(tree.labels[: tree.nl])
    extra = sorted(set(species) - t_species)
    if extra:
        raise AlignmentError("parameters not available for species: " + " ".join(extra))
    which = {sp: i for i, sp in enumerate(species)}
    leaf_rows = [which.get(tree.labels[i]) for i in range(tree.nl)]
    regions = E.candidate_regions(aln[0], opts.frames, opts.orf_mode, opts.min_codons)
    if not regions:
        out.lines.append("%s\tfailure\tFailure(\"no sufficiently long ORFs found\")" % name)
        return out
    offs, leaves = E.pack_regions(tree.nl, leaf_rows, aln, rc_aln, regions)
    res = engine.score_batch(offs, leaves, opts.strategy)
    six = opts.frames == 6
    for (rc, lo, hi), r in zip(regions, res):
        if r["status"] != 0:
            out.lines.append("%s\texception\t%d\t%d%s\t%s" % (name, lo, hi, ("\t-" if rc else "\t+") if six else "",
                                                              E.STATUS_NAMES.get(int(r["status"]), "error")))
        else:
            out.regions.append(RegionScore(rc, lo, hi, r))
    if not out.regions:
        out.lines.append("%s\tfailure\tFailure(\"no regions successfully evaluated\")" % name)
        return out

    bls_of = {}   # per strand: per-column spanning-subtree lengths, computed once

    def line(ty, rs: RegionScore):
        s = "%s\t%s\t%.4f" % (name, ty, rs.result["score"])
        if opts.frames != 1 or opts.orf_mode.lower() != "asis":
            s += "\t%d\t%d" % (rs.lo, rs.hi)
        if six:
            s += "\t" + ("-" if rs.rc else "+")
        if opts.bls:
            key = "rc" if rs.rc else "fwd"
            if key not in bls_of:
                bls_of[key] = BLS(tree, rc_aln if rs.rc else aln, leaf_rows)
            s += "\t%.4f" % bls_of[key](rs.lo, rs.hi)
        if opts.anc_comp:
            s += "\t%.4f" % rs.result["anc_comp_score"]
        refdna = (rc_aln if rs.rc else aln)[0][rs.lo:rs.hi + 1]
        if opts.dna:
            s += "\t" + refdna
        if opts.aa:
            s += "\t" + translate(refdna)
        return s

    if opts.all_scores:
        for rs in out.regions:
            out.lines.append(line("orf_score(decibans)", rs))
    # List.reduce max over (result, rc, lo, hi): by score, then anc score, then position
    best = max(out.regions, key=lambda x: (x.result["score"], x.result["anc_comp_score"], x.rc, x.lo, x.hi))
    out.best = best
    multi = opts.orf_mode.lower() != "asis" or opts.frames != 1
    out.lines.append(line("max_score(decibans)" if multi else "score(decibans)", best))
    return out
