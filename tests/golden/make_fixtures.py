"""Generate the golden fixtures under tests/golden/ from the reference tree.

Run from the repository root with the mlin/PhyloCSF sources available:

    python tests/golden/make_fixtures.py /path/to/PhyloCSF
    (or set PHYLOCSF_REFERENCE to that path)

Writes (all derived, none copied verbatim):
  phylocsf_gb300/params/<set>.npz
                      tree in CamlPaml T order (parent, children, branch, labels) parsed
                      from PhyloCSF_Parameters/<set>.nh, and the coding /
                      noncoding ECMs (strict lower triangle of S, pi) parsed
                      from PhyloCSF_Parameters/<set>_{coding,noncoding}.ECM
  examples.json       the three PhyloCSF_Examples alignments as (species, rows)
  beagle.json         the TinyTest data of lib/CamlPaml/test.ml:59-81
                      (sequences, tree, expected log-likelihood)
  pins.json           the accuracy windows asserted by src/test.ml:27-59
  oracle_fixed.json   oracle scores (strategy=fixed, rho=1) of the example
                      alignments, to pin the oracle without the reference tree
"""
from __future__ import annotations

import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

PARAM_SETS = ["12flies", "29mammals", "58mammals", "100vertebrates", "120mammals"]
EXAMPLES = ["tal-AA.fa", "ALDH2.exon5.fa", "Aldh2.mRNA.fa"]


def main(ref: str) -> None:
    pdir = os.path.join(ROOT, "phylocsf_gb300", "params")
    os.makedirs(pdir, exist_ok=True)
    il = np.tril_indices(64, -1)
    for name in PARAM_SETS:
        base = os.path.join(ref, "PhyloCSF_Parameters", name)
        t = O.load_tree(base + ".nh")
        Sc, pic = O.read_ecm(base + "_coding.ECM")
        Sn, pin = O.read_ecm(base + "_noncoding.ECM")
        np.savez_compressed(os.path.join(pdir, name + ".npz"), parent=t.parent, lchild=t.lchild, rchild=t.rchild,
                            branch=t.branch,
                            labels=np.array(t.labels), S_c=Sc[il], pi_c=pic, S_n=Sn[il], pi_n=pin)

    ex = {}
    for fa in EXAMPLES:
        with open(os.path.join(ref, "PhyloCSF_Examples", fa)) as f:
            sp, rows = O.input_mfa(f.read())
        ex[fa] = {"species": sp, "rows": rows}
    with open(os.path.join(HERE, "examples.json"), "w") as f:
        json.dump(ex, f)

    src = open(os.path.join(ref, "lib", "CamlPaml", "test.ml")).read()
    seqs = {nm: re.search(r'let %s = "([ACGT-]+)"' % nm, src).group(1) for nm in ("human", "chimp", "gorilla")}
    tree = re.search(r'Lexing.from_string "(\(\(human[^"]*)"', src).group(1)
    logl = float(re.search(r"\(-(1574\.\d+)\)", src).group(1)) * -1.0
    with open(os.path.join(HERE, "beagle.json"), "w") as f:
        json.dump({"tree": tree, "seqs": seqs, "logL": logl, "eps": 1e-3}, f)

    tsrc = open(os.path.join(ref, "src", "test.ml")).read()
    pins = []
    for m in re.finditer(r'run_PhyloCSF "(\w+)" \(?"\.\./PhyloCSF_Examples/([^ "]+)([^"]*)"', tsrc):
        start = m.end()
        nxt = tsrc.find("let ", start)
        body = tsrc[start:nxt if nxt > 0 else len(tsrc)]
        wins = [tuple(map(float, w)) for w in re.findall(r"within \((-?[\d.]+),(-?[\d.]+)\)", body)]
        eqs = [int(x) for x in re.findall(r"int_of_string \(List.nth ans \d\) \$hould # equal (\d+)", body)]
        flags = m.group(3).strip()
        strand = re.findall(r'List.nth ans 5 \$hould # equal "([+-])"', body)
        if flags.endswith("--frames="):
            flags += "6"     # the full (not SKIP_SLOW) run of src/test.ml:347-354
        pins.append({"params": m.group(1), "file": m.group(2), "flags": flags, "windows": wins, "ints": eqs,
                     "strand": strand[0] if strand else None})
    with open(os.path.join(HERE, "pins.json"), "w") as f:
        json.dump(pins, f, indent=1)

    # oracle fixed-strategy scores of the first two examples (tight FP64 values)
    O.set_sparse_leaves(True)
    fixed = {}
    for name, fa in (("12flies", "tal-AA.fa"), ("29mammals", "ALDH2.exon5.fa")):
        base = os.path.join(ref, "PhyloCSF_Parameters", name)
        t = O.load_tree(base + ".nh")
        mc = O.OModel.from_ecm(*O.read_ecm(base + "_coding.ECM"))
        mn = O.OModel.from_ecm(*O.read_ecm(base + "_noncoding.ECM"))
        sp, rows = ex[fa]["species"], ex[fa]["rows"]
        lv = O.pleaves(rows, O.leaf_rows_for(t, sp), 0, len(rows[0]) - 1)
        r = O.score_region(mc, mn, O.OTree(t), O.FIXED, lv)
        fixed[fa] = {"params": name, "score": r.score, "anc": r.anc, "lpr_c": r.lpr_c, "lpr_n": r.lpr_n,
                     "elpr_c": r.elpr_c, "elpr_n": r.elpr_n}
    with open(os.path.join(HERE, "oracle_fixed.json"), "w") as f:
        json.dump(fixed, f, indent=1)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PHYLOCSF_REFERENCE", "")
    if not ref or not os.path.isdir(os.path.join(ref, "PhyloCSF_Parameters")):
        raise SystemExit("usage: make_fixtures.py /path/to/PhyloCSF (or set PHYLOCSF_REFERENCE)")
    main(ref)
