"""Shared test helpers: fixtures -> oracle models and product engines."""
import json
import os

import numpy as np

from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
PARAMS = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "phylocsf_gb300", "params")


def fixture_params(name):
    d = np.load(os.path.join(PARAMS, name + ".npz"))

    def full(tri):
        S = np.zeros((64, 64))
        S[np.tril_indices(64, -1)] = tri
        return S + S.T

    tree = O.Tree([str(x) for x in d["labels"]], d["parent"].astype(np.int32), d["lchild"].astype(np.int32),
                  d["rchild"].astype(np.int32), d["branch"].astype(np.float64))
    return tree, full(d["S_c"]), d["pi_c"].copy(), full(d["S_n"]), d["pi_n"].copy()


_ORACLE_CACHE = {}


def oracle_models(name):
    if name not in _ORACLE_CACHE:
        tree, Sc, pic, Sn, pin = fixture_params(name)
        _ORACLE_CACHE[name] = (O.OModel.from_ecm(Sc, pic), O.OModel.from_ecm(Sn, pin), O.OTree(tree), tree)
    return _ORACLE_CACHE[name]


def examples():
    with open(os.path.join(GOLDEN, "examples.json")) as f:
        return json.load(f)


def pins():
    with open(os.path.join(GOLDEN, "pins.json")) as f:
        return json.load(f)


def beagle():
    with open(os.path.join(GOLDEN, "beagle.json")) as f:
        return json.load(f)


def oracle_fixed():
    with open(os.path.join(GOLDEN, "oracle_fixed.json")) as f:
        return json.load(f)


def parse_flags(flags):
    """The subset of PhyloCSF command-line flags used by the pinned runs."""
    o = {"frames": 1, "orf": "AsIs", "remove_ref_gaps": False, "anc": False, "aa": False}
    for f in flags.split():
        if f.startswith("--frames="):
            o["frames"] = int(f.split("=")[1])
        elif f.startswith("--orf="):
            o["orf"] = f.split("=")[1]
        elif f == "--removeRefGaps":
            o["remove_ref_gaps"] = True
        elif f == "--ancComp":
            o["anc"] = True
        elif f == "--aa":
            o["aa"] = True
    return o


def oracle_leaves_to_u8(lv):
    """oracle leaf codes (-1 = Marginalize) -> engine codes (64)."""
    a = np.asarray(lv, np.int32).copy()
    a[a < 0] = 64
    return a.astype(np.uint8)


def u8_to_oracle(lv):
    a = np.asarray(lv, np.int32).copy()
    a[a >= 64] = -1
    return a
