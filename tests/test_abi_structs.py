"""The ctypes mirrors of the C-ABI structs (phylocsf_gb300/engine.py) against the header
(include/phylocsf_engine.h): a C program compiled with the system compiler prints each
struct's size and every field's offset, and the ctypes layout must agree field by field.
A mismatch would let the library write past a Python-owned buffer.  No GPU."""
import ctypes
import os
import shutil
import subprocess

import pytest

from phylocsf_gb300 import engine as E

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STRUCTS = {
    "pcsf_tree": E._Tree,
    "pcsf_result": E.Result,
    "pcsf_omega_result": E.OmegaResult,
    "pcsf_stats": E.Stats,
}


def _c_layout(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "phylocsf_engine.h"', "int main(void) {"]
    for cname, py in STRUCTS.items():
        lines.append('printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for fname, _ in py._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, fname, cname, fname))
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True,
                   capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return dict((k, int(v)) for k, v in (line.rsplit(" ", 1) for line in out.strip().splitlines()))


def test_ctypes_structs_match_header(tmp_path):
    got = _c_layout(tmp_path)
    for cname, py in STRUCTS.items():
        assert got["%s size" % cname] == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got["%s.%s" % (cname, fname)] == getattr(py, fname).offset, (cname, fname)


def _prototypes():
    """name -> (return type, parameter count) of every pcsf_* function declared in include/*.h."""
    import re
    out = {}
    for h in ("phylocsf_engine.h", "phylocsf_host.h"):
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
        text = re.sub(r"^\s*#.*$", " ", text, flags=re.M)          # preprocessor lines
        # each declaration is the text between two semicolons (or braces)
        for chunk in re.split(r"[;{}]", text):
            m = re.search(r"((?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**)\s*(pcsf_[A-Za-z0-9_]+)\s*\(([^()]*)\)\s*$",
                          chunk, flags=re.S)
            if not m or "typedef" in chunk:
                continue
            ret, name, params = m.group(1).replace(" ", ""), m.group(2), " ".join(m.group(3).split())
            n = 0 if params in ("", "void") else params.count(",") + 1
            out[name] = (ret, n)
    return out


def test_ctypes_signatures_match_header():
    protos = _prototypes()
    assert len(protos) >= 30
    rets = {"int": ctypes.c_int, "int32_t": ctypes.c_int32, "int64_t": ctypes.c_int64, "void": None,
            "constchar*": ctypes.c_char_p}
    for name, (ret, n) in protos.items():
        assert name in E.SIGNATURES, name
        args, restype = E.SIGNATURES[name]
        assert len(args) == n, (name, len(args), n)
        assert ret in rets, (name, ret)
        want = rets[ret]
        assert restype is want or (want is not None and restype is not None and
                                   ctypes.sizeof(restype) == ctypes.sizeof(want)), (name, ret, restype)
    assert set(E.SIGNATURES) <= set(protos), sorted(set(E.SIGNATURES) - set(protos))
