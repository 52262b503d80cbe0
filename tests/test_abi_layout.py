"""The ctypes mirrors of the C ABI's structs (cellular_raza_gb300/_native.py, oracle/pyoracle.py)
have the same size and field offsets as the C declarations (include/crg.h,
oracle/chili_oracle.h): a small C program compiled with the host compiler prints them."""
import ctypes as C
import os
import shutil
import subprocess
import sys

import pytest

from cellular_raza_gb300 import _native as N

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def c_layout(tmp_path, header, structs):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", f'#include "{header}"', "int main(void) {"]
    for ctype, fields in structs.items():
        lines.append(f'  printf("{ctype} size %zu\\n", sizeof({ctype}));')
        for f in fields:
            lines.append(f'  printf("{ctype} {f} %zu\\n", offsetof({ctype}, {f}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    res = {}
    for line in out.splitlines():
        t, f, v = line.split()
        res[(t, f)] = int(v)
    return res


def check(layout, ctype, pytype):
    assert layout[(ctype, "size")] == C.sizeof(pytype), ctype
    for name, _ in pytype._fields_:
        assert layout[(ctype, name)] == getattr(pytype, name).offset, (ctype, name)


def test_crg_structs_match_ctypes(tmp_path):
    structs = {"crg_domain": [f for f, _ in N.CrgDomain._fields_],
               "crg_model": [f for f, _ in N.CrgModel._fields_]}
    lay = c_layout(tmp_path, os.path.join(ROOT, "include", "crg.h"), structs)
    check(lay, "crg_domain", N.CrgDomain)
    check(lay, "crg_model", N.CrgModel)


def test_oracle_structs_match_ctypes(tmp_path):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    structs = {"or_config": [f for f, _ in pyoracle.OrConfig._fields_],
               "or_cycle": [f for f, _ in pyoracle.OrCycle._fields_],
               "or_debug": [f for f, _ in pyoracle.OrDebug._fields_]}
    lay = c_layout(tmp_path, os.path.join(ROOT, "oracle", "chili_oracle.h"), structs)
    check(lay, "or_config", pyoracle.OrConfig)
    check(lay, "or_cycle", pyoracle.OrCycle)
    check(lay, "or_debug", pyoracle.OrDebug)
