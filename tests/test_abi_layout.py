"""Layout of the C ABI's structs as the C compiler sees them, against the ctypes
mirrors: the package's (nyles_gb300/_native.py) and the one the integration guide at the
repository root tells a reference maintainer to paste. A struct that gains a field in include/nyles_gb300.h
without its mirrors fails here (no GPU needed: gcc compiles a probe of the header)."""
import ctypes
import os
import re
import shutil
import subprocess

import pytest

from nyles_gb300 import _native as nat

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "nyles_gb300.h")


def _struct_fields(name):
    """(field names) of `typedef struct <name> { ... } <name>;` in the header, in order"""
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), src, flags=re.S).group(1)
    names = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        decl = re.sub(r"\[[^\]]*\]", "", decl)          # array extents
        parts = decl.split(None, 1) if not decl.startswith("long long") else ["long long", decl[9:]]
        for v in parts[1].split(","):
            names.append(v.strip().lstrip("*"))
    return names


def _c_layout(tmp_path, name, fields):
    """sizeof and offsetof of every field, printed by a probe compiled against the header"""
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "nyles_gb300.h"', "int main(void) {",
             '  printf("size %%zu\\n", sizeof(%s));' % name]
    for f in fields:
        lines.append('  printf("%s %%zu\\n", offsetof(%s, %s));' % (f, name, f))
    lines += ["  return 0;", "}"]
    src = tmp_path / ("probe_%s.c" % name)
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / ("probe_%s" % name)
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {k: int(v) for k, v in (line.split() for line in out.splitlines())}


def _integration_desc_class():
    """The NylesDesc class of the integration guide's section 3.1, executed as written
    (the CDLL line is left out: this check needs no library)."""
    text = open(os.path.join(REPO, "INTEGRATION.md")).read()
    block = re.search(r"### 3\.1.*?```python\n(.*?)```", text, flags=re.S).group(1)
    cls = re.search(r"(class NylesDesc\(ctypes\.Structure\):.*?\])\n", block, flags=re.S).group(1)
    ns = {"ctypes": ctypes}
    exec(cls, ns)
    return ns["NylesDesc"]


def _check(cstruct, pystruct, fields, layout):
    assert [f[0] for f in pystruct._fields_] == fields
    assert ctypes.sizeof(pystruct) == layout["size"]
    for f in fields:
        assert getattr(pystruct, f).offset == layout[f], f


def test_desc_layout_matches_header(tmp_path):
    fields = _struct_fields("NylesDesc")
    assert fields[-1] == "vf_order" and "tracer_diffusivity" in fields
    layout = _c_layout(tmp_path, "NylesDesc", fields)
    _check("NylesDesc", nat.NylesDesc, fields, layout)
    _check("NylesDesc", _integration_desc_class(), fields, layout)


def test_mg_stats_layout_matches_header(tmp_path):
    fields = _struct_fields("NylesMgStats")
    assert fields == ["nite", "res", "solves", "vcycles", "not_converged", "nonfinite"]
    layout = _c_layout(tmp_path, "NylesMgStats", fields)
    _check("NylesMgStats", nat.NylesMgStats, fields, layout)


def test_batch_table_layout_matches_header(tmp_path):
    fields = _struct_fields("NylesBatchTable")
    assert fields == ["delta", "active", "live", "loop_iterations"]
    layout = _c_layout(tmp_path, "NylesBatchTable", fields)
    _check("NylesBatchTable", nat.NylesBatchTable, fields, layout)
