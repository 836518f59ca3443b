"""The C ABI's structures as the Python binding declares them: every struct of
include/umcp_gpu.h has a ctypes counterpart with the same size and the same
offset for every field (checked by a small C program compiled against the
header). A field added on one side only would shift every field after it."""
from __future__ import annotations

import ctypes as C
import re
import shutil
import subprocess
from pathlib import Path

import pytest

import umcp_gb300 as U

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "umcp_gpu.h"

# ctypes class -> C typedef
PAIRS = {
    "Params": "umcp_params", "PlanInfo": "umcp_plan_info", "MeshInfo": "umcp_mesh_info",
    "Integrator": "umcp_integrator", "BatchOpts": "umcp_batch_opts", "BatchInfo": "umcp_batch_info",
    "Restraints": "umcp_restraints", "MinimizeOpts": "umcp_minimize_opts", "MinimizeInfo": "umcp_minimize_info",
    "MassOpts": "umcp_mass_opts", "MassInfo": "umcp_mass_info", "ServerOpts": "umcp_server_opts",
    "JobDesc": "umcp_job_desc", "JobInfo": "umcp_job_info", "ServerStats": "umcp_server_stats",
}


def _header_structs() -> set[str]:
    """Names of the header's `typedef struct { ... } name;` declarations."""
    text = HEADER.read_text()
    names = set()
    for m in re.finditer(r"typedef struct \{", text):
        close = re.search(r"^\}\s*(umcp_\w+);", text[m.end():], re.M)
        names.add(close.group(1))
    return names


def test_every_header_struct_has_a_binding():
    assert _header_structs() == set(PAIRS.values())


def test_sizes_and_field_offsets_match_the_header(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "umcp_gpu.h"', "int main(void) {"]
    for py, c in PAIRS.items():
        lines.append(f'  printf("{py} %zu\\n", sizeof({c}));')
        for name, *_ in getattr(U, py)._fields_:
            lines.append(f'  printf("{py}.{name} %zu\\n", offsetof({c}, {name}));')
    lines.append("  return 0;\n}")
    src, exe = tmp_path / "layout.c", tmp_path / "layout"
    src.write_text("\n".join(lines) + "\n")
    subprocess.run([cc, "-I", str(HEADER.parent), str(src), "-o", str(exe)], check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    seen = 0
    for line in out.splitlines():
        key, value = line.rsplit(" ", 1)
        if "." in key:
            py, name = key.split(".")
            assert getattr(getattr(U, py), name).offset == int(value), key
        else:
            assert C.sizeof(getattr(U, key)) == int(value), key
        seen += 1
    assert seen == len(PAIRS) + sum(len(getattr(U, py)._fields_) for py in PAIRS)


def test_every_prototype_is_bound_with_its_arity():
    """Each function the header declares is in the binding's signature table
    with as many argument types as the prototype has parameters."""
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    protos = {}
    for m in re.finditer(r"^[ \t]*(?:const\s+)?[A-Za-z_][\w ]*?[\s*]+(umcp_\w+)\s*\(([^;{]*?)\)\s*;", text, re.M | re.S):
        args = " ".join(m.group(2).split())
        protos[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1
    sigs = U._SIGNATURES
    assert len(protos) > 60 and set(protos) == set(sigs)
    assert {k: n for k, n in protos.items() if len(sigs[k]) != n} == {}
