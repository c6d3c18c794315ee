"""The ctypes mirrors of the C ABI's structs have the C layout.

A small C program, compiled here with the system compiler against
include/pdds.h, prints sizeof and the offset of every field of every
descriptor and info struct; each ctypes Structure of pdds_gb300._capi must
match it field by field, so a field added on one side only fails here, on
the CPU, instead of shifting every later field of a call."""
import ctypes
import os
import re
import shutil
import subprocess

import pytest

from pdds_gb300 import _capi as capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# ctypes class -> C struct type name
PAIRS = {
    "ProblemDesc": "pdds_problem_desc",
    "LayoutDesc": "pdds_layout_desc",
    "CircleDesc": "pdds_circle_desc",
    "SemilinearDesc": "pdds_semilinear_desc",
    "LayoutInfo": "pdds_layout_info",
    "StencilDesc": "pdds_stencil_desc",
    "EstimateDesc": "pdds_estimate_desc",
    "EstimateInfo": "pdds_estimate_info",
    "TuneInfo": "pdds_tune_info",
    "SolveDesc": "pdds_solve_desc",
    "SolveInfo": "pdds_solve_info",
    "InstanceDesc": "pdds_instance_desc",
    "BatchInfo": "pdds_batch_info",
    "BatchRunDesc": "pdds_batch_run_desc",
    "BatchRunInfo": "pdds_batch_run_info",
}


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "pdds.h"', "int main(void) {"]
    for cls, cname in PAIRS.items():
        st = getattr(capi, cls)
        lines.append(f'  printf("{cls} size %zu\\n", sizeof({cname}));')
        for f in st._fields_:
            lines.append(f'  printf("{cls} {f[0]} %zu\\n", offsetof({cname}, {f[0]}));')
    lines += ["  return 0;", "}"]
    d = tmp_path_factory.mktemp("abi")
    src = d / "abi.c"
    src.write_text("\n".join(lines) + "\n")
    exe = d / "abi"
    r = subprocess.run([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    got = {}
    for ln in out.splitlines():
        cls, field, v = ln.split()
        got[(cls, field)] = int(v)
    return got


@pytest.mark.parametrize("cls", sorted(PAIRS))
def test_struct_matches_c_layout(c_layout, cls):
    st = getattr(capi, cls)
    assert C_sizeof(st) == c_layout[(cls, "size")], cls
    for f in st._fields_:
        assert getattr(st, f[0]).offset == c_layout[(cls, f[0])], (cls, f[0])


def C_sizeof(st):
    return ctypes.sizeof(st)


def test_every_header_struct_has_a_mirror():
    hdr = open(os.path.join(ROOT, "include", "pdds.h")).read()
    structs = set(re.findall(r"typedef struct \{.*?\} (pdds_\w+);", hdr, re.S))
    assert structs == set(PAIRS.values())
