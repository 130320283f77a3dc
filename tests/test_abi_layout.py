"""The ctypes mirror of include/hairsim.h against the C compiler's own
layout of every struct (sizes and field offsets), on the CPU."""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile

import pytest

from barbu_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STRUCTS = {
    "hs_strand_params": abi.StrandParams,
    "hs_sim_params": abi.SimParams,
    "hs_layout": abi.Layout,
    "hs_server_config": abi.ServerConfig,
    "hs_request": abi.Request,
    "hs_tick_stats": abi.TickStats,
}


def c_layout():
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "hairsim.h"', 'int main(void) {']
    for cname, py in STRUCTS.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("  return 0;\n}")
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "layout.c"), os.path.join(d, "layout")
        open(src, "w").write("\n".join(lines))
        subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), "-o", exe, src], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    got = {}
    for line in out.splitlines():
        a, b, c = line.split()
        got[(a, b)] = int(c)
    return got


@pytest.mark.parametrize("cname", sorted(STRUCTS))
def test_ctypes_struct_matches_c_layout(cname):
    got = c_layout()
    py = STRUCTS[cname]
    assert got[(cname, "size")] == C.sizeof(py)
    for fname, _ in py._fields_:
        assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)


def test_header_compiles_as_c_and_cpp():
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "x.c")
        open(src, "w").write('#include "hairsim.h"\nint main(void){return 0;}\n')
        subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), "-o",
                        os.path.join(d, "x"), src], check=True)
        srcpp = os.path.join(d, "x.cc")
        open(srcpp, "w").write('#include "hairsim.h"\nint main(){return 0;}\n')
        subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), "-o",
                        os.path.join(d, "xx"), srcpp], check=True)
