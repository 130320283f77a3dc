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
    "hs_tess_params": abi.TessParams,
    "hs_tune_entry": abi.TuneEntry,
    "hs_frame_stats": abi.FrameStats,
    "hs_marschner_params": abi.MarschnerParams,
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


def test_cpp_wrapper_mirrors_hair_lifecycle(built_library):
    """include/hairsim.hpp: builds against the library; update() before
    setup() is a silent no-op as in the reference (src/fx/hair.cc:90-93);
    init() either succeeds (GPU present) or throws hs::Error (no GPU)."""
    prog = r'''
#include <cstdio>
#include "hairsim.hpp"
int main() {
  hs::Hair hair;
  hair.update(1.0f / 60.0f);                 // not initialised: no-op
  if (hair.initialized()) return 2;
  try {
    hair.init();
  } catch (const hs::Error& e) {
    std::printf("init: %d\n", static_cast<int>(e.status));
    return e.status == HS_ERR_CUDA ? 0 : 3;
  }
  std::vector<float> roots{0, 0, 0, 1, 0, 0}, normals{0, 1, 0, 1, 0, 0};
  hair.setup(roots, normals);
  hair.update(1.0f / 60.0f);
  std::printf("points %u, floats %zu\n", hair.points(), hair.readback().size());
  return hair.readback().size() == 2 * 4 * 4 ? 0 : 4;
}
'''
    libdir = os.path.dirname(built_library)
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "hair.cc")
        open(src, "w").write(prog)
        exe = os.path.join(d, "hair")
        subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), src, "-o", exe,
                        "-L", libdir, "-lhairsim", f"-Wl,-rpath,{libdir}"], check=True)
        r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, r.stdout + r.stderr
