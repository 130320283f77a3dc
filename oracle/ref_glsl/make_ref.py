"""Build the reference hair-simulation shader as a C++ shared library.

TEST INFRASTRUCTURE ONLY. Reads, in place and read-only,
  <reference>/src/shaders/hair/01_simulation/cs_simulation.glsl
  <reference>/src/shaders/hair/interop.h
and writes only under oracle/_ref/:
  oracle/_ref/cs_simulation_ref.cc   the shader text after the edits below
  oracle/_ref/libref_glsl.so         that text + glsl_shim.h + glsl_harness.inc

The shader text is not otherwise changed. The edits are mechanical and only
touch GLSL syntax that C++ has no spelling for:
  1. comments are stripped and `#version` is dropped;
  2. each `layout(std430, binding = B) readonly|writeonly buffer Blk { vec4 name[]; };`
     becomes `static vec4* name;` (the harness binds it);
  3. `layout(local_size_x = X) in;` becomes `static const unsigned kLocalSizeX = (X);`
  4. `inout T name` parameters become `T& name`;
and these macros are defined around the text: `uniform` and `shared` ->
`static`, `in` -> nothing, `xyz` -> the swizzle accessor, `main` -> glsl_main.
The result is used only to generate golden vectors on this machine (the
reference is not present where the GPU tests run); see tests/golden/.
"""
from __future__ import annotations

import argparse
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT_DIR = os.path.join(ORACLE, "_ref")
SHADER_REL = os.path.join("src", "shaders", "hair", "01_simulation", "cs_simulation.glsl")
SHADERS_INC_REL = os.path.join("src", "shaders")

_SSBO = re.compile(
    r"layout\s*\(\s*std430\s*,\s*binding\s*=\s*(\w+)\s*\)\s*(?:readonly|writeonly)?\s*"
    r"buffer\s+(\w+)\s*\{\s*vec4\s+(\w+)\s*\[\s*\]\s*;\s*\}\s*;"
)
_LOCAL_SIZE = re.compile(r"layout\s*\(\s*local_size_x\s*=\s*([^)]+)\)\s*in\s*;")
_INOUT = re.compile(r"\binout\s+(\w+)\s+(\w+)")


def translate(glsl: str) -> str:
    text = re.sub(r"/\*.*?\*/", "", glsl, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    text = re.sub(r"^\s*#version[^\n]*$", "", text, flags=re.M)
    text, n_ssbo = _SSBO.subn(lambda m: f"static vec4* {m.group(3)} = nullptr; /* binding {m.group(1)} */", text)
    text, n_ls = _LOCAL_SIZE.subn(lambda m: f"static const unsigned kLocalSizeX = ({m.group(1)});", text)
    text, _ = _INOUT.subn(lambda m: f"{m.group(1)}& {m.group(2)}", text)
    if n_ssbo != 4 or n_ls != 1:
        raise RuntimeError(f"unexpected shader structure: {n_ssbo} SSBO blocks, {n_ls} local_size layouts")
    head = (
        '#include "glsl_shim.h"\n'
        "namespace glsl {\n"
        "#define uniform static\n#define shared static\n#define in\n#define xyz xyz_swizzle()\n"
        "#define main glsl_main\n"
    )
    tail = (
        "\n#undef uniform\n#undef shared\n#undef in\n#undef xyz\n#undef main\n"
        "}  // namespace glsl\n"
        '#include "glsl_harness.inc"\n'
    )
    return head + text + tail


def build(reference: str, quiet: bool = False) -> str:
    shader = os.path.join(reference, SHADER_REL)
    if not os.path.isfile(shader):
        raise FileNotFoundError(shader)
    os.makedirs(OUT_DIR, exist_ok=True)
    with open(shader, "r", encoding="utf-8") as f:
        src = translate(f.read())
    cc = os.path.join(OUT_DIR, "cs_simulation_ref.cc")
    so = os.path.join(OUT_DIR, "libref_glsl.so")
    with open(cc, "w", encoding="utf-8") as f:
        f.write(src)
    cmd = [
        "g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
        "-I", HERE, "-I", os.path.join(reference, SHADERS_INC_REL), "-o", so, cc,
    ]
    subprocess.run(cmd, check=True, capture_output=quiet)
    return so


def main() -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--reference", default="/root/reference")
    args = ap.parse_args()
    print(build(args.reference))
    return 0


if __name__ == "__main__":
    sys.exit(main())
