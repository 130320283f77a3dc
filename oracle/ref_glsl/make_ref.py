"""Build the reference hair shaders as C++ shared libraries.

TEST INFRASTRUCTURE ONLY. Reads, in place and read-only,
  <reference>/src/shaders/hair/01_simulation/cs_simulation.glsl
  <reference>/src/shaders/hair/02_tess_stream/tes_stream_hair.glsl
  <reference>/src/shaders/shared/inc_maths.glsl (four functions of it)
  <reference>/src/shaders/hair/interop.h
and writes only under oracle/_ref/:
  oracle/_ref/cs_simulation_ref.cc   the simulation shader after the edits below
  oracle/_ref/libref_glsl.so         that text + glsl_shim.h + glsl_harness.inc
  oracle/_ref/tes_stream_ref.cc      the tessellation evaluation shader, edited
  oracle/_ref/libref_tes.so          that text + glsl_shim.h + tes_harness.inc

The shader text is not otherwise changed. The edits are mechanical and only
touch GLSL syntax that C++ has no spelling for:
  1. comments are stripped and `#version` is dropped;
  2. each `layout(std430, binding = B) readonly|writeonly buffer Blk { vec4 name[]; };`
     becomes `static vec4* name;` (the harness binds it);
  3. `layout(local_size_x = X) in;` becomes `static const unsigned kLocalSizeX = (X);`
  4. `inout T name` parameters become `T& name`;
and these macros are defined around the text: `uniform` and `shared` ->
`static`, `in` -> nothing, `xyz` -> the swizzle accessor, `main` -> glsl_main.
The tessellation evaluation shader gets the same treatment plus: the
`#include "shared/inc_maths.glsl"` line is replaced by the four functions
of that file it calls (maprange, smoothstep2, hermite_mix,
sample_triangle2), copied out by name; `layout(isolines) in;` is dropped;
its `in`/`patch in`/`out` variables become statics (arrays of the patch's
6 control points); the vec3 random-buffer block becomes a pointer; and
every floating-point literal gets an `f` suffix, since GLSL literals are
single precision and C++ ones are double.
The results are used only to generate golden vectors on this machine (the
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


TES_REL = os.path.join("src", "shaders", "hair", "02_tess_stream", "tes_stream_hair.glsl")
MATHS_REL = os.path.join("src", "shaders", "shared", "inc_maths.glsl")
TES_FUNCTIONS = ("maprange", "smoothstep2", "hermite_mix", "sample_triangle2")
_FLOAT_LITERAL = re.compile(r"(?<![\w.])(\d+\.\d*|\.\d+)(?![\w.])")


def strip_comments(text: str) -> str:
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    return re.sub(r"^\s*#version[^\n]*$", "", text, flags=re.M)


def extract_function(text: str, name: str) -> str:
    """The definition of `name` (signature to its closing brace)."""
    m = re.search(r"^[ \t]*\w+[ \t]+" + name + r"[ \t]*\(", text, flags=re.M)
    if not m:
        raise RuntimeError(f"{name} not found")
    i = text.index("{", m.end())
    depth = 0
    for k in range(i, len(text)):
        depth += {"{": 1, "}": -1}.get(text[k], 0)
        if depth == 0:
            return text[m.start():k + 1] + "\n"
    raise RuntimeError(f"{name}: unbalanced braces")


def translate_tes(tes: str, maths: str) -> str:
    maths = strip_comments(maths)
    funcs = "".join(extract_function(maths, f) for f in TES_FUNCTIONS)
    text = strip_comments(tes)
    text, n_inc = re.subn(r'#include\s+"shared/inc_maths.glsl"', lambda m: funcs, text)
    text, n_iso = re.subn(r"layout\s*\(\s*isolines\s*\)\s*in\s*;", "", text)
    text, n_in = re.subn(r"layout\s*\(\s*location\s*=\s*\d+\s*\)\s*in\s+(\w+)\s+(\w+)\s*\[\s*\]\s*;",
                         r"static \1 \2[6];", text)
    text, n_patch = re.subn(r"layout\s*\(\s*location\s*=\s*\d+\s*\)\s*patch\s+in\s+(\w+)\s+(\w+)\s*(\[\s*\])?\s*;",
                            lambda m: f"static {m.group(1)} {m.group(2)}{'[1]' if m.group(3) else ''};", text)
    text, n_out = re.subn(r"layout\s*\(\s*location\s*=\s*\d+\s*\)\s*out\s+(\w+)\s+(\w+)\s*;", r"static \1 \2;", text)
    text, n_buf = re.subn(r"layout\s*\(\s*std430\s*,\s*binding\s*=\s*(\w+)\s*\)\s*readonly\s+buffer\s+\w+\s*"
                          r"\{\s*vec3\s+(\w+)\s*\[\s*\]\s*;\s*\}\s*;",
                          lambda m: f"static vec3* {m.group(2)} = nullptr; /* binding {m.group(1)} */", text)
    if (n_inc, n_iso, n_in, n_patch, n_out, n_buf) != (1, 1, 2, 2, 2, 1):
        raise RuntimeError(f"unexpected shader structure: {(n_inc, n_iso, n_in, n_patch, n_out, n_buf)}")
    text = _FLOAT_LITERAL.sub(lambda m: m.group(1) + "f", text)
    head = (
        '#include "glsl_shim.h"\n'
        "namespace glsl {\n"
        "static vec3 gl_TessCoord;\n"
        "#define uniform static\n#define in\n#define xyz xyz_swizzle()\n#define xy xy_swizzle()\n"
        "#define main glsl_main\n"
    )
    tail = (
        "\n#undef uniform\n#undef in\n#undef xyz\n#undef xy\n#undef main\n"
        "}  // namespace glsl\n"
        '#include "tes_harness.inc"\n'
    )
    return head + text + tail


def build_tes(reference: str, quiet: bool = False) -> str:
    with open(os.path.join(reference, TES_REL), "r", encoding="utf-8") as f:
        tes = f.read()
    with open(os.path.join(reference, MATHS_REL), "r", encoding="utf-8") as f:
        maths = f.read()
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = os.path.join(OUT_DIR, "tes_stream_ref.cc")
    so = os.path.join(OUT_DIR, "libref_tes.so")
    with open(cc, "w", encoding="utf-8") as f:
        f.write(translate_tes(tes, maths))
    cmd = [
        "g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
        "-I", HERE, "-I", os.path.join(reference, SHADERS_INC_REL), "-o", so, cc,
    ]
    subprocess.run(cmd, check=True, capture_output=quiet)
    return so


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
    ap.add_argument("--reference", required=True, help="root of the tcoppex/barbu checkout")
    args = ap.parse_args()
    print(build(args.reference))
    print(build_tes(args.reference))
    return 0


if __name__ == "__main__":
    sys.exit(main())
