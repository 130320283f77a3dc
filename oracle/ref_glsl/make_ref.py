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
The skinning and Marschner shaders get the same kind of edits:
  <reference>/src/shaders/shared/inc_skinning.glsl -> oracle/_ref/libref_skin.so:
     apply_skinning, get_dual_quaternions_matrices and skinning_DQBS copied
     out by name (the linear-blend subroutine is not used here), Epsilon()
     from inc_constants.glsl; `subroutine(...)` qualifiers dropped, the
     subroutine uniform and the samplerBuffer become a function pointer and
     a texel pointer (skin_harness.inc binds them);
  <reference>/src/shaders/hair/marschner/cs_marschner_{m,n}.glsl ->
     oracle/_ref/libref_marschner_{m,n}.so: includes expanded in place
     (inc_marschner_n.glsl, inc_fresnel.glsl, inc_solver.glsl and
     inc_constants.glsl whole; of inc_maths.glsl only gaussian), `precision`
     and the work-group layout dropped, the rgba16f image becomes a handle
     that imageStore (marschner_harness.inc) writes through;
and in all of them `v.xyz = e;` / `v.xyz *= e;` become glsl_set_xyz /
glsl_mul_xyz calls (C++ has no swizzle lvalues), `out`/`inout T name`
parameters references, and float literals get an `f` suffix.
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


SKIN_REL = os.path.join("src", "shaders", "shared", "inc_skinning.glsl")
CONST_REL = os.path.join("src", "shaders", "shared", "inc_constants.glsl")
MARSCHNER_REL = os.path.join("src", "shaders", "hair", "marschner")
_SWZ_SET = re.compile(r"(\w+)\.xyz\s*=\s*([^;]+);")
_SWZ_MUL = re.compile(r"(\w+)\.xyz\s*\*=\s*([^;]+);")
_OUT = re.compile(r"\b(?:inout|out)\s+(\w+)\s+(\w+)")


def extract_all(text: str, name: str) -> str:
    """Every definition of `name` (overloads included), in file order;
    declarations without a body are skipped."""
    out = []
    for m in re.finditer(r"^[ \t]*\w+[ \t]+" + name + r"[ \t]*\(", text, flags=re.M):
        depth, k = 0, m.end() - 1
        while True:  # the parameter list
            depth += {"(": 1, ")": -1}.get(text[k], 0)
            k += 1
            if depth == 0:
                break
        rest = text[k:].lstrip()
        if not rest.startswith("{"):
            continue
        i = text.index("{", k)
        depth = 0
        for j in range(i, len(text)):
            depth += {"{": 1, "}": -1}.get(text[j], 0)
            if depth == 0:
                out.append(text[m.start():j + 1] + "\n")
                break
    if not out:
        raise RuntimeError(f"{name} not found")
    return "".join(out)


def glsl_to_cpp(text: str) -> str:
    """The expression-level edits shared by the skinning and Marschner
    shaders (see the module docstring)."""
    text = _SWZ_MUL.sub(lambda m: f"glsl_mul_xyz({m.group(1)}, {m.group(2)});", text)
    text = _SWZ_SET.sub(lambda m: f"glsl_set_xyz({m.group(1)}, {m.group(2)});", text)
    text = _OUT.sub(lambda m: f"{m.group(1)}& {m.group(2)}", text)
    return _FLOAT_LITERAL.sub(lambda m: m.group(1) + "f", text)


def _compile(cc: str, so: str, src: str, reference: str, quiet: bool) -> str:
    with open(cc, "w", encoding="utf-8") as f:
        f.write(src)
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-I", HERE,
           "-I", os.path.join(reference, SHADERS_INC_REL), "-o", so, cc]
    subprocess.run(cmd, check=True, capture_output=quiet)
    return so


def _read(reference: str, rel: str) -> str:
    with open(os.path.join(reference, rel), "r", encoding="utf-8") as f:
        return strip_comments(f.read())


def translate_skin(skin: str, constants: str) -> str:
    funcs = "".join(extract_all(skin, f) for f in ("apply_skinning", "get_dual_quaternions_matrices",
                                                    "skinning_DQBS"))
    text = extract_all(constants, "Epsilon") + funcs
    text = re.sub(r"\bsubroutine\s*\(\s*\w+\s*\)", "", text)
    head = (
        '#include "glsl_shim.h"\n'
        "namespace glsl {\n"
        "static samplerBuffer uSkinningDatas = nullptr;\n"
        "static void (*uSkinning)(uvec4, vec4, vec3&, vec3&) = nullptr;\n"
        "#define in\n#define xyz xyz_swizzle()\n"
    )
    tail = "\n#undef in\n#undef xyz\n}  // namespace glsl\n" + '#include "skin_harness.inc"\n'
    return head + glsl_to_cpp(text) + tail


def build_skin(reference: str, quiet: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    src = translate_skin(_read(reference, SKIN_REL), _read(reference, CONST_REL))
    return _compile(os.path.join(OUT_DIR, "skinning_ref.cc"), os.path.join(OUT_DIR, "libref_skin.so"), src,
                    reference, quiet)


def expand_includes(text: str, reference: str, seen: set) -> str:
    """Replaces `#include "X"` by the (comment-stripped) text of
    src/shaders/X, recursively; of inc_maths.glsl only gaussian."""
    def one(m):
        rel = m.group(1)
        if rel in seen:
            return ""
        seen.add(rel)
        body = _read(reference, os.path.join("src", "shaders", rel))
        if rel.endswith("inc_maths.glsl"):
            # Its own includes (the constants), then the one function used.
            heads = "".join(re.findall(r'#include\s+"[^"]+"', body))
            return "\n" + expand_includes(heads, reference, seen) + "\n" + extract_all(body, "gaussian") + "\n"
        return "\n" + expand_includes(body, reference, seen) + "\n"
    return re.sub(r'#include\s+"([^"]+)"', one, text)


def translate_marschner(shader: str, reference: str) -> str:
    text = expand_includes(shader, reference, set())
    text, n_prec = re.subn(r"precision\s+highp\s+float\s*;", "", text)
    text, n_img = re.subn(r"writeonly\s+uniform\s+layout\s*\(\s*rgba16f\s*\)\s*image2D\s+(\w+)\s*;",
                          r"static int \1 = 0;", text)
    text, n_ls = re.subn(r"layout\s*\(\s*local_size_x\s*=\s*\w+\s*,\s*local_size_y\s*=\s*\w+\s*\)\s*in\s*;", "",
                         text)
    if (n_prec, n_img, n_ls) != (1, 1, 1):
        raise RuntimeError(f"unexpected shader structure: {(n_prec, n_img, n_ls)}")
    head = (
        '#include "glsl_shim.h"\n'
        "namespace glsl {\n"
        "void imageStore(int img, ivec2 p, vec4 v);\n"
        "#define uniform static\n#define in\n#define xyz xyz_swizzle()\n#define xy xy_swizzle()\n"
        "#define main glsl_main\n"
    )
    tail = (
        "\n#undef uniform\n#undef in\n#undef xyz\n#undef xy\n#undef main\n"
        "}  // namespace glsl\n"
        '#include "marschner_harness.inc"\n'
    )
    return head + glsl_to_cpp(text) + tail


def build_marschner(reference: str, quiet: bool = False) -> list[str]:
    os.makedirs(OUT_DIR, exist_ok=True)
    out = []
    for part in ("m", "n"):
        src = translate_marschner(_read(reference, os.path.join(MARSCHNER_REL, f"cs_marschner_{part}.glsl")),
                                  reference)
        src = f"#define MARSCHNER_PART_{part.upper()} 1\n" + src
        out.append(_compile(os.path.join(OUT_DIR, f"marschner_{part}_ref.cc"),
                            os.path.join(OUT_DIR, f"libref_marschner_{part}.so"), src, reference, quiet))
    return out


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
    print(build_skin(args.reference))
    print(build_marschner(args.reference))
    return 0


if __name__ == "__main__":
    sys.exit(main())
