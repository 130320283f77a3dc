"""Compile the CPU oracle (TEST INFRASTRUCTURE ONLY).

oracle/hair_oracle.cc -> oracle/libhair_oracle.so, with OpenMP and with
floating-point contraction off so the FP32 instantiation rounds exactly as
written. When the reference tree is present, also builds the reference
shader as C++ into oracle/_ref/ (oracle/ref_glsl/make_ref.py).
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB = os.path.join(HERE, "libhair_oracle.so")
# The reference checkout: $BARBU_REFERENCE, else a `reference` directory
# beside this repository's root.
DEFAULT_REFERENCE = os.environ.get("BARBU_REFERENCE", os.path.join(os.path.dirname(ROOT), "reference"))


def build_oracle(quiet: bool = True) -> str:
    src = os.path.join(HERE, "hair_oracle.cc")
    cmd = [
        "g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
        "-fPIC", "-shared", "-I", os.path.join(ROOT, "include"), "-o", LIB, src,
    ]
    subprocess.run(cmd, check=True, capture_output=quiet)
    return LIB


def build_reference(reference: str = DEFAULT_REFERENCE, quiet: bool = True) -> str | None:
    """Builds oracle/_ref/libref_glsl.so, libref_tes.so, libref_skin.so and
    libref_marschner_{m,n}.so if the reference tree is present."""
    if not os.path.isdir(reference):
        return None
    sys.path.insert(0, os.path.join(HERE, "ref_glsl"))
    try:
        import make_ref  # noqa: E402
    finally:
        sys.path.pop(0)
    make_ref.build_tes(reference, quiet=quiet)
    make_ref.build_skin(reference, quiet=quiet)
    make_ref.build_marschner(reference, quiet=quiet)
    return make_ref.build(reference, quiet=quiet)


if __name__ == "__main__":
    print(build_oracle(quiet=False))
    print(build_reference(quiet=False))
