"""The C++ wrapper (include/hairsim.hpp) running frames on the GPU.

A C++ program built against the library drives hs::Hair exactly as the
reference's renderer drives its Hair class (src/core/renderer.cc:69-81:
set the bounding sphere, update(dt), read the positions back), on the
448-root scalp of the golden fixture, and its positions after 10 frames
must equal the reference shader's (tests/golden/ref_scalp.npz) bit for bit.
"""
from __future__ import annotations

import os
import subprocess
import tempfile

import numpy as np
import pytest

from tests import util

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROG = r'''
#include <cstdio>
#include <vector>
#include "hairsim.hpp"
static std::vector<float> slurp(const char* path, size_t n) {
  std::vector<float> v(n);
  FILE* f = std::fopen(path, "rb");
  if (!f || std::fread(v.data(), sizeof(float), n, f) != n) throw std::runtime_error(path);
  std::fclose(f);
  return v;
}
int main(int argc, char** argv) {
  // argv: dir, nroots, frames, seed, scale
  const std::string dir = argv[1];
  const size_t n = std::stoul(argv[2]);
  const int frames = std::stoi(argv[3]);
  hs::HairParameters p;
  p.seed = std::stoull(argv[4]);
  p.length_scale = std::stof(argv[5]);
  const auto roots = slurp((dir + "/roots.bin").c_str(), 3 * n);
  const auto normals = slurp((dir + "/normals.bin").c_str(), 3 * n);
  const auto dts = slurp((dir + "/dts.bin").c_str(), frames);
  const auto spheres = slurp((dir + "/spheres.bin").c_str(), 4 * frames);
  hs::Hair hair(p);
  hair.init();
  hair.setup(roots, normals);
  for (int f = 0; f < frames; ++f) {
    hair.set_bounding_sphere({spheres[4 * f], spheres[4 * f + 1], spheres[4 * f + 2], spheres[4 * f + 3]});
    hair.update(dts[f]);
  }
  const auto out = hair.readback();
  FILE* o = std::fopen((dir + "/out.bin").c_str(), "wb");
  std::fwrite(out.data(), sizeof(float), out.size(), o);
  std::fclose(o);
  return 0;
}
'''


def test_cpp_wrapper_frames_match_reference_shader(built_library):
    g = util.load_golden("scalp")
    frames = 10
    k = list(g["snap_frames"]).index(frames)
    libdir = os.path.dirname(built_library)
    with tempfile.TemporaryDirectory() as d:
        for name, a in (("roots", g["roots"]), ("normals", g["normals"]), ("dts", g["dts"][:frames]),
                        ("spheres", g["bspheres"][:frames])):
            np.ascontiguousarray(a, np.float32).tofile(os.path.join(d, name + ".bin"))
        src = os.path.join(d, "hair.cc")
        open(src, "w").write(PROG)
        exe = os.path.join(d, "hair")
        subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), src, "-o", exe,
                        "-L", libdir, "-lhairsim", f"-Wl,-rpath,{libdir}"], check=True)
        r = subprocess.run([exe, d, str(len(g["roots"])), str(frames), str(int(g["strand_seed"])),
                            repr(float(g["scale"]))], capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, r.stdout + r.stderr
        out = np.fromfile(os.path.join(d, "out.bin"), np.float32).reshape(g["pos_snap"][k].shape)
    util.assert_bit_equal(out, g["pos_snap"][k], "hs::Hair after 10 frames vs the reference shader")
