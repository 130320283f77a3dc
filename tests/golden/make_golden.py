"""Generate the golden vectors that pin the oracle to the reference shader.

Runs the reference's own hair-simulation compute shader
(src/shaders/hair/01_simulation/cs_simulation.glsl, compiled as C++ by
oracle/ref_glsl/make_ref.py, reading the reference tree in place) on seeded
inputs and stores inputs and outputs as .npz fixtures next to this script.
The reference tree only exists where the fixtures are made; the tests read
the fixtures.

Each fixture holds, for one scenario:
  roots, normals     (ns, 3) float32   strand roots and normals
  strand_seed        ()      uint64    seed of the length jitter
  pos0, vel0         (ns, 4, 4) float32  state after Hair::init_simulation
                     (oracle restatement of src/fx/hair.cc:262-288)
  dts                (F,) float32      dt of each frame
  bspheres           (F, 4) float32    uBoundingSphere of each frame
  scale              ()  float32       uScaleFactor (the app's lengthScale)
  snap_frames        (K,) int32        frames (1-based) that were stored
  pos_snap, vel_snap (K, ns, 4, 4) float32  shader output after those frames

Scenarios:
  scalp   the 448 roots of assets/models/InfiniteScan/Head_scalp.obj in the
          order Hair::setup gets them (unique v/vt/vn triples by first use,
          quads split (a,b,c),(c,d,a) as in mesh_data_manager.cc:199-208),
          lengthScale 1.45 (src/fx/hair.h:41), a sphere placed into the
          strands, dt = 1/60, 60 frames.
  sphere  512 roots on the unit sphere hanging under gravity onto a head
          sphere r = 1 that moves, variable dt, 60 frames.
  edge    hand-placed strands: roots inside the sphere, points on its
          surface, a zero-radius sphere, dt = 0 and dt = 0.1 frames.

ref_tess.npz pins the tessellation stream: the reference's tessellation
evaluation shader (src/shaders/hair/02_tess_stream/tes_stream_hair.glsl,
compiled as C++ by make_ref.py) on the scalp's positions after 60 frames
(the scalp fixture), the scalp mesh's own triangles, seeded tangents and
random buffer, for two settings of (instances, lines, subsegments):
  pos, tangents (448, 4, 4), faces (nf, 3) uint32, random (4096,),
  params_a/out_a, params_b/out_b: (instances, lines, subsegments, scale)
  and the (2 * segments, 4) vertices.

ref_skin.npz and ref_marschner.npz pin the skinning and Marschner oracles
to src/shaders/shared/inc_skinning.glsl and
src/shaders/hair/marschner/cs_marschner_{m,n}.glsl compiled as C++ (see
skin_case and marschner_case).

Usage: python tests/golden/make_golden.py --reference <tcoppex/barbu checkout>
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from barbu_gb300 import abi  # noqa: E402
from oracle import build as oracle_build  # noqa: E402

SEED = 0xBA5B0


def load_scalp(path: str):
    """Roots and normals of an OBJ in Hair::setup order."""
    v, vn = [], []
    faces = []
    with open(path, "r", encoding="utf-8") as f:
        for line in f:
            if line.startswith("v "):
                v.append([np.float32(t) for t in line.split()[1:4]])
            elif line.startswith("vn "):
                vn.append([np.float32(t) for t in line.split()[1:4]])
            elif line.startswith("f "):
                corners = [tuple(int(x) for x in c.split("/")) for c in line.split()[1:]]
                if len(corners) == 4:
                    a, b, c, d = corners
                    faces.extend([a, b, c, c, d, a])
                else:
                    faces.extend(corners[:3])
    seen = {}
    order = []
    for key in faces:
        if key not in seen:
            seen[key] = len(order)
            order.append(key)
    roots = np.array([v[k[0] - 1] for k in order], dtype=np.float32)
    normals = np.array([vn[k[2] - 1] for k in order], dtype=np.float32)
    return roots, normals


def load_scalp_faces(path: str) -> np.ndarray:
    """Triangles of the scalp as strand indices (Hair::setup order)."""
    faces = []
    with open(path, "r", encoding="utf-8") as f:
        for line in f:
            if line.startswith("f "):
                corners = [tuple(int(x) for x in c.split("/")) for c in line.split()[1:]]
                if len(corners) == 4:
                    a, b, c, d = corners
                    faces.extend([a, b, c, c, d, a])
                else:
                    faces.extend(corners[:3])
    seen = {}
    for key in faces:
        if key not in seen:
            seen[key] = len(seen)
    return np.array([seen[k] for k in faces], dtype=np.uint32).reshape(-1, 3)


def run(name, roots, normals, dts, bspheres, scale, snap_frames, seed=SEED):
    sp = abi.strand_params(4, abi.HS_LENGTH_REFERENCE, 0.5, 0.1, seed)
    pos0, vel0 = oracle.init(roots, normals, sp, dtype=np.float32)
    p, v = pos0.copy(), vel0.copy()
    ps, vs = [], []
    for f in range(len(dts)):
        p, v = oracle.ref_glsl_frame(p, v, float(dts[f]), float(scale), bspheres[f])
        if f + 1 in snap_frames:
            ps.append(p.copy())
            vs.append(v.copy())
    out = os.path.join(HERE, f"ref_{name}.npz")
    np.savez_compressed(
        out, roots=roots, normals=normals, strand_seed=np.uint64(seed), pos0=pos0, vel0=vel0,
        dts=np.asarray(dts, np.float32), bspheres=np.asarray(bspheres, np.float32),
        scale=np.float32(scale), snap_frames=np.asarray(snap_frames, np.int32),
        pos_snap=np.stack(ps), vel_snap=np.stack(vs))
    return out


def scalp_case(reference: str):
    roots, normals = load_scalp(os.path.join(reference, "assets", "models", "InfiniteScan", "Head_scalp.obj"))
    lo, hi = roots.min(0), roots.max(0)
    centre = 0.5 * (lo + hi)
    # A sphere just below the scalp's centre, reaching into the strands.
    r = 0.45 * float(np.max(hi - lo))
    c = centre - np.float32(0.25) * np.asarray([0, hi[1] - lo[1], 0], np.float32)
    F = 60
    bs = np.tile(np.asarray([c[0], c[1], c[2], r], np.float32), (F, 1))
    dts = np.full(F, 1.0 / 60.0, np.float32)
    return run("scalp", roots, normals, dts, bs, 1.45, [1, 2, 10, 60])


def sphere_case():
    rng = np.random.default_rng(SEED + 1)
    ns = 512
    d = rng.normal(size=(ns, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    roots = d.astype(np.float32)
    normals = roots.copy()
    F = 60
    t = np.cumsum(rng.uniform(1 / 90, 1 / 30, F))
    dts = np.diff(np.concatenate([[0.0], t])).astype(np.float32)
    bs = np.zeros((F, 4), np.float32)
    bs[:, 0] = 0.05 * np.sin(2 * np.pi * t)
    bs[:, 3] = 1.0
    return run("sphere", roots, normals, dts, bs, 1.45, [1, 2, 30, 60])


def edge_case():
    roots = np.array([
        [0.0, 0.5, 0.0],      # root inside the sphere (roots never collide)
        [0.0, 1.0, 0.0],      # root on the sphere, strand straight up
        [1.0, 0.0, 0.0],      # strand sideways, falls onto the sphere
        [0.0, -1.0, 0.0],     # strand under the sphere, hangs free
        [0.0, 0.0, 1.0],
        [-0.7, 0.7, 0.0],
        [3.0, 3.0, 3.0],      # far away
        [1e-3, 1.0, -1e-3],
    ], np.float32)
    normals = np.array([
        [0, 1, 0], [0, 1, 0], [1, 0, 0], [0, -1, 0], [0, 0, 1], [-0.7071068, 0.7071068, 0], [0, 1, 0], [0, 1, 0],
    ], np.float32)
    dts = np.array([1 / 60, 0.0, 1 / 60, 0.1, 1 / 30, 1 / 60, 1 / 60, 1 / 60], np.float32)
    bs = np.tile(np.array([0, 0, 0, 1.0], np.float32), (len(dts), 1))
    bs[6] = [0, 0, 0, 0.0]    # zero radius: nothing collides
    bs[7] = [0.2, 0.1, 0, 1.2]
    return run("edge", roots, normals, dts, bs, 1.45, [1, 2, 3, 4, 5, 6, 7, 8])


def tess_case(reference: str):
    obj = os.path.join(reference, "assets", "models", "InfiniteScan", "Head_scalp.obj")
    faces = load_scalp_faces(obj)
    scalp = np.load(os.path.join(HERE, "ref_scalp.npz"))
    pos = scalp["pos_snap"][-1]
    rng = np.random.default_rng(SEED + 7)
    tangents = rng.uniform(-0.1, 0.1, pos.shape).astype(np.float32)
    tangents[..., 3] = 0
    rand = rng.random(abi.HS_TESS_RANDOM_SIZE).astype(np.float32)
    params_a = (3, 2, 16, 1.45)   # Parameters_t::tess and lengthScale (src/fx/hair.h:33-42)
    params_b = (2, 3, 4, 1.0)
    fa, fb = faces[:16], faces[16:80]
    out_a = oracle.ref_tes_stream(pos, tangents, fa, rand, *params_a)
    out_b = oracle.ref_tes_stream(pos, tangents, fb, rand, *params_b)
    out = os.path.join(HERE, "ref_tess.npz")
    np.savez_compressed(out, pos=pos, tangents=tangents, faces_a=fa, faces_b=fb, random=rand,
                        params_a=np.asarray(params_a, np.float32), out_a=out_a,
                        params_b=np.asarray(params_b, np.float32), out_b=out_b)
    return out


def skin_case() -> str:
    """ref_skin.npz: the reference's dual-quaternion skinning
    (apply_skinning + skinning_DQBS, src/shaders/shared/inc_skinning.glsl,
    compiled as C++) of seeded rest points: the skinned cylinder's roots with
    their two-bone influences under the animated 4-bone rig, and random
    points with four random influences over an 8-bone palette, including
    first weights of 0 and exactly Epsilon() = 1e-6 (no skinning) and a
    bone whose quaternion is negated (antipodal to the others)."""
    from barbu_gb300 import scenarios
    spec = scenarios.skinned(ns=2048, npoints=4)
    rng = np.random.default_rng(SEED + 21)
    n = 2048
    rest = rng.uniform(-1.0, 2.5, (n, 3)).astype(np.float32)
    bones = rng.integers(0, 8, (n, 4)).astype(np.uint8)
    weights = rng.dirichlet([1.0, 1.0, 1.0, 1.0], n)[:, :3].astype(np.float32)
    weights[:16, 0] = 0.0
    weights[16:32, 0] = np.float32(1e-6)
    dq = oracle.matrix_to_dual_quat(np.concatenate([spec.rig.matrices(17), spec.rig.matrices(41)]))
    dq[5] = -dq[5]  # the same rotation, antipodal
    rest = np.concatenate([spec.roots, rest])
    bones = np.concatenate([spec.bones, bones])
    weights = np.concatenate([spec.weights, weights])
    out = oracle.ref_skin(rest, bones, weights, dq)
    path = os.path.join(HERE, "ref_skin.npz")
    np.savez_compressed(path, rest=rest, bones=bones, weights=weights, dq=dq, out=out)
    return path


def marschner_case() -> str:
    """ref_marschner.npz: the reference's Marschner tables (cs_marschner_m
    and cs_marschner_n, compiled as C++) for the reference's shading
    parameters at resolution 64, and for other parameters at 32."""
    sets = [(64, 1.55, 0.20, -5.0, 5.0), (32, 1.40, 0.55, -7.0, 8.0)]
    out = {}
    for k, (res, eta, absorption, ar, br) in enumerate(sets):
        m, n = oracle.ref_marschner(res, eta, absorption, ar, br)
        out[f"params_{k}"] = np.asarray([res, eta, absorption, ar, br], np.float32)
        out[f"m_{k}"] = m
        out[f"n_{k}"] = n
    path = os.path.join(HERE, "ref_marschner.npz")
    np.savez_compressed(path, **out)
    return path


def main() -> int:
    ap = argparse.ArgumentParser(description="generate golden vectors from the reference shader")
    ap.add_argument("--reference", required=True, help="root of the tcoppex/barbu checkout")
    args = ap.parse_args()
    oracle_build.build_oracle()
    oracle_build.build_reference(args.reference)
    for out in (scalp_case(args.reference), sphere_case(), edge_case(), tess_case(args.reference), skin_case(),
                marschner_case()):
        z = np.load(out)
        print(out, os.path.getsize(out), "bytes", {k: z[k].shape for k in z.files})
    return 0


if __name__ == "__main__":
    sys.exit(main())
