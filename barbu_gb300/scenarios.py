"""Seeded synthetic grooms for the benchmark workloads.

The reference has no dataset: its only input is one scalp mesh
(assets/models/InfiniteScan/Head_scalp.obj, 448 roots). These generators
produce the workload shapes the benchmarks are quoted on, from fixed seeds:

  plain   4,096 roots uniform on the unit sphere, N = 16, length 0.5 in
          equal segments, DFTL S = 4, damping 0.9, one sphere r = 1 that
          moves with the roots, x = 0.2 sin(2 pi t) (rigid root transform).
  large   262,144 roots on an icosphere of 5 subdivisions (20,480 faces):
          root k lies on face floor(k * 20480 / 262144) at hashed barycentric
          coordinates, projected on the unit sphere, then displaced by hash
          noise of amplitude 0.05; normal = the projected direction. N = 32,
          lengths uniform in [0.3, 0.8], 16 spheres with r in [0.1, 0.4]
          centred at hashed directions and distances in [1.0, 1.6], wind
          (1.5 sin 0.7t, 0, 0.5) with per-strand jitter +-20%, S = 8.
  batched 64 grooms with strand counts log-uniform in [1,024, 131,072],
          N from {8, 16, 24, 32}, each with its own rigid root motion
          (rotation <= 30 deg/s about a hashed axis, translation amplitude
          0.3) and 1..16 spheres.
  skinned 1,048,576 roots on the side of a cylinder (radius 0.5, height 2,
          8 rings x 64 segments = 448 quads; root k on quad
          floor(k * 448 / ns) at hashed coordinates, normal radial),
          N = 64, length 0.6, S = 8, DFTL, roots skinned by dual-quaternion
          blending to a chain of 4 bones along the axis, 2 weights per root
          (the two bones around its height, linear in height). Each bone's
          local rotation follows a seeded random walk (axis-angle vector,
          steps of at most 1.5 deg, pulled back by 2 % a frame, magnitude
          clamped to 25 deg: at most 2 deg of change per frame). 32
          spheres (r in [0.1, 0.25]) in a shell 0.7-1.1 from the axis ride
          on the bone at their height.
Roots are generated in float64 and rounded to float32 once.
"""
from __future__ import annotations

import dataclasses
import functools
import math

import numpy as np

from . import abi

SEED = 0xBA5B0


def _rng(seed: int, stream: int) -> np.random.Generator:
    return np.random.default_rng([seed, stream])


def _normalize(v: np.ndarray) -> np.ndarray:
    n = np.sqrt(v[..., 0] * v[..., 0] + v[..., 1] * v[..., 1] + v[..., 2] * v[..., 2])
    return v / n[..., None]


@functools.lru_cache(maxsize=8)
def icosphere(subdiv: int):
    """Vertices (float64, unit) and faces of a subdivided icosahedron."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    V = [np.asarray(v, np.float64) for v in verts]
    V = [v / math.sqrt(float(v @ v)) for v in V]
    F = faces
    for _ in range(subdiv):
        cache = {}
        nf = []

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = 0.5 * (V[a] + V[b])
                V.append(m / math.sqrt(float(m @ m)))
                cache[key] = len(V) - 1
            return cache[key]

        for a, b, c in F:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        F = nf
    return np.asarray(V), np.asarray(F, np.int64)


def _morton_order(p: np.ndarray, bits: int = 10) -> np.ndarray:
    """Indices sorting points in [-1, 1]^3 along a Z-order curve."""
    q = np.clip(((p + 1.0) * 0.5 * ((1 << bits) - 1)).astype(np.int64), 0, (1 << bits) - 1)
    code = np.zeros(len(p), dtype=np.int64)
    for b in range(bits):
        for axis in range(3):
            code |= ((q[:, axis] >> b) & 1) << (3 * b + axis)
    return np.argsort(code, kind="stable")


def sphere_roots(ns: int, seed: int, stream: int = 1):
    """Uniform roots on the unit sphere, normals = roots, in Z-order: a
    scalp mesh's vertices are spatially coherent, and so are these, which
    keeps the 32 strands of a warp near one another."""
    d = _normalize(_rng(seed, stream).normal(size=(ns, 3)))
    d = d[_morton_order(d)]
    return d.astype(np.float32), d.astype(np.float32)


def icosphere_roots(ns: int, seed: int, subdiv: int = 5, noise: float = 0.05):
    V, F = icosphere(subdiv)
    rng = _rng(seed, 2)
    face = (np.arange(ns, dtype=np.int64) * len(F)) // ns
    u = rng.random(ns)
    v = rng.random(ns)
    flip = u + v > 1.0
    u[flip], v[flip] = 1.0 - u[flip], 1.0 - v[flip]
    a, b, c = V[F[face, 0]], V[F[face, 1]], V[F[face, 2]]
    p = a + u[:, None] * (b - a) + v[:, None] * (c - a)
    n = _normalize(p)
    roots = n + noise * (2.0 * rng.random((ns, 3)) - 1.0)
    return roots.astype(np.float32), n.astype(np.float32)


def shell_spheres(k: int, seed: int, r_lo=0.1, r_hi=0.4, d_lo=1.0, d_hi=1.6, stream: int = 3):
    rng = _rng(seed, stream)
    dirs = _normalize(rng.normal(size=(k, 3)))
    dist = rng.uniform(d_lo, d_hi, size=k)
    r = rng.uniform(r_lo, r_hi, size=k)
    out = np.zeros((k, 4), np.float32)
    out[:, :3] = dirs * dist[:, None]
    out[:, 3] = r
    return out


def wind_at(t: float) -> np.ndarray:
    """(1.5 sin(0.7 t), 0, 0.5), evaluated in float64 then rounded."""
    return np.array([1.5 * math.sin(0.7 * t), 0.0, 0.5], np.float32)


def translation_x(t: float, amp: float = 0.2) -> np.ndarray:
    """Column-major 4x4 translation by (amp sin(2 pi t), 0, 0)."""
    m = np.eye(4, dtype=np.float32)
    m[3, 0] = np.float32(amp * math.sin(2.0 * math.pi * t))
    return m.reshape(16)


def rigid_motion(t: float, axis: np.ndarray, omega_deg: float, amp: float, phase: float) -> np.ndarray:
    """Rotation by omega*t about axis, translation amp*sin(2 pi t + phase)
    along the axis' perpendicular; column-major 4x4 (float32)."""
    ang = math.radians(omega_deg) * t
    x, y, z = axis
    c, s = math.cos(ang), math.sin(ang)
    C = 1.0 - c
    R = np.array([[c + x * x * C, x * y * C - z * s, x * z * C + y * s],
                  [y * x * C + z * s, c + y * y * C, y * z * C - x * s],
                  [z * x * C - y * s, z * y * C + x * s, c + z * z * C]])
    M = np.eye(4)
    M[:3, :3] = R
    M[:3, 3] = amp * math.sin(2.0 * math.pi * t + phase) * np.array([z, x, y])
    return M.T.astype(np.float32).reshape(16)  # column-major


@dataclasses.dataclass
class GroomSpec:
    roots: np.ndarray
    normals: np.ndarray
    strand: abi.StrandParams
    sim: abi.SimParams
    lengths: np.ndarray | None
    spheres: np.ndarray
    wind_jitter: float = 0.0
    moving_roots: str = "none"          # "none" | "translate_x" | "rigid"
    axis: np.ndarray | None = None
    omega_deg: float = 0.0
    amp: float = 0.0
    phase: float = 0.0
    wind: bool = False

    @property
    def nstrands(self) -> int:
        return self.roots.shape[0]

    @property
    def npoints(self) -> int:
        return int(self.strand.points_per_strand)

    def transform(self, t: float) -> np.ndarray | None:
        if self.moving_roots == "translate_x":
            return translation_x(t, self.amp)
        if self.moving_roots == "rigid":
            return rigid_motion(t, self.axis, self.omega_deg, self.amp, self.phase)
        return None

    def spheres_at(self, t: float) -> np.ndarray:
        m = self.transform(t)
        if m is None or self.moving_roots != "translate_x":
            return self.spheres
        s = self.spheres.copy()
        s[:, 0] += m[12]
        return s


def plain(ns: int = 4096, npoints: int = 16, seed: int = SEED + 1) -> GroomSpec:
    roots, normals = sphere_roots(ns, seed)
    sp = abi.strand_params(npoints, abi.HS_LENGTH_TOTAL, 0.5, 0.0, seed)
    sim = abi.sim_params_dftl(substeps=4, damping=0.9, root_mode=abi.HS_ROOT_RIGID)
    return GroomSpec(roots, normals, sp, sim, None, np.array([[0, 0, 0, 1.0]], np.float32),
                     moving_roots="translate_x", amp=0.2)


def large(ns: int = 262144, npoints: int = 32, seed: int = SEED + 2, nspheres: int = 16) -> GroomSpec:
    roots, normals = icosphere_roots(ns, seed)
    lengths = _rng(seed, 4).uniform(0.3, 0.8, size=ns).astype(np.float32)
    sp = abi.strand_params(npoints, abi.HS_LENGTH_TOTAL, 0.5, 0.0, seed)
    sim = abi.sim_params_dftl(substeps=8, damping=0.9, wind_jitter=0.2)
    return GroomSpec(roots, normals, sp, sim, lengths, shell_spheres(nspheres, seed), wind_jitter=0.2, wind=True)


def batched(ngrooms: int = 64, seed: int = SEED + 3, lo: int = 1024, hi: int = 131072,
            scale: float = 1.0) -> list[GroomSpec]:
    rng = _rng(seed, 5)
    out = []
    for g in range(ngrooms):
        ns = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi))) * scale))
        ns = max(1, ns)
        npoints = int(rng.choice([8, 16, 24, 32]))
        gseed = seed * 1000 + g
        roots, normals = sphere_roots(ns, gseed)
        lengths = rng.uniform(0.3, 0.8, size=ns).astype(np.float32)
        sp = abi.strand_params(npoints, abi.HS_LENGTH_TOTAL, 0.5, 0.0, gseed)
        sim = abi.sim_params_dftl(substeps=8, damping=0.9, root_mode=abi.HS_ROOT_RIGID)
        k = int(rng.integers(1, 17))
        spheres = shell_spheres(k, gseed)
        axis = _normalize(rng.normal(size=3))
        out.append(GroomSpec(roots, normals, sp, sim, lengths, spheres, moving_roots="rigid", axis=axis,
                             omega_deg=float(rng.uniform(0.0, 30.0)), amp=0.3,
                             phase=float(rng.uniform(0, 2 * math.pi))))
    return out


# ---- skinned (cylinder, 4-bone chain) -------------------------------------

CYL_RADIUS = 0.5
CYL_HEIGHT = 2.0
CYL_RINGS = 8
CYL_SEGMENTS = 64
SKIN_BONES = 4


def cylinder_roots(ns: int, seed: int, radius: float = CYL_RADIUS, height: float = CYL_HEIGHT,
                   rings: int = CYL_RINGS, segments: int = CYL_SEGMENTS):
    """Roots on the side of a y-axis cylinder, quad by quad (consecutive
    strands share a quad), normals radial."""
    rng = _rng(seed, 6)
    nquads = (rings - 1) * segments
    quad = (np.arange(ns, dtype=np.int64) * nquads) // ns
    ring, seg = quad // segments, quad % segments
    u, v = rng.random(ns), rng.random(ns)
    theta = (seg + u) * (2.0 * math.pi / segments)
    y = (ring + v) * (height / (rings - 1))
    n = np.stack([np.cos(theta), np.zeros(ns), np.sin(theta)], axis=1)
    roots = np.stack([radius * np.cos(theta), y, radius * np.sin(theta)], axis=1)
    return roots.astype(np.float32), n.astype(np.float32)


def cylinder_skin(roots: np.ndarray, height: float = CYL_HEIGHT, nbones: int = SKIN_BONES):
    """Two influences per root: the bones below and above its height,
    weights linear in height. The heavier bone goes in slot 0 (a first
    weight <= 1e-6 would switch skinning off) and the other in slot 3,
    slots 1-2 carry weight 0: (b_hi, b_hi, b_hi, b_lo), (w, 0, 0)."""
    seg = height / (nbones - 1)
    y = roots[:, 1].astype(np.float64)
    k = np.clip(np.floor(y / seg).astype(np.int64), 0, nbones - 2)
    f = np.clip((y - k * seg) / seg, 0.0, 1.0)
    heavy_hi = f >= 0.5
    b_main = np.where(heavy_hi, k + 1, k)
    b_other = np.where(heavy_hi, k, k + 1)
    w_main = np.where(heavy_hi, f, 1.0 - f)
    bones = np.stack([b_main, b_main, b_main, b_other], axis=1).astype(np.uint8)
    weights = np.zeros((len(y), 3), np.float32)
    weights[:, 0] = w_main.astype(np.float32)
    return bones, weights


def _axis_angle_matrix(v: np.ndarray) -> np.ndarray:
    ang = float(np.linalg.norm(v))
    if ang == 0.0:
        return np.eye(3)
    x, y, z = v / ang
    c, s = math.cos(ang), math.sin(ang)
    C = 1.0 - c
    return np.array([[c + x * x * C, x * y * C - z * s, x * z * C + y * s],
                     [y * x * C + z * s, c + y * y * C, y * z * C - x * s],
                     [z * x * C - y * s, z * y * C + x * s, c + z * z * C]])


class SkinRig:
    """A chain of bones along the cylinder axis (bone b's joint at height
    b * height / (nbones - 1)), animated by seeded random walks. Frame f's
    skinning matrices (global pose x inverse bind) are column-major 4x4,
    computed in float64 and rounded once."""

    def __init__(self, seed: int, nbones: int = SKIN_BONES, height: float = CYL_HEIGHT,
                 step_deg: float = 1.5, pull: float = 0.02, clamp_deg: float = 25.0):
        self.seed, self.nbones, self.height = seed, nbones, height
        self.step, self.pull, self.clamp = math.radians(step_deg), pull, math.radians(clamp_deg)
        self.joint_y = np.arange(nbones) * (height / (nbones - 1))
        self._angles = [np.zeros((nbones, 3))]

    def angles(self, frame: int) -> np.ndarray:
        while len(self._angles) <= frame:
            f = len(self._angles)
            rng = _rng(self.seed, 1000 + f)
            d = _normalize(rng.normal(size=(self.nbones, 3))) * (self.step * rng.random((self.nbones, 1)))
            a = (1.0 - self.pull) * self._angles[-1] + d
            n = np.linalg.norm(a, axis=1, keepdims=True)
            a = np.where(n > self.clamp, a * (self.clamp / np.maximum(n, 1e-300)), a)
            self._angles.append(a)
        return self._angles[frame]

    def global_poses(self, frame: int) -> list[np.ndarray]:
        a = self.angles(frame)
        G = []
        for b in range(self.nbones):
            L = np.eye(4)
            L[:3, :3] = _axis_angle_matrix(a[b])
            L[1, 3] = self.joint_y[b] - (self.joint_y[b - 1] if b > 0 else 0.0)
            G.append(L if b == 0 else G[b - 1] @ L)
        return G

    def matrices(self, frame: int) -> np.ndarray:
        out = np.zeros((self.nbones, 16), np.float32)
        for b, G in enumerate(self.global_poses(frame)):
            inv_bind = np.eye(4)
            inv_bind[1, 3] = -self.joint_y[b]
            out[b] = (G @ inv_bind).T.astype(np.float32).reshape(16)
        return out


def skinned_spheres(k: int, seed: int, height: float = CYL_HEIGHT, nbones: int = SKIN_BONES):
    """Rest spheres around the cylinder and the bone each one rides on."""
    rng = _rng(seed, 7)
    theta = rng.uniform(0.0, 2.0 * math.pi, k)
    dist = rng.uniform(0.7, 1.1, k)
    y = rng.uniform(-0.3, height, k)
    r = rng.uniform(0.1, 0.25, k)
    rest = np.stack([dist * np.cos(theta), y, dist * np.sin(theta), r], axis=1)
    bone = np.clip(np.rint(y / (height / (nbones - 1))), 0, nbones - 1).astype(np.int64)
    return rest, bone


@dataclasses.dataclass
class SkinnedSpec:
    roots: np.ndarray
    normals: np.ndarray
    strand: abi.StrandParams
    sim: abi.SimParams
    bones: np.ndarray
    weights: np.ndarray
    rig: SkinRig
    sphere_rest: np.ndarray
    sphere_bone: np.ndarray
    lengths: np.ndarray | None = None

    @property
    def nstrands(self) -> int:
        return self.roots.shape[0]

    @property
    def npoints(self) -> int:
        return int(self.strand.points_per_strand)

    def spheres_at(self, frame: int) -> np.ndarray:
        """Each sphere moved rigidly by its bone's skinning matrix (float64)."""
        out = np.zeros((len(self.sphere_rest), 4), np.float32)
        M = self.rig.matrices(frame).astype(np.float64).reshape(-1, 4, 4).transpose(0, 2, 1)
        for j, (s, b) in enumerate(zip(self.sphere_rest, self.sphere_bone)):
            c = M[b] @ np.array([s[0], s[1], s[2], 1.0])
            out[j, :3] = c[:3]
            out[j, 3] = s[3]
        return out


def skinned(ns: int = 1048576, npoints: int = 64, seed: int = SEED + 5, nspheres: int = 32,
            substeps: int = 8, length: float = 0.6) -> SkinnedSpec:
    roots, normals = cylinder_roots(ns, seed)
    sp = abi.strand_params(npoints, abi.HS_LENGTH_TOTAL, length, 0.0, seed)
    sim = abi.sim_params_dftl(substeps=substeps, damping=0.9, root_mode=abi.HS_ROOT_SKINNED)
    bones, weights = cylinder_skin(roots)
    rest, bone = skinned_spheres(nspheres, seed)
    return SkinnedSpec(roots, normals, sp, sim, bones, weights, SkinRig(seed), rest, bone)
