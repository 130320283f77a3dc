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
