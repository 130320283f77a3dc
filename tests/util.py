"""Helpers shared by the tests: golden fixtures, strand lengths, checks."""
from __future__ import annotations

import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ("scalp", "sphere", "edge")


def load_golden(name: str) -> dict:
    z = np.load(os.path.join(GOLDEN, f"ref_{name}.npz"))
    return {k: z[k] for k in z.files}


def strand_lengths(pos, scale: float = 1.0) -> np.ndarray:
    """Settled strand length: scale * sum of rest lengths, per strand."""
    return scale * pos[:, 1:, 3].astype(np.float64).sum(axis=1)


def finite_strands(a) -> np.ndarray:
    return np.isfinite(a).all(axis=(1, 2))


def bits(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


def assert_bit_equal(a, b, what: str):
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = np.ascontiguousarray(b, dtype=np.float32)
    assert a.shape == b.shape, (what, a.shape, b.shape)
    diff = bits(a) != bits(b)
    if diff.any():
        idx = np.argwhere(diff)[:5]
        raise AssertionError(f"{what}: {int(diff.sum())} words differ, first at {idx.tolist()}: "
                             f"{a[tuple(idx[0])]!r} vs {b[tuple(idx[0])]!r}")


def max_pos_error_rel(p32, p64, lengths) -> float:
    """max over strands of max point distance / strand length."""
    d = np.linalg.norm(p32[..., :3].astype(np.float64) - p64[..., :3], axis=-1).max(axis=1)
    return float((d / lengths).max())


def segment_lengths(pos) -> np.ndarray:
    p = pos[..., :3].astype(np.float64)
    return np.linalg.norm(p[:, 1:] - p[:, :-1], axis=-1)


def random_roots_on_sphere(ns: int, seed: int, radius: float = 1.0):
    rng = np.random.default_rng(seed)
    d = rng.normal(size=(ns, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return (radius * d).astype(np.float32), d.astype(np.float32)


SIDE_SPHERES = np.array([[0.75, -1.35, 0.0, 0.3], [-0.75, -1.35, 0.0, 0.3],
                         [0.0, -1.35, 0.75, 0.3], [0.0, -1.35, -0.75, 0.3]], np.float32)


def hanging_roots(ns: int, seed: int, cap: float = -0.6):
    """Roots on the lower cap of the unit sphere (y < cap)."""
    rng = np.random.default_rng(seed)
    out = []
    while sum(len(o) for o in out) < ns:
        d = rng.normal(size=(4 * ns, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        out.append(d[d[:, 1] < cap])
    return np.concatenate(out)[:ns].astype(np.float32)


def hanging_spec(ns: int, n: int, substeps: int = 4, spheres=None, seed: int = 5):
    """A well-conditioned DFTL scene: strands hanging straight down from the
    lower cap, swinging in the jittered wind; optionally four spheres beside
    them that the swinging strands brush against."""
    from barbu_gb300 import abi, scenarios
    roots = hanging_roots(ns, seed)
    normals = np.tile(np.array([[0.0, -1.0, 0.0]], np.float32), (ns, 1))
    lengths = np.random.default_rng(seed).uniform(0.3, 0.8, ns).astype(np.float32)
    sp = abi.strand_params(n, abi.HS_LENGTH_TOTAL, 0.5, 0.0, 7)
    sim = abi.sim_params_dftl(substeps=substeps, damping=0.9, wind_jitter=0.2)
    sph = SIDE_SPHERES if spheres == "side" else np.zeros((0, 4), np.float32)
    return scenarios.GroomSpec(roots, normals, sp, sim, lengths, sph, wind=True)
