"""CPU oracle for the hair-strand simulation step.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, always as the checker. The library in
barbu_gb300/ never imports it.

Two native pieces sit behind this module:
  * libhair_oracle.so (hair_oracle.cc): the restatement, in FP32 and FP64.
    Reference mode follows src/shaders/hair/01_simulation/cs_simulation.glsl
    and is pinned bit for bit against the shader's own text through the
    golden vectors in tests/golden/. DFTL mode follows Mueller et al. 2012
    and is unpinned by the reference.
  * _ref/libref_glsl.so: the reference shader compiled as C++
    (ref_glsl/make_ref.py). Only buildable where the reference tree exists;
    used to make and check the golden vectors.

Arrays are numpy, shaped (nstrands, npoints, 4), strand-major like the
reference's position/velocity streams (src/fx/hair.cc:242-288).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from barbu_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libhair_oracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libref_glsl.so")
REF_TES_PATH = os.path.join(HERE, "_ref", "libref_tes.so")

_lib = None
_ref = None

_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


def _vp(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def lib():
    """Loads (building first if needed) libhair_oracle.so."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            from oracle import build as _b
            _b.build_oracle()
        L = C.CDLL(LIB_PATH)
        for name in ("oracle_frame_f32", "oracle_frame_f64"):
            fn = getattr(L, name)
            fn.restype = C.c_int
            fn.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32,
                           C.POINTER(abi.SimParams), C.c_uint64, C.c_float, C.c_void_p,
                           C.c_uint32, C.c_void_p, C.c_void_p, C.c_int]
        for name in ("oracle_frame_form_f32", "oracle_frame_form_f64"):
            fn = getattr(L, name)
            fn.restype = C.c_int
            fn.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32,
                           C.POINTER(abi.SimParams), C.c_uint64, C.c_float, C.c_void_p,
                           C.c_uint32, C.c_void_p, C.c_void_p, C.c_int, C.c_int]
        for name in ("oracle_init_f32", "oracle_init_f64"):
            fn = getattr(L, name)
            fn.restype = C.c_int
            fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32,
                           C.POINTER(abi.StrandParams)]
        for name in ("oracle_rigid_targets_f32", "oracle_rigid_targets_f64"):
            fn = getattr(L, name)
            fn.restype = None
            fn.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]
        L.oracle_hash_u01.restype = C.c_float
        for name in ("oracle_skin_targets_f32", "oracle_skin_targets_f64"):
            fn = getattr(L, name)
            fn.restype = None
            fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]
        L.oracle_tess_f32.restype = None
        L.oracle_tess_f32.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p,
                                      C.c_uint32, C.c_uint32, C.c_uint32, C.c_float, C.c_void_p]
        for name in ("oracle_marschner_f32", "oracle_marschner_f64"):
            fn = getattr(L, name)
            fn.restype = None
            fn.argtypes = [C.c_uint32, C.c_float, C.c_float, C.c_float, C.c_float, C.c_void_p, C.c_void_p]
        L.oracle_matrix_to_dual_quat.restype = None
        L.oracle_matrix_to_dual_quat.argtypes = [C.c_void_p, C.c_void_p]
        L.oracle_hash_u01.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32]
        L.oracle_max_threads.restype = C.c_int
        _lib = L
    return _lib


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def _suffix(dtype) -> str:
    dt = np.dtype(dtype)
    if dt == np.float32:
        return "f32"
    if dt == np.float64:
        return "f64"
    raise TypeError(f"oracle runs in float32 or float64, not {dt}")


def init(roots, normals, sp: abi.StrandParams, dtype=np.float64, lengths=None):
    """Hair::init_simulation (src/fx/hair.cc:262-288) -> (pos, vel)."""
    roots = np.ascontiguousarray(roots, dtype=np.float32).reshape(-1, 3)
    normals = np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3)
    ns = roots.shape[0]
    n = int(sp.points_per_strand)
    pos = np.zeros((ns, n, 4), dtype=dtype)
    vel = np.zeros((ns, n, 4), dtype=dtype)
    keep = None
    if lengths is not None:
        keep = np.ascontiguousarray(lengths, dtype=np.float32)
        sp.lengths = keep.ctypes.data_as(C.POINTER(C.c_float))
    rc = getattr(lib(), "oracle_init_" + _suffix(dtype))(
        _vp(pos), _vp(vel), _vp(roots), _vp(normals), ns, C.byref(sp))
    if keep is not None:
        sp.lengths = None
    if rc != 0:
        raise ValueError("oracle_init rejected its arguments")
    return pos, vel


FORM_CONTRACT, FORM_WORLD, FORM_SEGMENT = 0, 1, 2


def frame(pos, vel, sim: abi.SimParams, dt: float, *, seed: int = 0, wind=None, spheres=None,
          root_targets=None, strand_base: int = 0, nthreads: int = 0, form: int = FORM_CONTRACT):
    """One frame (Hair::update) in place on pos, vel of shape (ns, N, 4).

    form (DFTL mode only): FORM_CONTRACT runs the library's arithmetic
    (the segment form in float32, world coordinates in float64);
    FORM_WORLD and FORM_SEGMENT pick one restatement in either precision."""
    assert pos.flags.c_contiguous and vel.flags.c_contiguous and pos.dtype == vel.dtype
    ns, n, four = pos.shape
    assert four == 4 and vel.shape == pos.shape
    w = None if wind is None else np.ascontiguousarray(wind, dtype=np.float32).reshape(3)
    sph = None
    nsph = 0
    if spheres is not None:
        sph = np.ascontiguousarray(spheres, dtype=np.float32).reshape(-1, 4)
        nsph = sph.shape[0]
    tg = None
    if root_targets is not None:
        tg = np.ascontiguousarray(root_targets, dtype=pos.dtype).reshape(ns, 3)
    rc = getattr(lib(), "oracle_frame_form_" + _suffix(pos.dtype))(
        _vp(pos), _vp(vel), ns, n, strand_base, C.byref(sim), seed, dt, _vp(w), nsph, _vp(sph),
        _vp(tg), nthreads, form)
    if rc != 0:
        raise ValueError("oracle_frame rejected its arguments")


def rigid_targets(rest_roots, m, dtype=np.float64):
    """t = M * r for each rest root, M 4x4 column-major (16 floats)."""
    rest = np.ascontiguousarray(rest_roots, dtype=np.float32).reshape(-1, 3)
    mm = np.ascontiguousarray(m, dtype=np.float32).reshape(16)
    out = np.zeros((rest.shape[0], 3), dtype=dtype)
    getattr(lib(), "oracle_rigid_targets_" + _suffix(dtype))(_vp(out), _vp(rest), rest.shape[0], _vp(mm))
    return out


def skin_targets(rest_roots, bones, weights, dq, dtype=np.float64):
    """Dual-quaternion skinned root targets (see oracle_skin_targets_*):
    rest (ns, 3), bones (ns, 4) uint8, weights (ns, 3), dq (nbones, 8)."""
    rest = np.ascontiguousarray(rest_roots, dtype=np.float32).reshape(-1, 3)
    b = np.ascontiguousarray(bones, dtype=np.uint8).reshape(-1, 4)
    w = np.ascontiguousarray(weights, dtype=np.float32).reshape(-1, 3)
    q = np.ascontiguousarray(dq, dtype=np.float32).reshape(-1, 8)
    assert b.shape[0] == w.shape[0] == rest.shape[0] and int(b.max(initial=0)) < q.shape[0]
    out = np.zeros((rest.shape[0], 3), dtype=dtype)
    getattr(lib(), "oracle_skin_targets_" + _suffix(dtype))(_vp(out), _vp(rest), _vp(b), _vp(w), rest.shape[0], _vp(q))
    return out


def matrix_to_dual_quat(m):
    """Rigid 4x4 column-major matrices (nb, 16) -> dual quaternions (nb, 8), float."""
    mm = np.ascontiguousarray(m, dtype=np.float32).reshape(-1, 16)
    out = np.zeros((mm.shape[0], 8), np.float32)
    for k in range(mm.shape[0]):
        lib().oracle_matrix_to_dual_quat(_vp(mm[k]), _vp(out[k]))
    return out


def tess(pos, tangents, faces, random, ninstances=3, nlines=2, nsubsegments=16, scale=1.45):
    """The tessellation stream (see oracle_tess_f32): pos, tangents (ns, N, 4)
    float32, faces (nf, 3), random (4096,). Returns (2 * segments, 4)."""
    p = np.ascontiguousarray(pos, dtype=np.float32)
    t = np.ascontiguousarray(tangents, dtype=np.float32)
    assert p.shape == t.shape and p.ndim == 3 and p.shape[2] == 4
    f = np.ascontiguousarray(faces, dtype=np.uint32).reshape(-1, 3)
    r = np.ascontiguousarray(random, dtype=np.float32).reshape(-1)
    assert r.size == abi.HS_TESS_RANDOM_SIZE and (f.size == 0 or int(f.max()) < p.shape[0])
    n = p.shape[1]
    segs = ninstances * f.shape[0] * (n - 1) * nlines * nsubsegments
    out = np.zeros((2 * segs, 4), np.float32)
    lib().oracle_tess_f32(_vp(p), _vp(t), n, _vp(f), f.shape[0], _vp(r), ninstances, nlines, nsubsegments,
                          float(np.float32(scale)), _vp(out))
    return out


def marschner(resolution=128, eta=1.55, absorption=0.2, ar=-5.0, br=5.0, dtype=np.float64):
    """The Marschner M and N tables (see oracle_marschner_*): two
    (resolution, resolution, 4) arrays, row y = sin(theta_r) or cos(theta_d)."""
    m = np.zeros((resolution, resolution, 4), dtype)
    n = np.zeros((resolution, resolution, 4), dtype)
    getattr(lib(), "oracle_marschner_" + _suffix(dtype))(resolution, eta, absorption, ar, br, _vp(m), _vp(n))
    return m, n


def hash_u01(seed: int, stream: int, idx: int) -> float:
    return float(lib().oracle_hash_u01(seed, stream, idx))


# ---- the reference shader compiled as C++ ----------------------------------

def ref_glsl_available() -> bool:
    return os.path.exists(REF_PATH)


def _ref_lib():
    global _ref
    if _ref is None:
        L = C.CDLL(REF_PATH)
        L.ref_glsl_dispatch.restype = C.c_int
        L.ref_glsl_dispatch.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32,
                                        C.c_float, C.c_float, C.c_void_p]
        L.ref_glsl_local_size.restype = C.c_int
        _ref = L
    return _ref


def ref_glsl_local_size() -> int:
    return int(_ref_lib().ref_glsl_local_size())


def ref_glsl_frame(pos, vel, dt: float, scale: float, bsphere):
    """Hair::update through the reference shader: dispatch then swap.

    pos, vel: float32 (nroots, 4, 4). Returns the new (pos, vel)."""
    assert pos.dtype == np.float32 and vel.dtype == np.float32
    ns, n, _ = pos.shape
    assert n == ref_glsl_local_size()
    pw = np.zeros_like(pos)
    vw = np.zeros_like(vel)
    bs = np.ascontiguousarray(bsphere, dtype=np.float32).reshape(4)
    rc = _ref_lib().ref_glsl_dispatch(_vp(np.ascontiguousarray(pos)), _vp(np.ascontiguousarray(vel)),
                                      _vp(pw), _vp(vw), ns, dt, scale, _vp(bs))
    if rc != 0:
        raise RuntimeError("ref_glsl_dispatch failed")
    return pw, vw


def ref_tes_available() -> bool:
    return os.path.exists(REF_TES_PATH)


def ref_tes_stream(pos, tangents, faces, random, ninstances=3, nlines=2, nsubsegments=16, scale=1.45):
    """The reference's tessellation evaluation shader compiled as C++
    (oracle/_ref/libref_tes.so), driven like oracle.tess (N = 4 only)."""
    L = C.CDLL(REF_TES_PATH)
    L.ref_tes_stream.restype = C.c_int
    L.ref_tes_stream.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p,
                                 C.c_uint32, C.c_uint32, C.c_uint32, C.c_float, C.c_void_p]
    p = np.ascontiguousarray(pos, dtype=np.float32)
    t = np.ascontiguousarray(tangents, dtype=np.float32)
    f = np.ascontiguousarray(faces, dtype=np.uint32).reshape(-1, 3)
    r = np.ascontiguousarray(random, dtype=np.float32).reshape(-1)
    n = p.shape[1]
    segs = ninstances * f.shape[0] * (n - 1) * nlines * nsubsegments
    out = np.zeros((2 * segs, 4), np.float32)
    rc = L.ref_tes_stream(_vp(p), _vp(t), n, _vp(f), f.shape[0], _vp(r), ninstances, nlines, nsubsegments,
                          float(np.float32(scale)), _vp(out))
    if rc != 0:
        raise ValueError("ref_tes_stream: the reference shader has 4 points per strand")
    return out


# ---- the reference's skinning and Marschner shaders compiled as C++ --------

REF_SKIN_PATH = os.path.join(HERE, "_ref", "libref_skin.so")
REF_MARSCHNER_PATHS = (os.path.join(HERE, "_ref", "libref_marschner_m.so"),
                       os.path.join(HERE, "_ref", "libref_marschner_n.so"))


def ref_skin_available() -> bool:
    return os.path.exists(REF_SKIN_PATH)


def ref_skin(rest_roots, bones, weights, dq):
    """apply_skinning + skinning_DQBS (inc_skinning.glsl) compiled as C++
    (oracle/_ref/libref_skin.so): rest (n, 3), bones (n, 4) uint8, weights
    (n, 3), dq (nbones, 8) -> (n, 3) float32."""
    L = C.CDLL(REF_SKIN_PATH)
    L.ref_skin.restype = C.c_int
    L.ref_skin.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p]
    rest = np.ascontiguousarray(rest_roots, dtype=np.float32).reshape(-1, 3)
    b = np.ascontiguousarray(bones, dtype=np.uint8).reshape(-1, 4)
    w = np.ascontiguousarray(weights, dtype=np.float32).reshape(-1, 3)
    q = np.ascontiguousarray(dq, dtype=np.float32).reshape(-1, 8)
    out = np.zeros_like(rest)
    if L.ref_skin(_vp(rest), _vp(b), _vp(w), rest.shape[0], _vp(q), q.shape[0], _vp(out)) != 0:
        raise ValueError("ref_skin: bone index beyond the palette")
    return out


def ref_marschner_available() -> bool:
    return all(os.path.exists(p) for p in REF_MARSCHNER_PATHS)


def ref_marschner(resolution=128, eta=1.55, absorption=0.2, ar=-5.0, br=5.0):
    """cs_marschner_m.glsl and cs_marschner_n.glsl compiled as C++: the M
    and N tables, (resolution, resolution, 4) float32 each."""
    Lm, Ln = (C.CDLL(p) for p in REF_MARSCHNER_PATHS)
    Lm.ref_marschner_m.argtypes = [C.c_uint32, C.c_float, C.c_float, C.c_void_p]
    Ln.ref_marschner_n.argtypes = [C.c_uint32, C.c_float, C.c_float, C.c_void_p]
    m = np.zeros((resolution, resolution, 4), np.float32)
    n = np.zeros((resolution, resolution, 4), np.float32)
    Lm.ref_marschner_m(resolution, ar, br, _vp(m))
    Ln.ref_marschner_n(resolution, eta, absorption, _vp(n))
    return m, n
