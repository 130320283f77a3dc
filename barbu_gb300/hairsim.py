"""Python binding of the C-ABI in include/hairsim.h (libhairsim.so).

`Hair` mirrors the reference's host class (src/fx/hair.h:24-121): init,
setup, update, set_bounding_sphere, initialized, deinit, plus readback of the
control-point buffer the renderer consumes. `Context` and `Groom` expose the
rest of the C-ABI (many spheres, wind, root transforms, batched updates).

The library is the only compute path: if libhairsim.so is missing this
module raises on first use; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libhairsim.so")

_lib = None


class HairSimError(RuntimeError):
    def __init__(self, status: int, where: str, message: str):
        self.status = status
        super().__init__(f"{where}: {abi.STATUS_NAMES.get(status, status)}: {message}")


def _declare(L):
    vp, u32, u64, f32, sz = C.c_void_p, C.c_uint32, C.c_uint64, C.c_float, C.c_size_t
    st = C.c_int
    sig = {
        "hs_create": (st, [C.POINTER(vp)]),
        "hs_destroy": (st, [vp]),
        "hs_ctx_stream": (st, [vp, C.POINTER(vp)]),
        "hs_sync": (st, [vp]),
        "hs_ctx_launch_count": (st, [vp, C.POINTER(u64)]),
        "hs_groom_init": (st, [vp, vp, vp, u32, C.POINTER(abi.StrandParams), C.POINTER(abi.SimParams), C.POINTER(vp)]),
        "hs_groom_init_from_state": (st, [vp, vp, vp, u32, u32, u64, C.POINTER(abi.SimParams), C.POINTER(vp)]),
        "hs_groom_destroy": (st, [vp]),
        "hs_groom_set_params": (st, [vp, C.POINTER(abi.SimParams)]),
        "hs_groom_info": (st, [vp, C.POINTER(u32), C.POINTER(u32)]),
        "hs_set_bounding_sphere": (st, [vp, vp]),
        "hs_set_spheres": (st, [vp, vp, u32]),
        "hs_set_wind": (st, [vp, vp]),
        "hs_set_root_transform": (st, [vp, vp]),
        "hs_set_roots": (st, [vp, vp, u32]),
        "hs_set_root_transforms": (st, [C.POINTER(vp), u32, vp]),
        "hs_update": (st, [vp, f32]),
        "hs_update_many": (st, [vp, C.POINTER(vp), u32, f32]),
        "hs_update_many_noalloc": (st, [vp, C.POINTER(vp), u32, f32]),
        "hs_set_skin": (st, [vp, vp, vp, u32]),
        "hs_tess_params_reference": (None, [C.POINTER(abi.TessParams)]),
        "hs_tess_setup": (st, [vp, vp, u32, vp, vp, u32]),
        "hs_tess_count": (st, [vp, C.POINTER(abi.TessParams), C.POINTER(u64)]),
        "hs_tess_stream": (st, [vp, C.POINTER(abi.TessParams), C.POINTER(u64)]),
        "hs_tess_device": (st, [vp, C.POINTER(vp), C.POINTER(u64)]),
        "hs_tess_readback": (st, [vp, vp, sz]),
        "hs_export": (st, [vp, u32, u32, vp, sz]),
        "hs_groom_stats": (st, [vp, C.POINTER(abi.FrameStats)]),
        "hs_marschner_params_reference": (None, [C.POINTER(abi.MarschnerParams)]),
        "hs_marschner_luts": (st, [vp, C.POINTER(abi.MarschnerParams), u32, vp, vp]),
        "hs_set_bone_dual_quats": (st, [vp, vp, u32]),
        "hs_set_bone_matrices": (st, [vp, vp, u32]),
        "hs_autotune": (st, [vp, C.POINTER(vp), u32, f32, C.POINTER(u32)]),
        "hs_tune_override": (st, [vp, u32, u32, u32, u32, u32]),
        "hs_tune_entries": (st, [vp, C.POINTER(abi.TuneEntry), u32, C.POINTER(u32)]),
        "hs_readback": (st, [vp, vp, sz]),
        "hs_readback_velocities": (st, [vp, vp, sz]),
        "hs_readback_async": (st, [vp, vp, sz]),
        "hs_readback_xyz": (st, [vp, vp, sz]),
        "hs_readback_xyz_async": (st, [vp, vp, sz]),
        "hs_readback_wait": (st, [vp]),
        "hs_readback_many_async": (st, [vp, C.POINTER(vp), u32, u32, vp, sz]),
        "hs_readback_drain": (st, [vp, u32]),
        "hs_device_positions": (st, [vp, C.POINTER(vp), C.POINTER(abi.Layout)]),
        "hs_groom_strand_order": (st, [vp, C.POINTER(C.c_uint32), C.c_uint32, C.POINTER(C.c_uint32)]),
        "hs_groom_set_mapping": (st, [vp, C.c_uint32]),
        "hs_groom_mapping": (st, [vp, C.POINTER(C.c_uint32)]),
        "hs_sim_params_reference": (None, [C.POINTER(abi.SimParams)]),
        "hs_sim_params_dftl": (None, [C.POINTER(abi.SimParams)]),
        "hs_strand_params_reference": (None, [C.POINTER(abi.StrandParams)]),
        "hs_last_error_string": (C.c_char_p, []),
        "hs_server_create": (st, [vp, C.POINTER(abi.ServerConfig), C.POINTER(vp)]),
        "hs_server_destroy": (st, [vp]),
        "hs_server_submit": (st, [vp, C.POINTER(abi.Request), C.POINTER(u64)]),
        "hs_server_tick": (st, [vp, f32, C.POINTER(abi.TickStats)]),
        "hs_server_poll": (st, [vp, u64, C.POINTER(u32), C.POINTER(u32)]),
        "hs_server_set_spheres": (st, [vp, u64, vp, u32]),
        "hs_server_set_root_transform": (st, [vp, u64, vp]),
        "hs_server_set_bone_matrices": (st, [vp, u64, vp, u32]),
        "hs_server_collect": (st, [vp, u64, vp, vp, sz]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args


def lib():
    """Loads libhairsim.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -m barbu_gb300.build` "
                              "(the library has no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        _declare(L)
        _lib = L
    return _lib


def marschner_params_reference() -> abi.MarschnerParams:
    p = abi.MarschnerParams()
    lib().hs_marschner_params_reference(C.byref(p))
    return p


def tess_params_reference() -> abi.TessParams:
    p = abi.TessParams()
    lib().hs_tess_params_reference(C.byref(p))
    return p


def last_error() -> str:
    return lib().hs_last_error_string().decode()


def check(status: int, where: str):
    if status != abi.HS_OK:
        raise HairSimError(status, where, last_error())


_F32 = np.dtype(np.float32)


def _f32(a, n=None):
    if not (a.__class__ is np.ndarray and a.dtype is _F32 and a.flags.c_contiguous):
        a = np.ascontiguousarray(a, dtype=np.float32)
    if n is not None and a.size != n:
        raise ValueError(f"expected {n} floats, got {a.size}")
    return a


def _ptr(a):
    """The address of an array's data, for a c_void_p argument. It keeps
    no reference: the caller holds `a` in a local for the duration of the
    call (the per-frame setters run in microseconds, and a ctypes pointer
    object cost more than the library call)."""
    return a.ctypes.data


class Context:
    """hs_ctx: one CUDA stream on the current device."""

    def __init__(self):
        h = C.c_void_p()
        check(lib().hs_create(C.byref(h)), "hs_create")
        self.h = h

    def close(self):
        if self.h:
            check(lib().hs_destroy(self.h), "hs_destroy")
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        s = C.c_void_p()
        check(lib().hs_ctx_stream(self.h, C.byref(s)), "hs_ctx_stream")
        return s.value or 0

    def sync(self):
        check(lib().hs_sync(self.h), "hs_sync")

    def readback_wait(self):
        """Waits for every asynchronous readback of this context."""
        check(lib().hs_readback_wait(self.h), "hs_readback_wait")

    def readback_drain(self, keep: int):
        """hs_readback_drain: waits until at most `keep` asynchronous
        readbacks of this context are in flight, the oldest first."""
        check(lib().hs_readback_drain(self.h, keep), "hs_readback_drain")

    def readback_many_async(self, grooms, out: np.ndarray, comps: int = 3, handles=None) -> np.ndarray:
        """hs_readback_many_async: every groom's strand-major positions, comps
        floats a point, one after the other in `out` (pinned float32, at
        least comps * sum(nstrands * npoints) floats), filled once
        readback_wait or readback_drain has returned for it."""
        if out.dtype != np.float32 or not out.flags.c_contiguous:
            raise ValueError("readback_many_async: out must be a C-contiguous float32 array")
        h = handles if handles is not None else self._handles(grooms)
        check(lib().hs_readback_many_async(self.h, h, len(grooms), comps, out.ctypes.data_as(C.c_void_p), out.size),
              "hs_readback_many_async")
        return out

    def launch_count(self) -> int:
        n = C.c_uint64()
        check(lib().hs_ctx_launch_count(self.h, C.byref(n)), "hs_ctx_launch_count")
        return n.value

    def groom(self, roots, normals, strand: abi.StrandParams, sim: abi.SimParams, lengths=None) -> "Groom":
        roots = _f32(roots).reshape(-1, 3)
        normals = _f32(normals, roots.size).reshape(-1, 3)
        h = C.c_void_p()
        keep = None
        if lengths is not None:
            keep = _f32(lengths, roots.shape[0])
            strand.lengths = keep.ctypes.data_as(C.POINTER(C.c_float))
        try:
            check(lib().hs_groom_init(self.h, _ptr(roots), _ptr(normals), roots.shape[0], C.byref(strand),
                                      C.byref(sim), C.byref(h)), "hs_groom_init")
        finally:
            if keep is not None:
                strand.lengths = None
        return Groom(self, h)

    def _handles(self, grooms):
        arr = (C.c_void_p * len(grooms))(*[g.h for g in grooms])
        return arr

    def update_many(self, grooms, dt: float, handles=None):
        """hs_update_many: one frame for every groom of the list. `handles`
        (from handles_of) skips rebuilding the pointer array each frame."""
        h = handles if handles is not None else self._handles(grooms)
        check(lib().hs_update_many(self.h, h, len(grooms), dt), "hs_update_many")

    def update_many_noalloc(self, grooms, dt: float, handles=None):
        """hs_update_many_noalloc: hs_update_many without any allocation, its
        scratch in a fixed device array (at most abi.HS_NOALLOC_MAX_GROOMS
        grooms per call; calls overlapping on the GPU race on that array)."""
        h = handles if handles is not None else self._handles(grooms)
        check(lib().hs_update_many_noalloc(self.h, h, len(grooms), dt), "hs_update_many_noalloc")

    def handles_of(self, grooms):
        return self._handles(grooms)

    def set_root_transforms(self, grooms, m, handles=None):
        """hs_set_root_transforms: one 4x4 column-major matrix per groom."""
        a = _f32(m, 16 * len(grooms))
        h = handles if handles is not None else self._handles(grooms)
        check(lib().hs_set_root_transforms(h, len(grooms), _ptr(a)), "hs_set_root_transforms")

    def marschner_luts(self, params: "abi.MarschnerParams", fmt: int, d_m: int, d_n: int):
        """hs_marschner_luts into device buffers d_m, d_n (0 to skip one)."""
        check(lib().hs_marschner_luts(self.h, C.byref(params), fmt, C.c_void_p(d_m or None),
                                      C.c_void_p(d_n or None)), "hs_marschner_luts")

    def tune_entries(self) -> list[dict]:
        """hs_tune_entries: the autotuner's chosen shapes, one per bucket class."""
        n = C.c_uint32()
        check(lib().hs_tune_entries(self.h, None, 0, C.byref(n)), "hs_tune_entries")
        arr = (abi.TuneEntry * max(1, n.value))()
        check(lib().hs_tune_entries(self.h, arr, n.value, C.byref(n)), "hs_tune_entries")
        return [{f: getattr(arr[k], f) for f, _ in abi.TuneEntry._fields_ if f != "reserved"} for k in range(n.value)]

    def autotune(self, grooms, dt: float) -> int:
        """hs_autotune: returns the number of launch shapes tried."""
        n = C.c_uint32()
        check(lib().hs_autotune(self.h, self._handles(grooms), len(grooms), dt, C.byref(n)), "hs_autotune")
        return n.value

    def tune_override(self, points: int, mode: int, variant: int, warps_per_block: int = 4, waves: int = 1):
        """hs_tune_override: pins the batched launch shape for (points, mode)."""
        check(lib().hs_tune_override(self.h, points, mode, variant, warps_per_block, waves), "hs_tune_override")

    def groom_from_state(self, pos, vel, sim: abi.SimParams, seed: int = 0) -> "Groom":
        pos = _f32(pos)
        vel = _f32(vel, pos.size)
        ns, n, four = pos.shape
        assert four == 4
        h = C.c_void_p()
        check(lib().hs_groom_init_from_state(self.h, _ptr(pos), _ptr(vel), ns, n, seed, C.byref(sim), C.byref(h)),
              "hs_groom_init_from_state")
        return Groom(self, h)


class Groom:
    """hs_groom: one set of strands resident on the device."""

    def __init__(self, ctx: Context, h):
        self.ctx = ctx
        self.h = h
        ns, n = C.c_uint32(), C.c_uint32()
        check(lib().hs_groom_info(self.h, C.byref(ns), C.byref(n)), "hs_groom_info")
        self.nstrands, self.npoints = ns.value, n.value

    def destroy(self):
        if self.h and self.ctx.h:
            check(lib().hs_groom_destroy(self.h), "hs_groom_destroy")
        self.h = None

    def set_params(self, sim: abi.SimParams):
        check(lib().hs_groom_set_params(self.h, C.byref(sim)), "hs_groom_set_params")

    def set_bounding_sphere(self, xyzr):
        a = _f32(xyzr, 4)
        check(lib().hs_set_bounding_sphere(self.h, _ptr(a)), "hs_set_bounding_sphere")

    def set_spheres(self, xyzr):
        a = _f32(xyzr).reshape(-1, 4)
        check(lib().hs_set_spheres(self.h, _ptr(a), a.shape[0]), "hs_set_spheres")

    def set_wind(self, w):
        a = _f32(w, 3)
        check(lib().hs_set_wind(self.h, _ptr(a)), "hs_set_wind")

    def set_root_transform(self, m):
        a = _f32(m, 16)
        check(lib().hs_set_root_transform(self.h, _ptr(a)), "hs_set_root_transform")

    def set_roots(self, xyz):
        a = _f32(xyz, 3 * self.nstrands)
        check(lib().hs_set_roots(self.h, _ptr(a), self.nstrands), "hs_set_roots")

    def set_skin(self, bones, weights):
        """hs_set_skin: 4 bone indices (uint8) and the first 3 weights per
        strand; the 4th weight is 1 - (w0 + w1 + w2)."""
        b = np.ascontiguousarray(bones, dtype=np.uint8)
        if b.size != 4 * self.nstrands:
            raise ValueError(f"expected {4 * self.nstrands} bone indices, got {b.size}")
        w = _f32(weights, 3 * self.nstrands)
        check(lib().hs_set_skin(self.h, _ptr(b), _ptr(w), self.nstrands), "hs_set_skin")

    def set_bone_dual_quats(self, dq):
        """hs_set_bone_dual_quats: (nbones, 8) real xyzw then dual xyzw."""
        a = _f32(dq).reshape(-1, 8)
        check(lib().hs_set_bone_dual_quats(self.h, _ptr(a), a.shape[0]), "hs_set_bone_dual_quats")

    def set_bone_matrices(self, m):
        """hs_set_bone_matrices: (nbones, 16) rigid column-major skinning matrices."""
        a = _f32(m).reshape(-1, 16)
        check(lib().hs_set_bone_matrices(self.h, _ptr(a), a.shape[0]), "hs_set_bone_matrices")

    def stats(self) -> dict | None:
        """hs_groom_stats: bounds, kinetic energy and largest speed of the
        last frame (None before the first update)."""
        st = abi.FrameStats()
        check(lib().hs_groom_stats(self.h, C.byref(st)), "hs_groom_stats")
        if not st.valid:
            return None
        return {"bounds_min": list(st.bounds_min), "bounds_max": list(st.bounds_max),
                "kinetic_energy": st.kinetic_energy, "max_speed": st.max_speed}

    def export(self, d_ptr: int, capacity_floats: int, layout: int = abi.HS_EXPORT_STRAND_MAJOR,
               field: int = abi.HS_FIELD_POSITIONS):
        """hs_export: device-to-device copy of positions or velocities into
        the device buffer at d_ptr (asynchronous on the context stream)."""
        check(lib().hs_export(self.h, field, layout, C.c_void_p(d_ptr), capacity_floats), "hs_export")

    def tess_setup(self, faces, tangents, random):
        """hs_tess_setup: triangles (nf, 3) of strand indices, tangents
        (nstrands, N, 4), random buffer (HS_TESS_RANDOM_SIZE floats)."""
        f = np.ascontiguousarray(faces, dtype=np.uint32).reshape(-1, 3)
        t = _f32(tangents, 4 * self.nstrands * self.npoints)
        r = _f32(random).reshape(-1)
        check(lib().hs_tess_setup(self.h, _ptr(f), f.shape[0], _ptr(t), _ptr(r), r.size), "hs_tess_setup")

    def tess_stream(self, params=None) -> int:
        """hs_tess_stream: returns the number of vertices written."""
        p = params if params is not None else tess_params_reference()
        n = C.c_uint64()
        check(lib().hs_tess_stream(self.h, C.byref(p), C.byref(n)), "hs_tess_stream")
        return n.value

    def tess_readback(self) -> np.ndarray:
        """The last pass's vertices, (count, 4): x, y, z, relative position."""
        d, n = C.c_void_p(), C.c_uint64()
        check(lib().hs_tess_device(self.h, C.byref(d), C.byref(n)), "hs_tess_device")
        out = np.empty((n.value, 4), np.float32)
        check(lib().hs_tess_readback(self.h, out.ctypes.data_as(C.c_void_p), out.size), "hs_tess_readback")
        return out

    def update(self, dt: float):
        check(lib().hs_update(self.h, dt), "hs_update")

    def readback(self, out=None) -> np.ndarray:
        """Positions (x, y, z, restlength), shape (nstrands, npoints, 4)."""
        if out is None:
            out = np.empty((self.nstrands, self.npoints, 4), np.float32)
        check(lib().hs_readback(self.h, out.ctypes.data_as(C.c_void_p), out.size), "hs_readback")
        return out

    def readback_async(self, out: np.ndarray) -> np.ndarray:
        """Queues a copy of the positions into `out` (pinned float32 memory of
        shape (nstrands, npoints, 4)); `out` holds them after
        Context.readback_wait()."""
        if out.dtype != np.float32 or not out.flags.c_contiguous:
            raise ValueError("readback_async: out must be a C-contiguous float32 array")
        check(lib().hs_readback_async(self.h, out.ctypes.data_as(C.c_void_p), out.size), "hs_readback_async")
        return out

    def readback_xyz(self, out=None) -> np.ndarray:
        """Positions without the rest lengths, shape (nstrands, npoints, 3)."""
        if out is None:
            out = np.empty((self.nstrands, self.npoints, 3), np.float32)
        check(lib().hs_readback_xyz(self.h, out.ctypes.data_as(C.c_void_p), out.size), "hs_readback_xyz")
        return out

    def readback_xyz_async(self, out: np.ndarray) -> np.ndarray:
        """readback_async of (x, y, z) only: `out` pinned float32 of shape
        (nstrands, npoints, 3), filled once Context.readback_wait() returns."""
        if out.dtype != np.float32 or not out.flags.c_contiguous:
            raise ValueError("readback_xyz_async: out must be a C-contiguous float32 array")
        check(lib().hs_readback_xyz_async(self.h, out.ctypes.data_as(C.c_void_p), out.size),
              "hs_readback_xyz_async")
        return out

    def readback_velocities(self, out=None) -> np.ndarray:
        if out is None:
            out = np.empty((self.nstrands, self.npoints, 4), np.float32)
        check(lib().hs_readback_velocities(self.h, out.ctypes.data_as(C.c_void_p), out.size),
              "hs_readback_velocities")
        return out

    def device_positions(self):
        p = C.c_void_p()
        lay = abi.Layout()
        check(lib().hs_device_positions(self.h, C.byref(p), C.byref(lay)), "hs_device_positions")
        return p.value, lay

    def set_mapping(self, mapping: int):
        """hs_groom_set_mapping: HS_MAPPING_AUTO, _THREAD or _LANES."""
        check(lib().hs_groom_set_mapping(self.h, mapping), "hs_groom_set_mapping")

    def mapping(self) -> int:
        """The mapping the next update takes (HS_MAPPING_THREAD or _LANES)."""
        m = C.c_uint32()
        check(lib().hs_groom_mapping(self.h, C.byref(m)), "hs_groom_mapping")
        return m.value

    def strand_order(self) -> np.ndarray:
        """order[j] = the caller's index of stored strand j (column j of
        device_positions)."""
        out = np.empty(self.nstrands, np.uint32)
        n = C.c_uint32()
        check(lib().hs_groom_strand_order(self.h, out.ctypes.data_as(C.POINTER(C.c_uint32)), out.size,
                                          C.byref(n)), "hs_groom_strand_order")
        return out


class Hair:
    """The reference's Hair class (src/fx/hair.h:24-121) over the C-ABI.

    init()                 -> a context (src/fx/hair.cc:26-40)
    setup(roots, normals)  -> hs_groom_init (src/fx/hair.cc:42-64); the
                              reference reads roots and normals from the
                              scalp mesh, here the caller passes them
    update(dt)             -> hs_update (src/fx/hair.cc:89-125)
    set_bounding_sphere(v) -> hs_set_bounding_sphere (src/fx/hair.h:72-74)
    initialized()          -> nroots != 0 (src/fx/hair.h:76-78)
    deinit()               -> release everything (src/fx/hair.cc:66-87)
    The reference's UI parameters keep their defaults: maxlength 0.5,
    lengthScale 1.45 (src/fx/hair.h:27-51), which the update passes as
    uScaleFactor (src/fx/hair.cc:108).
    """

    def __init__(self, max_length: float = 0.5, length_scale: float = 1.45, seed: int = 0):
        self.max_length = max_length
        self.length_scale = length_scale
        self.seed = seed
        self.ctx = None
        self.groom = None
        self.nroots = 0
        self._bsphere = np.array([0.0, 0.0, 0.0, 1.0], np.float32)  # uBoundingSphere default (:43)

    def init(self):
        self.ctx = Context()

    def deinit(self):
        if self.groom is not None:
            self.groom.destroy()
            self.groom = None
        if self.ctx is not None:
            self.ctx.close()
            self.ctx = None
        self.nroots = 0

    def setup(self, roots, normals):
        if self.ctx is None:
            raise HairSimError(abi.HS_ERR_NOT_INITIALIZED, "Hair.setup", "call init() first")
        sp = abi.strand_params(4, abi.HS_LENGTH_REFERENCE, self.max_length, 0.1, self.seed)
        sim = abi.sim_params_reference(self.length_scale)
        self.groom = self.ctx.groom(roots, normals, sp, sim)
        self.nroots = self.groom.nstrands

    def initialized(self) -> bool:
        return self.nroots != 0

    def set_bounding_sphere(self, xyzr):
        self._bsphere = np.asarray(xyzr, np.float32).reshape(4).copy()

    def update(self, dt: float):
        if not self.initialized():
            return  # the reference logs and returns (src/fx/hair.cc:90-93)
        self.groom.set_bounding_sphere(self._bsphere)
        self.groom.update(dt)

    def readback(self) -> np.ndarray:
        return self.groom.readback()


class Server:
    """hs_server: a served stream of grooms over one context."""

    def __init__(self, ctx: Context, budget_bytes: int, max_grooms: int = 0):
        cfg = abi.ServerConfig()
        cfg.budget_bytes = budget_bytes
        cfg.max_grooms = max_grooms
        h = C.c_void_p()
        check(lib().hs_server_create(ctx.h, C.byref(cfg), C.byref(h)), "hs_server_create")
        self.ctx = ctx
        self.h = h
        self._shapes = {}

    def close(self):
        if self.h:
            check(lib().hs_server_destroy(self.h), "hs_server_destroy")
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, roots, normals, strand: abi.StrandParams, sim: abi.SimParams, frames: int, spheres=None,
               wind=(0.0, 0.0, 0.0), swing_amp: float = 0.0, swing_omega: float = 0.0, keep: bool = False,
               lengths=None, skin_bones=None, skin_weights=None) -> int:
        roots = _f32(roots).reshape(-1, 3)
        normals = _f32(normals, roots.size).reshape(-1, 3)
        q = abi.Request()
        q.root_pos = roots.ctypes.data_as(C.POINTER(C.c_float))
        q.root_nrm = normals.ctypes.data_as(C.POINTER(C.c_float))
        keep_len = None
        if lengths is not None:
            keep_len = _f32(lengths, roots.shape[0])
            q.lengths = keep_len.ctypes.data_as(C.POINTER(C.c_float))
        q.nstrands = roots.shape[0]
        q.frames = frames
        q.strand = strand
        q.sim = sim
        sph = None
        if spheres is not None and len(spheres):
            sph = _f32(spheres).reshape(-1, 4)
            q.spheres = sph.ctypes.data_as(C.POINTER(C.c_float))
            q.nspheres = sph.shape[0]
        q.keep_result = 1 if keep else 0
        q.wind[:] = tuple(float(w) for w in wind)
        q.swing_amp = swing_amp
        q.swing_omega = swing_omega
        keep_skin = None
        if skin_bones is not None:
            keep_skin = (np.ascontiguousarray(skin_bones, dtype=np.uint8).reshape(-1, 4),
                         _f32(skin_weights, 3 * roots.shape[0]))
            q.skin_bones = keep_skin[0].ctypes.data_as(C.POINTER(C.c_uint8))
            q.skin_weights = keep_skin[1].ctypes.data_as(C.POINTER(C.c_float))
        t = C.c_uint64()
        check(lib().hs_server_submit(self.h, C.byref(q), C.byref(t)), "hs_server_submit")
        self._shapes[t.value] = (roots.shape[0], int(strand.points_per_strand))
        return t.value

    def set_spheres(self, ticket: int, xyzr):
        """hs_server_set_spheres: the groom's spheres from its next frame."""
        a = _f32(xyzr).reshape(-1, 4)
        check(lib().hs_server_set_spheres(self.h, ticket, _ptr(a), a.shape[0]), "hs_server_set_spheres")

    def set_root_transform(self, ticket: int, m):
        a = _f32(m, 16)
        check(lib().hs_server_set_root_transform(self.h, ticket, _ptr(a)), "hs_server_set_root_transform")

    def set_bone_matrices(self, ticket: int, m):
        a = _f32(m).reshape(-1, 16)
        check(lib().hs_server_set_bone_matrices(self.h, ticket, _ptr(a), a.shape[0]), "hs_server_set_bone_matrices")

    def tick(self, dt: float) -> abi.TickStats:
        st = abi.TickStats()
        check(lib().hs_server_tick(self.h, dt, C.byref(st)), "hs_server_tick")
        return st

    def poll(self, ticket: int):
        state, frames = C.c_uint32(), C.c_uint32()
        check(lib().hs_server_poll(self.h, ticket, C.byref(state), C.byref(frames)), "hs_server_poll")
        return state.value, frames.value

    def collect(self, ticket: int):
        ns, n = self._shapes[ticket]
        pos = np.empty((ns, n, 4), np.float32)
        vel = np.empty((ns, n, 4), np.float32)
        check(lib().hs_server_collect(self.h, ticket, pos.ctypes.data_as(C.c_void_p), vel.ctypes.data_as(C.c_void_p),
                                      pos.size), "hs_server_collect")
        return pos, vel
