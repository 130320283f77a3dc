"""ctypes mirror of the POD types and constants of include/hairsim.h.

Only data definitions live here (no library is loaded), so both the library
binding (barbu_gb300.hairsim) and the test checker can share them.
"""
from __future__ import annotations

import ctypes as C

HS_MIN_POINTS_PER_STRAND = 2
HS_MAX_POINTS_PER_STRAND = 64
HS_MAX_SPHERES = 32
HS_MAX_BONES = 8
HS_TESS_RANDOM_SIZE = 4096
HS_EXPORT_STRAND_MAJOR = 0
HS_EXPORT_POINT_MAJOR = 1
HS_FIELD_POSITIONS = 0
HS_FIELD_VELOCITIES = 1
HS_LUT_HALF4 = 0
HS_LUT_FLOAT4 = 1
HS_MAX_SUBSTEPS = 64
HS_MAX_ITERATIONS = 64
HS_NOALLOC_MAX_GROOMS = 256

# hs_status
HS_OK = 0
HS_ERR_INVALID_ARG = 1
HS_ERR_OUT_OF_MEMORY = 2
HS_ERR_ADMISSION_DENIED = 3
HS_ERR_CUDA = 4
HS_ERR_TIMEOUT = 5
HS_ERR_NOT_INITIALIZED = 6
HS_ERR_UNSUPPORTED = 7

STATUS_NAMES = {
    HS_OK: "HS_OK",
    HS_ERR_INVALID_ARG: "HS_ERR_INVALID_ARG",
    HS_ERR_OUT_OF_MEMORY: "HS_ERR_OUT_OF_MEMORY",
    HS_ERR_ADMISSION_DENIED: "HS_ERR_ADMISSION_DENIED",
    HS_ERR_CUDA: "HS_ERR_CUDA",
    HS_ERR_TIMEOUT: "HS_ERR_TIMEOUT",
    HS_ERR_NOT_INITIALIZED: "HS_ERR_NOT_INITIALIZED",
    HS_ERR_UNSUPPORTED: "HS_ERR_UNSUPPORTED",
}

# hs_mode
HS_MODE_REFERENCE = 0
HS_MODE_DFTL = 1

# hs_root_mode
HS_ROOT_PINNED = 0
HS_ROOT_RIGID = 1
HS_ROOT_EXPLICIT = 2
HS_ROOT_SKINNED = 3

# hs_variant
HS_VARIANT_REGISTERS = 0
HS_VARIANT_REGISTERS_SHARED = 1
HS_VARIANT_STREAM = 2
HS_VARIANT_STREAM_TMEM = 6  # 3-5 are not built
HS_VARIANT_LANES = 7

HS_CONTRACT_EXACT = 0
HS_CONTRACT_FAST = 1

HS_MAPPING_AUTO = 0
HS_MAPPING_THREAD = 1
HS_MAPPING_LANES = 2

# hs_length_rule
HS_LENGTH_REFERENCE = 0
HS_LENGTH_TOTAL = 1


class StrandParams(C.Structure):
    _fields_ = [
        ("points_per_strand", C.c_uint32),
        ("length_rule", C.c_uint32),
        ("max_length", C.c_float),
        ("length_jitter", C.c_float),
        ("seed", C.c_uint64),
        ("lengths", C.POINTER(C.c_float)),
        ("strand_base", C.c_uint32),
        ("keep_order", C.c_uint32),
    ]


class SimParams(C.Structure):
    _fields_ = [
        ("mode", C.c_uint32),
        ("substeps", C.c_uint32),
        ("iterations", C.c_uint32),
        ("root_mode", C.c_uint32),
        ("gravity", C.c_float * 3),
        ("gravity_scale", C.c_float),
        ("damping", C.c_float),
        ("length_scale", C.c_float),
        ("wind_jitter", C.c_float),
        ("contract", C.c_uint32),
    ]


class TessParams(C.Structure):
    _fields_ = [
        ("ninstances", C.c_uint32),
        ("nlines", C.c_uint32),
        ("nsubsegments", C.c_uint32),
        ("length_scale", C.c_float),
    ]


class TuneEntry(C.Structure):
    _fields_ = [
        ("capacity", C.c_uint32),
        ("mode", C.c_uint32),
        ("tiles_log2", C.c_uint32),
        ("variant", C.c_uint32),
        ("warps_per_block", C.c_uint32),
        ("waves", C.c_uint32),
        ("ms", C.c_float),
        ("contract", C.c_uint32),
    ]


class FrameStats(C.Structure):
    _fields_ = [
        ("bounds_min", C.c_float * 3),
        ("bounds_max", C.c_float * 3),
        ("max_speed", C.c_float),
        ("valid", C.c_uint32),
        ("kinetic_energy", C.c_double),
    ]


class MarschnerParams(C.Structure):
    _fields_ = [
        ("eta", C.c_float),
        ("absorption", C.c_float),
        ("eccentricity", C.c_float),
        ("ar", C.c_float),
        ("br", C.c_float),
        ("glint_scale", C.c_float),
        ("azimuthal_width", C.c_float),
        ("delta_caustic", C.c_float),
        ("delta_hm", C.c_float),
        ("resolution", C.c_uint32),
    ]


class Layout(C.Structure):
    _fields_ = [
        ("nstrands", C.c_uint32),
        ("points_per_strand", C.c_uint32),
        ("strand_stride", C.c_uint32),
        ("reserved", C.c_uint32),
    ]


# hs_request_state
HS_REQ_QUEUED = 0
HS_REQ_RESIDENT = 1
HS_REQ_DONE = 2
HS_REQ_GONE = 3


class ServerConfig(C.Structure):
    _fields_ = [
        ("budget_bytes", C.c_uint64),
        ("max_grooms", C.c_uint32),
        ("reserved", C.c_uint32),
    ]


class Request(C.Structure):
    _fields_ = [
        ("root_pos", C.POINTER(C.c_float)),
        ("root_nrm", C.POINTER(C.c_float)),
        ("lengths", C.POINTER(C.c_float)),
        ("nstrands", C.c_uint32),
        ("frames", C.c_uint32),
        ("strand", StrandParams),
        ("sim", SimParams),
        ("spheres", C.POINTER(C.c_float)),
        ("nspheres", C.c_uint32),
        ("keep_result", C.c_uint32),
        ("wind", C.c_float * 3),
        ("swing_amp", C.c_float),
        ("swing_omega", C.c_float),
        ("reserved", C.c_uint32),
        ("skin_bones", C.POINTER(C.c_uint8)),
        ("skin_weights", C.POINTER(C.c_float)),
    ]


class TickStats(C.Structure):
    _fields_ = [
        ("advanced", C.c_uint32),
        ("queued", C.c_uint32),
        ("admitted", C.c_uint32),
        ("retired", C.c_uint32),
        ("resident_bytes", C.c_uint64),
        ("point_substeps", C.c_uint64),
        ("tick_ms", C.c_double),
    ]


def groom_state_bytes(nstrands: int, npoints: int) -> int:
    """Device bytes of one groom's state: positions, velocities, rest roots
    and the frame statistics (32 B per 32-strand tile)."""
    stride = (nstrands + 31) // 32 * 32
    return 16 * stride * (2 * npoints + 1) + 32 * (stride // 32)


def sim_params_reference(length_scale: float = 1.0) -> SimParams:
    """The constants cs_simulation.glsl hard-codes (:71-72, :100-102, :197)."""
    p = SimParams()
    p.mode = HS_MODE_REFERENCE
    p.substeps = 1
    p.iterations = 8
    p.root_mode = HS_ROOT_PINNED
    p.gravity[:] = (0.0, -9.81, 0.0)
    p.gravity_scale = 20.0
    p.damping = 0.80
    p.length_scale = length_scale
    p.wind_jitter = 0.0
    return p


def sim_params_dftl(substeps: int = 4, damping: float = 0.9, wind_jitter: float = 0.0,
                    root_mode: int = HS_ROOT_PINNED, iterations: int = 1,
                    contract: int = 0) -> SimParams:
    p = SimParams()
    p.mode = HS_MODE_DFTL
    p.contract = contract
    p.substeps = substeps
    p.iterations = iterations
    p.root_mode = root_mode
    p.gravity[:] = (0.0, -9.81, 0.0)
    p.gravity_scale = 1.0
    p.damping = damping
    p.length_scale = 1.0
    p.wind_jitter = wind_jitter
    return p


def strand_params(n: int, length_rule: int = HS_LENGTH_REFERENCE, max_length: float = 0.5,
                  length_jitter: float = 0.1, seed: int = 0, strand_base: int = 0,
                  keep_order: bool = False) -> StrandParams:
    p = StrandParams()
    p.points_per_strand = n
    p.length_rule = length_rule
    p.max_length = max_length
    p.length_jitter = length_jitter
    p.seed = seed
    p.lengths = None
    p.strand_base = strand_base
    p.keep_order = 1 if keep_order else 0
    return p
