"""The C-ABI boundary on the CPU: the library builds, loads, exports every
symbol include/*.h declares, and reports errors instead of crashing. No
kernel runs here."""
from __future__ import annotations

import ctypes as C
import glob
import os
import re
import subprocess

import pytest

from barbu_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols() -> list[str]:
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h, encoding="utf-8").read()
        names += re.findall(r"HS_API\s+[\w\s\*]+?\b(hs_\w+)\s*\(", text)
    return sorted(set(names))


def test_header_declares_the_reference_interface():
    names = declared_symbols()
    for required in ("hs_create", "hs_destroy", "hs_groom_init", "hs_update", "hs_set_bounding_sphere",
                     "hs_readback", "hs_device_positions", "hs_groom_destroy"):
        assert required in names


def test_library_exports_every_declared_symbol(built_library):
    L = C.CDLL(built_library)
    for name in declared_symbols():
        assert hasattr(L, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", built_library], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\b(hs_\w+)\b", out))
    assert set(declared_symbols()) <= exported
    # Nothing else of ours leaks out of the library.
    assert exported == set(declared_symbols()), sorted(exported - set(declared_symbols()))


def test_python_binding_declares_every_entry_point():
    """barbu_gb300/hairsim.py gives every C-ABI entry point a ctypes
    signature (no call goes through ctypes' default int conversion)."""
    src = open(os.path.join(ROOT, "barbu_gb300", "hairsim.py"), encoding="utf-8").read()
    bound = set(re.findall(r'"(hs_\w+)":', src))
    assert bound == set(declared_symbols()), (sorted(set(declared_symbols()) - bound), sorted(bound - set(declared_symbols())))


def test_parameter_presets_match_reference_constants(built_library):
    from barbu_gb300 import hairsim
    L = hairsim.lib()
    p = abi.SimParams()
    L.hs_sim_params_reference(C.byref(p))
    assert (p.mode, p.substeps, p.iterations) == (abi.HS_MODE_REFERENCE, 1, 8)
    assert p.gravity_scale == 20.0 and abs(p.damping - 0.8) < 1e-7
    assert p.gravity[0] == 0.0 and abs(p.gravity[1] + 9.81) < 1e-6 and p.gravity[2] == 0.0
    s = abi.StrandParams()
    L.hs_strand_params_reference(C.byref(s))
    assert s.points_per_strand == 4 and abs(s.max_length - 0.5) < 1e-7 and abs(s.length_jitter - 0.1) < 1e-7
    q = abi.SimParams()
    L.hs_sim_params_dftl(C.byref(q))
    assert q.mode == abi.HS_MODE_DFTL and q.substeps == 4 and abs(q.damping - 0.9) < 1e-7


def test_ctypes_structs_match_header_sizes():
    assert C.sizeof(abi.SimParams) == 48
    assert C.sizeof(abi.StrandParams) == 40
    assert C.sizeof(abi.Layout) == 16


def _gpu_visible() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_gpu_visible(), reason="checks the no-GPU error path")
def test_create_without_gpu_reports_error(built_library):
    from barbu_gb300 import hairsim
    with pytest.raises(hairsim.HairSimError) as e:
        hairsim.Context()
    assert e.value.status == abi.HS_ERR_CUDA
    assert hairsim.last_error()


def test_null_arguments_rejected_without_device(built_library):
    from barbu_gb300 import hairsim
    L = hairsim.lib()
    assert L.hs_update(None, C.c_float(0.016)) == abi.HS_ERR_INVALID_ARG
    assert L.hs_destroy(None) == abi.HS_ERR_INVALID_ARG
    assert L.hs_set_spheres(None, None, 0) == abi.HS_ERR_INVALID_ARG
    assert b"null" in L.hs_last_error_string()
