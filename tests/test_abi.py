"""The C-ABI library: builds, loads and exports every entry point of
include/*.h (no GPU needed; nothing here launches device work)."""
import ctypes as C
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(ifl_[a-z0-9_]+)\s*\(", src))
    return names


@pytest.fixture(scope="module")
def lib(ifl):
    return ifl.load_library()


def test_header_declares_entry_points():
    names = _declared()
    assert {"ifl_create", "ifl_update", "ifl_add_inflow", "ifl_read_field", "ifl_destroy"} <= names


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in sorted(_declared()) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_mirror_lists_every_export(ifl):
    assert set(ifl.EXPORTS) <= _declared()


def test_default_params_follow_reference(ifl, lib):
    p = ifl.Params()
    lib.ifl_default_params(C.byref(p), 3, 128, 128)
    assert (p.variant, p.w, p.h, p.precision) == (3, 128, 128, ifl.FP64)
    assert p.density_air == 0.1 and p.max_iter_pressure == 600
    lib.ifl_default_params(C.byref(p), 7, 64, 32)
    assert p.max_iter_pressure == 2000 and p.max_iter_heat == 2000
    assert p.density_soot == 1.0 and p.diffusion == 0.01


@pytest.mark.parametrize("field,value", [("variant", 0), ("variant", 9), ("w", 1), ("h", 0),
                                         ("precision", 5), ("density_air", 0.0), ("max_iter_heat", -1)])
def test_create_rejects_bad_parameters_without_touching_the_gpu(ifl, lib, field, value):
    p = ifl.Params()
    lib.ifl_default_params(C.byref(p), 3, 16, 16)
    setattr(p, field, value)
    h = C.c_void_p()
    assert lib.ifl_create(C.byref(p), C.byref(h)) == ifl.ERR_ARG
    assert not h.value


def test_flip_fp32_form_adds_only_solver_arrays(ifl, lib):
    """Step 8 keeps FP64 fields and particles in both forms; IFL_FP32 adds the
    FP32-form PCG arrays (no GPU needed: the byte count is computed on the host)."""
    p = ifl.Params()
    lib.ifl_default_params(C.byref(p), ifl.FLIP, 64, 64)
    lib.ifl_device_bytes.restype = C.c_int64
    b64 = lib.ifl_device_bytes(C.byref(p))
    p.precision = ifl.FP32
    b32 = lib.ifl_device_bytes(C.byref(p))
    assert b64 > 0 and b32 > b64
    assert b32 - b64 < 11 * 4 * 4 * 64 * 96 * 32  # the FP32 matrix, records and vectors only


def test_null_handles_are_rejected(ifl, lib):
    assert lib.ifl_update(None, 0.1) == ifl.ERR_ARG
    assert lib.ifl_destroy(None) == ifl.ERR_ARG
    assert lib.ifl_add_inflow(None, *([0.0] * 8)) == ifl.ERR_ARG
    assert lib.ifl_last_error(None) == b"invalid handle"
    assert lib.ifl_version().startswith(b"ifluids-gb300")
