"""The C-ABI library loads and exports every entry point include/gmgs.h declares.

No compute calls: these run without a GPU.  Calls exercised here only touch
host-side logic (defaults, status strings, argument validation that fails
before any CUDA call).
"""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "gmgs.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(gmgs_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_header_declares_the_path():
    names = declared_functions()
    for required in ("gmgs_create", "gmgs_set_bc", "gmgs_solve", "gmgs_stress", "gmgs_grad",
                     "gmgs_apply_operator", "gmgs_apply_preconditioner", "gmgs_destroy"):
        assert required in names


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_binding_covers_every_declared_symbol():
    from gmgs import _lib
    assert set(declared_functions()) == set(_lib.SIGNATURES)


def test_default_params_match_reference_globals(lib):
    from gmgs import _lib
    p = _lib.Params()
    lib.gmgs_default_params(C.byref(p))
    # src/GlobalVariables.m:3-23
    assert (p.tol, p.max_it, p.omega, p.youngs_modulus, p.poisson_ratio, p.coarsest_resolution_control) == \
        (1e-3, 20000, 0.4, 1.0, 0.3, 10000)
    assert p.num_levels == 0 and p.precision == 0


def test_status_strings(lib):
    for code in range(13):
        assert lib.gmgs_status_string(code)
    assert lib.gmgs_status_string(0) == b"ok"


def test_create_rejects_bad_arguments_before_touching_cuda(lib):
    from gmgs import _lib
    h = C.c_void_p()
    occ = np.ones(8, np.int32)
    ptr = occ.ctypes.data_as(C.POINTER(C.c_int32))
    assert lib.gmgs_create(None, 2, 2, 2, None, None, C.byref(h)) == _lib.ERR_INVALID_ARGUMENT
    assert lib.gmgs_create(ptr, 0, 2, 2, None, None, C.byref(h)) == _lib.ERR_INVALID_ARGUMENT
    bad = (C.c_double * 3)(1.0, -1.0, 1.0)
    assert lib.gmgs_create(ptr, 2, 2, 2, bad, None, C.byref(h)) == _lib.ERR_INVALID_ARGUMENT
    p = _lib.Params()
    lib.gmgs_default_params(C.byref(p))
    p.poisson_ratio = 0.5
    assert lib.gmgs_create(ptr, 2, 2, 2, None, C.byref(p), C.byref(h)) == _lib.ERR_INVALID_ARGUMENT
    lib.gmgs_default_params(C.byref(p))
    # 8 voxels < coarsestResolutionControl_ (DiscretizeDesignDomain.m:30-32)
    assert lib.gmgs_create(ptr, 2, 2, 2, None, C.byref(p), C.byref(h)) == _lib.ERR_RESOLUTION
    p.num_levels = 1          # SetupSolver.m:19-21
    assert lib.gmgs_create(ptr, 2, 2, 2, None, C.byref(p), C.byref(h)) == _lib.ERR_RESOLUTION
    assert h.value is None
    assert b"Resolution" in lib.gmgs_last_error(None) or b"resolution" in lib.gmgs_last_error(None)


def test_null_handle_queries(lib):
    from gmgs import _lib
    v = C.c_int32()
    assert lib.gmgs_num_levels(None, C.byref(v)) == _lib.ERR_INVALID_ARGUMENT
    assert lib.gmgs_set_bc(None, None, 0, None, 0) != _lib.OK
    lib.gmgs_destroy(None)


def test_missing_library_fails_loudly(tmp_path):
    from gmgs import _lib
    with pytest.raises(_lib.GMGSLibraryMissing):
        _lib.load(tmp_path / "libgmgs.so")


def test_checked_build_compiles_and_exports_every_symbol():
    """build.py --debug (GMGS_CHECKED) compiles on its own objects into
    libgmgs_checked.so, which exports the same C ABI."""
    import sys
    sys.path.insert(0, str(ROOT / "gmgs-3d_gb300"))
    import build as B
    path = B.build(debug=True)
    assert path.name == "libgmgs_checked.so" and path != B.LIB
    from gmgs import _lib
    chk = _lib.load(path)
    for name in declared_functions():
        assert hasattr(chk, name), name
