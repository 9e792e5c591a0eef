"""The MATLAB MEX shim (gmgs-3d_gb300/matlab/gmgs_mex.c) compiles as C99
against include/gmgs.h with warnings as errors, and every libgmgs symbol it
calls resolves in the built library.  MATLAB is not available here, so the
MATLAB API comes from a declarations-only stand-in (tests/mex_stub/mex.h)
and the shim itself is not run."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
SHIM = ROOT / "gmgs-3d_gb300" / "matlab" / "gmgs_mex.c"
LIBDIR = ROOT / "gmgs-3d_gb300" / "gmgs"


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_mex_shim_compiles_and_links(tmp_path, lib):
    obj = tmp_path / "gmgs_mex.o"
    cc = ["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-fPIC", "-I", str(ROOT / "include"),
          "-I", str(ROOT / "tests" / "mex_stub"), "-c", str(SHIM), "-o", str(obj)]
    r = subprocess.run(cc, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    so = tmp_path / "gmgs_mex.so"
    # the MATLAB API stays undefined (MATLAB provides it); libgmgs's must resolve
    link = ["gcc", "-shared", "-o", str(so), str(obj), "-L", str(LIBDIR), "-lgmgs", "-Wl,--no-undefined",
            "-Wl,--unresolved-symbols=ignore-in-object-files"]
    r = subprocess.run(link, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    nm = subprocess.run(["nm", "-u", str(obj)], capture_output=True, text=True).stdout
    used = sorted({l.split()[-1] for l in nm.splitlines() if l.split()[-1].startswith("gmgs_")})
    assert "gmgs_solve" in used and "gmgs_stress" in used and "gmgs_set_bc" in used
    for name in used:
        assert hasattr(lib, name), name
