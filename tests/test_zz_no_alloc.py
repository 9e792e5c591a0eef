"""gmgs_dot_dev_noalloc: the inner product for callers that cannot allocate
device memory (hosts whose device memory belongs to their own allocator, such
as a MATLAB MEX shim on gpuArray buffers, and code paths that cannot afford
the device synchronisation of cudaMalloc/cudaFree).  It keeps its scratch in
a static device array inside libgmgs, so it must agree with the handle-based
gmgs_dot_dev, call after call, and refuse lengths beyond that array.

This file is collected last on purpose, so a failure here stops a
`pytest -x` run only after every other test has run."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def handle_solver():
    from gmgs import Solver
    # any handle serves gmgs_dot_dev; a small solid block is enough
    return Solver(np.ones((8, 8, 8), np.int32), num_levels=2)


# 3,000,001 is not a multiple of the 8,192-element chunk and spans 367
# blocks, more than the 256 threads of the last block: its strided walk over
# the partials runs more than once.
@pytest.mark.parametrize("n", [1, 8192, 8193, 3_000_001])
def test_noalloc_dot_matches_handle_dot_twice(handle_solver, n):
    torch = pytest.importorskip("torch")
    from gmgs import _lib
    lib = _lib.load()
    rng = np.random.default_rng(1000 + n)
    x = torch.tensor(rng.standard_normal(n), device="cuda")
    y = torch.tensor(rng.standard_normal(n), device="cuda")
    out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    ref = handle_solver.dot_dev(x.data_ptr(), y.data_ptr(), n)
    scale = float(torch.sum(torch.abs(x * y)).item())
    got = []
    for _ in range(2):          # the static scratch keeps the previous call's contents
        st = lib.gmgs_dot_dev_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), n,
                                      C.c_void_p(out.data_ptr()), stream)
        assert st == 0, lib.gmgs_last_error(None)
        torch.cuda.synchronize()
        got.append(out.item())
    assert got[0] == got[1]
    assert abs(got[0] - ref) <= 1e-12 * scale


def test_noalloc_dot_rejects_oversize_and_bad_arguments():
    torch = pytest.importorskip("torch")
    from gmgs import _lib
    lib = _lib.load()
    x = torch.zeros(4, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    p = C.c_void_p(x.data_ptr())
    o = C.c_void_p(out.data_ptr())
    # checked before any device access, so the short buffers are never read
    assert lib.gmgs_dot_dev_noalloc(p, p, _lib.DOT_NOALLOC_MAX_N + 1, o, None) == _lib.ERR_INVALID_ARGUMENT
    assert b"GMGS_DOT_NOALLOC_MAX_N" in lib.gmgs_last_error(None)
    assert lib.gmgs_dot_dev_noalloc(None, p, 4, o, None) == _lib.ERR_INVALID_ARGUMENT
    assert lib.gmgs_dot_dev_noalloc(p, p, -1, o, None) == _lib.ERR_INVALID_ARGUMENT
    assert lib.gmgs_dot_dev_noalloc(p, p, 0, o, None) == 0
    torch.cuda.synchronize()
    assert out.item() == 0.0


def test_noalloc_dot_allocates_no_device_memory():
    """The property the entry point exists for: after a first call on the
    device, further calls leave the device's free memory unchanged."""
    torch = pytest.importorskip("torch")
    from gmgs import _lib
    lib = _lib.load()
    n = 1_000_003
    x = torch.ones(n, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    args = (C.c_void_p(x.data_ptr()), C.c_void_p(x.data_ptr()), n, C.c_void_p(out.data_ptr()), None)
    assert lib.gmgs_dot_dev_noalloc(*args) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(5):
        assert lib.gmgs_dot_dev_noalloc(*args) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert out.item() == float(n)
