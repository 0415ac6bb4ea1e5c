"""lss_tridiag_thomas_lu_noalloc: the Thomas-LU line solve for callers that may not
allocate device memory during a call (inside a memory pool or allocator they do not own,
real-time paths, hosts that reserve all device memory up front).

It is checked through the C-ABI against lss_tridiag_thomas_lu (the allocating entry point,
same kernel) on two calls in a row -- the second with different inputs, so state left in the
shared fixed scratch by the first call cannot leak into the result -- for its size limit, and for
what it exists for: after the per-device warm-up (a call with lines = 0) a solve leaves the
device's free memory unchanged.
This file is collected last so a failure here stops a -x run only after every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(rng, n, lines, dtype):
    lo = rng.uniform(-1, 0, (n, lines)).astype(dtype)
    up = rng.uniform(-1, 0, (n, lines)).astype(dtype)
    dg = (2.5 + rng.uniform(0, 1, (n, lines))).astype(dtype)
    rhs = rng.normal(size=(n, lines)).astype(dtype)
    blo = rng.normal(size=lines).astype(dtype)
    bhi = rng.normal(size=lines).astype(dtype)
    return lo, dg, up, rhs, blo, bhi


def _call(lib, fn, precision, arrays, stream):
    import torch

    dt = torch.float32 if precision == 1 else torch.float64
    dev = [torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device="cuda") for a in arrays]
    x = torch.full_like(dev[3], float("nan"))
    n, lines = dev[0].shape
    rc = getattr(lib, fn)(precision, n, lines, dev[0].data_ptr(), dev[1].data_ptr(), dev[2].data_ptr(),
                          dev[3].data_ptr(), dev[4].data_ptr(), dev[5].data_ptr(), x.data_ptr(), ctypes.c_void_p(stream))
    torch.cuda.synchronize()
    return rc, x.cpu().numpy()


@pytest.mark.parametrize("precision,n,lines", [(0, 256, 1000), (1, 130, 777), (0, 4, 3)])
def test_noalloc_matches_allocating_entry_point_twice(lss, precision, n, lines):
    import torch

    from linear_system_solvers_gb300 import _lib as L

    lib = L.load()
    stream = torch.cuda.current_stream().cuda_stream
    dtype = np.float32 if precision == 1 else np.float64
    rng = np.random.default_rng(n + lines)
    for _ in range(2):
        arrays = _inputs(rng, n, lines, dtype)
        rc_ref, ref = _call(lib, "lss_tridiag_thomas_lu", precision, arrays, stream)
        rc, got = _call(lib, "lss_tridiag_thomas_lu_noalloc", precision, arrays, stream)
        assert rc_ref == L.OK and rc == L.OK, lib.lss_adi_last_error()
        assert np.array_equal(got, ref)


def test_noalloc_rejects_sizes_beyond_its_scratch(lss):
    from linear_system_solvers_gb300 import _lib as L

    lib = L.load()
    # 1025 * 1024 doubles = 8 MiB + 8 KiB > the 8 MiB fixed scratch: rejected before any launch
    rc = lib.lss_tridiag_thomas_lu_noalloc(0, 1025, 1024, 1, 1, 1, 1, 1, 1, 1, None)
    assert rc == L.EINVAL
    assert "exceeds the fixed scratch" in lib.lss_adi_last_error().decode()


def test_noalloc_call_after_warm_up_allocates_nothing(lss):
    import torch

    from linear_system_solvers_gb300 import _lib as L

    lib = L.load()
    stream = torch.cuda.current_stream().cuda_stream
    # the per-device warm-up: address lookup and module load, no solve
    assert lib.lss_tridiag_thomas_lu_noalloc(0, 64, 0, None, None, None, None, None, None, None,
                                             ctypes.c_void_p(stream)) == L.OK
    rng = np.random.default_rng(5)
    arrays = _inputs(rng, 200, 3000, np.float64)
    dev = [torch.as_tensor(np.ascontiguousarray(a), device="cuda") for a in arrays]
    x = torch.empty_like(dev[3])
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        rc = lib.lss_tridiag_thomas_lu_noalloc(0, 200, 3000, dev[0].data_ptr(), dev[1].data_ptr(), dev[2].data_ptr(),
                                               dev[3].data_ptr(), dev[4].data_ptr(), dev[5].data_ptr(), x.data_ptr(),
                                               ctypes.c_void_p(stream))
        assert rc == L.OK, lib.lss_adi_last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    rc_ref, ref = _call(lib, "lss_tridiag_thomas_lu", 0, arrays, stream)
    assert rc_ref == L.OK
    assert np.array_equal(x.cpu().numpy(), ref)
