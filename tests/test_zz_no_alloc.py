"""The allocation-free cooSort (epet_coo_sort_noalloc) against the regular
epet_coo_sort, through the C ABI.

epet_coo_sort_noalloc serves callers that cannot let the library allocate
device memory during a call (stream capture, real-time loops, integrations
whose allocator owns the device); its scratch is a fixed device array inside
the library.  Two calls in a row with different inputs check that the shared
array's leftover contents never leak into a result.  Kept last in collection
order so a failure here comes after every other test has run."""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _sorted(lib, fn, row, col, val, *extra):
    r, c, v = (torch.from_numpy(a.copy()).cuda() for a in (row, col, val))
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    args = [C.c_void_p(v.data_ptr()), C.c_void_p(r.data_ptr()), C.c_void_p(c.data_ptr()),
            len(val), *extra, stream]
    st = fn(*args)
    assert st == 0, lib.epet_last_error()
    torch.cuda.synchronize()
    return r.cpu().numpy(), c.cpu().numpy(), v.cpu().numpy()


def test_noalloc_matches_regular_two_calls(gpu_lib):
    lib = gpu_lib
    rng = np.random.default_rng(21)
    for n, nrow, ncol in ((200_000, 150_000, 140_608), (37_000, 5_000, 300)):
        row = rng.integers(0, nrow, n).astype(np.int32)
        col = rng.integers(0, ncol, n).astype(np.int32)
        val = rng.random(n).astype(np.float32)
        want = _sorted(lib, lib.epet_coo_sort, row, col, val, None, 0)
        got = _sorted(lib, lib.epet_coo_sort_noalloc, row, col, val)
        for a, b in zip(got, want):
            assert (a.view(np.uint32) == b.view(np.uint32)).all()
        order = np.lexsort((np.arange(n), col, row))
        assert (got[0] == row[order]).all() and (got[1] == col[order]).all()


def test_noalloc_rejects_oversize(gpu_lib):
    lib = gpu_lib
    n = (1 << 18) + 1
    t = torch.zeros(n, dtype=torch.int32, device="cuda")
    f = torch.zeros(n, dtype=torch.float32, device="cuda")
    st = lib.epet_coo_sort_noalloc(C.c_void_p(f.data_ptr()), C.c_void_p(t.data_ptr()),
                                   C.c_void_p(t.data_ptr()), n, None)
    assert st == 2  # EPET_ERR_CAPACITY
    assert b"at most" in lib.epet_last_error()
