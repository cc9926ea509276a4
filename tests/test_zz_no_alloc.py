"""The allocation-free cooSort (epet_coo_sort_noalloc) against the regular
epet_coo_sort, through the C ABI.

epet_coo_sort_noalloc serves callers that cannot let the library allocate
device memory: a host application whose own allocator owns the device's
memory, or an integration with a memory budget fixed at start-up.  Its
scratch is a fixed device array inside the library, shared by every call.
Two calls in a row with different inputs check that the array's leftover
contents never leak into a result, and the library's allocation counter and
the device's free memory show that a call allocates nothing.  Kept last in
collection order so a failure here comes after every other test has run."""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _sorted(lib, fn, row, col, val, *extra):
    r, c, v = (torch.from_numpy(a.copy()).cuda() for a in (row, col, val))
    args = [C.c_void_p(v.data_ptr()), C.c_void_p(r.data_ptr()), C.c_void_p(c.data_ptr()),
            len(val), *extra, _stream()]
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


def test_noalloc_signed_ids_and_extremes(gpu_lib):
    """Negative ids and the int32 extremes sort in signed order (the
    reference's comparator), stably; the second call follows a larger one."""
    lib = gpu_lib
    rng = np.random.default_rng(8)
    for n in (50_000, 1_000):
        row = rng.integers(-2**31, 2**31, n, dtype=np.int64).astype(np.int32)
        row[::7] = row[3]  # repeated rows, so columns decide
        col = rng.integers(-3, 4, n).astype(np.int32)
        col[:4] = [2**31 - 1, -2**31, 0, -1]
        val = rng.random(n).astype(np.float32)
        got = _sorted(lib, lib.epet_coo_sort_noalloc, row, col, val)
        order = np.lexsort((np.arange(n), col, row))
        assert (got[0] == row[order]).all() and (got[1] == col[order]).all()
        assert (got[2].view(np.uint32) == val[order].view(np.uint32)).all()


def test_noalloc_allocates_nothing(gpu_lib):
    lib = gpu_lib
    rng = np.random.default_rng(3)
    n = 1 << 18
    row = torch.from_numpy(rng.integers(0, 5_000_000, n).astype(np.int32)).cuda()
    col = torch.from_numpy(rng.integers(0, 140_608, n).astype(np.int32)).cuda()
    val = torch.rand(n, device="cuda")
    args = [C.c_void_p(val.data_ptr()), C.c_void_p(row.data_ptr()), C.c_void_p(col.data_ptr()), n]
    assert lib.epet_coo_sort_noalloc(*args, _stream()) == 0  # warm: modules loaded
    torch.cuda.synchronize()
    a0, free0 = lib.epet_device_allocations(), torch.cuda.mem_get_info()[0]
    assert lib.epet_coo_sort_noalloc(*args, _stream()) == 0, lib.epet_last_error()
    torch.cuda.synchronize()
    assert lib.epet_device_allocations() == a0
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_oversize(gpu_lib):
    lib = gpu_lib
    n = (1 << 18) + 1
    t = torch.zeros(n, dtype=torch.int32, device="cuda")
    f = torch.zeros(n, dtype=torch.float32, device="cuda")
    st = lib.epet_coo_sort_noalloc(C.c_void_p(f.data_ptr()), C.c_void_p(t.data_ptr()),
                                   C.c_void_p(t.data_ptr()), n, None)
    assert st == 2  # EPET_ERR_CAPACITY
    assert b"at most" in lib.epet_last_error()
