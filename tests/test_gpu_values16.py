"""16-bit system-matrix storage (BF16 / FP16 values with a per-row FP32 scale,
16-bit column steps): exact columns, bounded value error, products and MLEM
against the oracle."""
import ctypes as C

import numpy as np
import pytest
import torch

from epetreco_gb300 import api
from epetreco_gb300._lib import Csr16C, CsrC, check, lib
from epetreco_gb300.problem import config

pytestmark = pytest.mark.gpu

FORMATS = {"bf16": 1, "fp16": 2}


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def compress(rp, col, val, n, fmt):
    """Returns the device arrays of the 16-bit layout of a host CSR."""
    m = len(rp) - 1
    rp_d, col_d, val_d = dev(rp.astype(np.int64)), dev(col.astype(np.int32)), dev(val.astype(np.float32))
    a = CsrC(m, n, len(col), rp_d.data_ptr(), col_d.data_ptr() if len(col) else None,
             val_d.data_ptr() if len(col) else None)
    cnt = torch.empty(m + 1, dtype=torch.int64, device="cuda")
    n16 = C.c_int64(0)
    check(lib().epet_csr16_count(C.byref(a), C.c_void_p(cnt.data_ptr()), C.byref(n16), stream()))
    cap = max(n16.value, 8)
    out = dict(row_ptr=torch.empty(m + 1, dtype=torch.int64, device="cuda"),
               base=torch.empty(cap // 8, dtype=torch.int32, device="cuda"),
               scale=torch.empty(max(m, 1), dtype=torch.float32, device="cuda"),
               delta=torch.zeros(cap, dtype=torch.int16, device="cuda"),
               q=torch.zeros(cap, dtype=torch.int16, device="cuda"))
    c16 = Csr16C(m, n, cap, *(out[k].data_ptr() for k in ("row_ptr", "base", "scale", "delta", "q")),
                 fmt)
    check(lib().epet_csr_compress(C.byref(a), fmt, C.byref(c16), stream()))
    torch.cuda.synchronize()
    return c16, out, (rp_d, col_d, val_d)


def decode(out, fmt):
    """Columns and values per row: chunks of 8, col = base[chunk] + offset."""
    rp = out["row_ptr"].cpu().numpy()
    base = out["base"].cpu().numpy().astype(np.int64)
    scale = out["scale"].cpu().numpy()
    d = out["delta"].cpu().numpy().view(np.uint16).astype(np.int64)
    q = out["q"].cpu().numpy().view(np.uint16)
    if fmt == 1:
        qv = (q.astype(np.uint32) << 16).view(np.float32)
    else:
        qv = q.view(np.float16).astype(np.float32)
    cols, vals = [], []
    for r in range(len(rp) - 1):
        assert rp[r] % 8 == 0 and rp[r + 1] % 8 == 0
        k = np.arange(rp[r], rp[r + 1])
        c = base[k // 8] + d[k]
        v = qv[k].astype(np.float64) * scale[r]
        keep = v != 0
        cols.append(c[keep])
        vals.append(v[keep])
    return cols, vals


@pytest.fixture(scope="module")
def mat(gpu_lib):
    p = config("small")["problem"]
    rows = np.sort(np.random.default_rng(8).choice(p.nchannels, 600, replace=False)).astype(np.int32)
    A = api.systemMatrixCalculation(p, dev(rows))
    return p, rows, A, tuple(t.cpu().numpy() for t in (A.row_ptr, A.col, A.val))


@pytest.mark.parametrize("fmt", ["bf16", "fp16"])
def test_columns_exact_values_bounded(mat, fmt):
    p, rows, A, (rp, col, val) = mat
    f = FORMATS[fmt]
    c16, out, _ = compress(rp, col, val, p.nvoxels, f)
    cols, vals = decode(out, f)
    tol = 2.0 ** -8 if fmt == "bf16" else 2.0 ** -11
    for r in range(len(rp) - 1):
        cc, vv = col[rp[r]:rp[r + 1]], val[rp[r]:rp[r + 1]].astype(np.float64)
        sc = vv.max() if len(vv) else 1.0
        # every non-zero survives with its exact column (fp16 may flush
        # values below 2^-24 of the row maximum to zero)
        keep = vv > (0 if fmt == "bf16" else sc * 2.0 ** -24)
        dec = dict(zip(cols[r].tolist(), vals[r].tolist()))
        assert set(cc[keep].tolist()) <= set(dec)
        got = np.array([dec.get(c, 0.0) for c in cc])
        err = np.abs(got - vv)
        assert (err <= tol * vv + sc * 2.0 ** -24).all()


def test_wide_column_gaps_end_chunks(gpu_lib):
    rp = np.array([0, 4, 5, 5], np.int64)
    col = np.array([0, 70000, 200000, 299999, 5], np.int32)
    val = np.array([1.0, 2.0, 3.0, 4.0, 0.5], np.float32)
    for f in (1, 2):
        c16, out, _ = compress(rp, col, val, 300000, f)
        # every gap in row 0 exceeds 65535 columns: four chunks of 8; row 1: one
        assert c16.nnz == 8 * 4 + 8
        cols, vals = decode(out, f)
        assert cols[0].tolist() == [0, 70000, 200000, 299999] and cols[1].tolist() == [5]
        assert len(cols[2]) == 0
        assert np.allclose(vals[0], [1, 2, 3, 4], rtol=4e-3)


def test_fixed_chunks_and_padding(gpu_lib):
    """Rows of every length 0..40 with small gaps: whole chunks, padded."""
    rng = np.random.default_rng(4)
    lens = np.arange(41)
    rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    col = np.concatenate([np.sort(rng.choice(4000, l, replace=False)) for l in lens]).astype(np.int32)
    val = rng.random(len(col)).astype(np.float32) + 0.01
    c16, out, _ = compress(rp, col, val, 4000, 1)
    assert c16.nnz == sum((l + 7) // 8 * 8 for l in lens)
    cols, vals = decode(out, 1)
    for r in range(len(lens)):
        assert cols[r].tolist() == col[rp[r]:rp[r + 1]].tolist()


def test_unordered_columns(mat, oracle):
    """Columns in any order within a row (as a reconstruction stores them):
    each chunk's base is its smallest column, entries keep their places, and
    a chunk ends before its column range would reach 65536."""
    p, rows, A, (rp, col, val) = mat
    rng = np.random.default_rng(6)
    col2, val2 = col.copy(), val.copy()
    for r in range(len(rp) - 1):
        k = rng.permutation(rp[r + 1] - rp[r]) + rp[r]
        col2[rp[r]:rp[r + 1]], val2[rp[r]:rp[r + 1]] = col[k], val[k]
    c16, out, keep_alive = compress(rp, col2, val2, p.nvoxels, 1)
    cols, vals = decode(out, 1)
    for r in range(len(rp) - 1):
        assert cols[r].tolist() == col2[rp[r]:rp[r + 1]].tolist()
    x = np.random.default_rng(2).random(p.nvoxels).astype(np.float32)
    y = torch.zeros(len(rows), device="cuda")
    check(lib().epet_csr16_mv(C.byref(c16), 1.0, C.c_void_p(dev(x).data_ptr()), 0.0,
                              C.c_void_p(y.data_ptr()), stream()))
    yo = oracle.csrmv_f64(0, rp, col, val, x.astype(np.float64), p.nvoxels)
    assert (np.abs(y.cpu().numpy() - yo) / np.abs(yo)).max() < 3e-3
    # a descending row whose range exceeds 65535: chunks split, offsets >= 0
    rp3 = np.array([0, 5], np.int64)
    col3 = np.array([200000, 150000, 140000, 100000, 3], np.int32)
    val3 = np.array([1.0, 2.0, 3.0, 4.0, 5.0], np.float32)
    c16, out, _ = compress(rp3, col3, val3, 300000, 1)
    cols, vals = decode(out, 1)
    assert cols[0].tolist() == col3.tolist()
    assert np.allclose(vals[0], val3, rtol=4e-3)


@pytest.mark.parametrize("fmt", ["bf16", "fp16"])
def test_product_against_oracle(mat, oracle, fmt):
    p, rows, A, (rp, col, val) = mat
    f = FORMATS[fmt]
    c16, out, keep_alive = compress(rp, col, val, p.nvoxels, f)
    x = np.random.default_rng(2).random(p.nvoxels).astype(np.float32)
    y = torch.zeros(len(rows), device="cuda")
    check(lib().epet_csr16_mv(C.byref(c16), 1.0, C.c_void_p(dev(x).data_ptr()), 0.0,
                              C.c_void_p(y.data_ptr()), stream()))
    yo = oracle.csrmv_f64(0, rp, col, val, x.astype(np.float64), p.nvoxels)
    rel = np.abs(y.cpu().numpy() - yo) / np.abs(yo)
    assert rel.max() < (3e-3 if fmt == "bf16" else 4e-4), rel.max()


@pytest.mark.parametrize("fmt", ["bf16", "fp16"])
def test_mlem_16bit_within_1e3_of_fp64(gpu_lib, oracle, fmt):
    """The 16-bit forms' bound: image error <= 1e-3 relative L2 vs the FP64 oracle."""
    from epetreco_gb300.phantom import measurement
    p = config("small")["problem"]
    rows, y, _ = measurement(p, 1e6)
    s = api.sensitivity(p)
    R = api.Mlem(p, rows, y, s, value_format=FORMATS[fmt])
    R.iterate(5)
    x = R.image().cpu().numpy()
    A = api.systemMatrixCalculation(p, rows)
    rp, col, val = (t.cpu().numpy() for t in (A.row_ptr, A.col, A.val))
    sn = s.cpu().numpy().astype(np.float64)
    sn /= sn.sum()
    x0 = np.full(p.nvoxels, 1.0 / p.nvoxels)
    x64 = oracle.mlem_f64(rp, col, val, y.cpu().numpy().astype(np.float64), sn, x0, 5,
                          p.nvoxels)
    err = np.linalg.norm(x - x64) / np.linalg.norm(x64)
    assert err <= 1e-3, err
    st = R.stats()
    assert st["bytes_per_iteration"] < 0.62 * 16 * st["nnz"]


def test_unaligned_16bit_streams_are_rejected(gpu_lib):
    rp = np.array([0, 3], np.int64)
    col = np.array([1, 2, 9], np.int32)
    val = np.array([1.0, 2.0, 3.0], np.float32)
    c16, out, _ = compress(rp, col, val, 10, 1)
    c16.q = out["q"].data_ptr() + 2
    y = torch.zeros(1, device="cuda")
    x = torch.ones(10, device="cuda")
    st = lib().epet_csr16_mv(C.byref(c16), 1.0, C.c_void_p(x.data_ptr()), 0.0,
                             C.c_void_p(y.data_ptr()), stream())
    assert st != 0 and b"aligned" in lib().epet_last_error()
