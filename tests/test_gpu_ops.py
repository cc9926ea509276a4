"""Sparse-format and MLEM operators on the GPU against the reference's known
answers (its own unit tests) and the golden fixtures; MLEM driver parity
with the oracle; edge cases."""
import numpy as np
import pytest
import torch

from epetreco_gb300 import api
from epetreco_gb300._lib import EpetError
from epetreco_gb300.problem import Problem, VoxelGrid, config, two_head_setup

pytestmark = pytest.mark.gpu


def bits(a):
    return np.asarray(a, np.float32).view(np.uint32)


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_coosort_kat(gpu_lib, golden):
    # test_cooSort.cu:17-33
    a = dev(np.array([1, 3, 2, 2, 1, 3], np.int32))
    b = dev(np.array([2, 2, 1, 2, 1, 1], np.int32))
    c = dev(np.array([2, 6, 3, 4, 1, 5], np.float32))
    api.cooSort(c, a, b)
    assert (a.cpu().numpy() == golden["coosort_row"]).all()
    assert (b.cpu().numpy() == golden["coosort_col"]).all()
    assert (c.cpu().numpy() == golden["coosort_val"]).all()


def test_coosort_stable_random(gpu_lib, golden):
    row, col, val = golden["coosort_rand_in"]
    r, c, v = dev(row.copy()), dev(col.copy()), dev(val.view(np.float32).copy())
    api.cooSort(v, r, c)
    ro, co, vo = golden["coosort_rand_out"]
    assert (r.cpu().numpy() == ro).all() and (c.cpu().numpy() == co).all()
    assert (bits(v.cpu().numpy()) == vo.view(np.uint32)).all()


def test_coosort_large_matches_numpy(gpu_lib):
    rng = np.random.default_rng(9)
    n = 300_000
    row = rng.integers(0, 200_000, n).astype(np.int32)
    col = rng.integers(0, 140_608, n).astype(np.int32)
    val = np.arange(n, dtype=np.float32)  # ties keep input order
    r, c, v = dev(row), dev(col), dev(val)
    api.cooSort(v, r, c)
    order = np.lexsort((np.arange(n), col, row))
    assert (r.cpu().numpy() == row[order]).all()
    assert (c.cpu().numpy() == col[order]).all()
    assert (v.cpu().numpy() == val[order]).all()


@pytest.mark.parametrize("ncols", [(1 << 18) + 1, (1 << 27) + 3])
def test_csc_beyond_two_radix_passes(gpu_lib, ncols):
    """Column-major copies of grids above 2^18 voxels (three and four 9-bit
    passes): stable transpose against numpy, empty columns included."""
    rng = np.random.default_rng(ncols & 0xffff)
    m = 3000
    lens = rng.integers(0, 300, m)
    rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    hot = np.unique(rng.integers(0, ncols, 2000))  # columns shared by many rows
    col = np.concatenate([np.sort(rng.choice(hot, l, replace=False)) for l in lens]).astype(
        np.int32)
    val = rng.random(col.size).astype(np.float32)
    A = api.Csr(dev(rp), dev(col), dev(val), ncols)
    At = api.csr_to_csc(A)
    r = np.repeat(np.arange(m), lens)
    order = np.lexsort((r, col))
    cnt = np.bincount(col, minlength=ncols)
    got_ptr = At.col_ptr.cpu().numpy()
    assert got_ptr[0] == 0 and (np.diff(got_ptr) == cnt).all()
    assert (At.row.cpu().numpy() == r[order]).all()
    assert (bits(At.val.cpu().numpy()) == bits(val[order])).all()


def test_coo2csr_kat(gpu_lib, golden):
    # test_cusparseWrapper.cu:20-55
    csr = api.convertCoo2Csr(dev(golden["coo2csr_row"]), 9, 4)
    assert list(csr.cpu().numpy()) == [0, 1, 4, 6, 9]


def test_csr2ecsr_kat(gpu_lib, golden):
    # test_convertCsr2Ecsr.cu:7-26
    e = api.convertCsr2Ecsr(dev(golden["ecsr_yrid"]), 3, dev(golden["ecsr_csr"].astype(np.int64)),
                            7)
    assert list(e.cpu().numpy()) == [0, 3, 3, 5]


def test_mlem_operations_kat(gpu_lib, golden):
    # test_mlemOperations.cu:39-44
    n = 10
    A = dev(np.array([(i + 1) ** 2 for i in range(n)], np.float32))
    B = dev(np.full(n, 10, np.float32))
    C = dev(np.arange(1, n + 1, dtype=np.float32))
    D = torch.zeros(n, device="cuda")
    api.divides(D, A, C)
    assert (bits(D.cpu().numpy()) == bits(golden["mlem_divides"])).all()
    api.dividesMultiplies(D, A, B, C)
    assert (bits(D.cpu().numpy()) == bits(golden["mlem_divmul"])).all()
    norm = api.sum(D)
    assert norm == 550.0
    api.scales(D, np.float32(1.0 / norm))
    assert (bits(D.cpu().numpy()) == bits(golden["mlem_scales"])).all()


def test_divides_multiplies_guard(gpu_lib):
    r = torch.zeros(1, device="cuda")
    api.dividesMultiplies(r, dev(np.array([2.0], np.float32)), dev(np.array([3.0], np.float32)),
                          dev(np.array([0.0], np.float32)))
    assert r.item() == 6.0


def test_sum_f64_accuracy(gpu_lib):
    x = np.random.default_rng(1).random(1_000_003).astype(np.float32)
    assert abs(api.sum(dev(x)) - x.astype(np.float64).sum()) < 1e-6


# ------------------------------------------------------------ edge cases

def test_empty_row_list(gpu_lib):
    p = config("small")["problem"]
    empty = torch.zeros(0, dtype=torch.int32, device="cuda")
    A = api.systemMatrixCalculation(p, empty)
    assert A.m == 0 and A.nnz == 0
    cnl, vxl, off = api.getWorkqueue(p, empty)
    assert cnl.numel() == 0
    y = api.CSRmv(0, A, torch.ones(p.nvoxels, device="cuda"))
    assert y.numel() == 0


def test_channels_missing_the_grid(gpu_lib):
    """A grid off to the side: no candidates, empty rows."""
    s = two_head_setup(4, 45.0)
    g = VoxelGrid((0.2, 0.2, 0.2), (0.002,) * 3, (8, 8, 8))
    p = Problem(s, g, 10)
    rows = torch.arange(0, 500, dtype=torch.int32, device="cuda")
    A = api.systemMatrixCalculation(p, rows)
    assert A.nnz == 0 and (A.row_ptr == 0).all()


def test_invalid_arguments_raise(gpu_lib):
    p = config("small")["problem"]
    bad = Problem(p.setup, p.grid, 0)
    with pytest.raises(EpetError, match="nrays"):
        api.systemMatrixCalculation(bad, torch.zeros(1, dtype=torch.int32, device="cuda"))


def test_capacity_error_reports_required(gpu_lib):
    import ctypes as C
    from epetreco_gb300._lib import CsrC, lib, problem_struct
    p = config("small")["problem"]
    rows = torch.tensor([100, 200, 3000], dtype=torch.int32, device="cuda")
    A = api.systemMatrixCalculation(p, rows)
    rp = torch.empty(4, dtype=torch.int64, device="cuda")
    col = torch.empty(5, dtype=torch.int32, device="cuda")
    val = torch.empty(5, dtype=torch.float32, device="cuda")
    cs = CsrC(3, p.nvoxels, 0, rp.data_ptr(), col.data_ptr(), val.data_ptr())
    nnz = C.c_int64(0)
    st = lib().epet_sm_build(C.byref(problem_struct(p)), C.c_void_p(rows.data_ptr()), 3,
                             C.byref(cs), 5, C.byref(nnz), 0, None, 0,
                             C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 2 and nnz.value == A.nnz
    assert (rp == A.row_ptr).all()


def test_degenerate_single_voxel_grid(gpu_lib, oracle):
    """One voxel, one angle: candidates and values still match the oracle."""
    s = two_head_setup(1, 0.0)
    g = VoxelGrid((-0.004, -0.004, -0.004), (0.008,) * 3, (1, 1, 1))
    p = Problem(s, g, 16)
    rows = np.arange(p.nchannels, dtype=np.int32)
    A = api.systemMatrixCalculation(p, dev(rows))
    trig = api.trig_table(p).cpu().numpy()
    rnd = api.dump_uniforms(p, dev(rows)).cpu().numpy()
    orp, ocol, oval = oracle.sm_build_csr(p, rows, p.nrays, rnd, exact=True, trig=trig)
    assert (A.row_ptr.cpu().numpy() == orp).all()
    assert (bits(A.val.cpu().numpy()) == bits(oval)).all()


# ---------------------------------------------------------- MLEM driver

@pytest.fixture(scope="module")
def small_recon(gpu_lib):
    from epetreco_gb300.phantom import phantom_image
    p = config("small")["problem"]
    rng = np.random.default_rng(4)
    rows = np.sort(rng.choice(p.nchannels, 4000, replace=False)).astype(np.int32)
    x_true = phantom_image(p, 1)
    A = api.systemMatrixCalculation(p.with_seed(7919), dev(rows))
    ybar = api.CSRmv(0, A, dev(x_true)).double()
    lam = ybar * (2e5 / ybar.sum())
    y = torch.poisson(lam, generator=torch.Generator(device="cuda").manual_seed(2)).float()
    keep = (y > 0).cpu().numpy()
    rows = rows[keep]
    y = y[torch.from_numpy(keep).cuda()].contiguous()
    s = api.sensitivity(p, dev(rows))
    return p, rows, y, s


@pytest.mark.parametrize("layout", [api.LAYOUT_GROUPED, api.LAYOUT_CSC], ids=["grouped", "csc"])
def test_mlem_matches_oracle(small_recon, oracle, layout):
    """5 iterations: image within 1e-4 relative L2 of the oracle's fp32
    sequence (reco.cu:209-281) on the same matrix, and within 1e-4 of the
    fp64 oracle, in both layouts of the stored matrix."""
    p, rows, y, s = small_recon
    R = api.Mlem(p, dev(rows), y, s, use_graph=True, layout=layout)
    R.iterate(5)
    x = R.image().cpu().numpy()
    A = api.systemMatrixCalculation(p, dev(rows))
    rp, col, val = (t.cpu().numpy() for t in (A.row_ptr, A.col, A.val))
    s_n = s.cpu().numpy()
    s_n = (s_n / s_n.astype(np.float64).sum()).astype(np.float32)
    x0 = np.full(p.nvoxels, np.float32(1.0 / p.nvoxels), np.float32)
    xo = oracle.mlem(rp, col, val, y.cpu().numpy(), s_n, x0, 5, p.nvoxels)
    err = np.linalg.norm(x - xo) / np.linalg.norm(xo)
    assert err <= 1e-4, err
    x64 = oracle.mlem_f64(rp, col, val, y.cpu().numpy().astype(np.float64),
                          s_n.astype(np.float64), x0.astype(np.float64), 5, p.nvoxels)
    err64 = np.linalg.norm(x - x64) / np.linalg.norm(x64)
    assert err64 <= 1e-4, err64
    assert abs(x.astype(np.float64).sum() - 1.0) < 1e-5


def test_mlem_graph_equals_eager(small_recon):
    p, rows, y, s = small_recon
    a = api.Mlem(p, dev(rows), y, s, use_graph=True)
    b = api.Mlem(p, dev(rows), y, s, use_graph=False)
    la = a.iterate(3, loglik=True)
    lb = b.iterate(3, loglik=True)
    assert torch.equal(a.image(), b.image())
    assert la == lb


def test_mlem_row_order_does_not_matter(small_recon):
    """The reconstruction stores its rows in crystal-pair order (a bijective
    key of the channel), so a shuffled measurement list gives the same
    matrices and the bit-identical image and log-likelihood."""
    p, rows, y, s = small_recon
    perm = np.random.default_rng(5).permutation(len(rows))
    a = api.Mlem(p, dev(rows), y, s)
    b = api.Mlem(p, dev(rows[perm]), y[dev(perm)].contiguous(), s)
    la = a.iterate(4, loglik=True)
    lb = b.iterate(4, loglik=True)
    assert torch.equal(a.image(), b.image())
    assert la == lb


def test_mlem_loglik_increases(small_recon):
    p, rows, y, s = small_recon
    R = api.Mlem(p, dev(rows), y, s)
    lls = [R.iterate(1, loglik=True) for _ in range(6)]
    assert all(b >= a - 1e-6 * abs(a) for a, b in zip(lls[1:], lls[2:]))


def test_sensitivity_matches_oracle(small_recon, oracle):
    p, rows, y, s = small_recon
    A = api.systemMatrixCalculation(p, dev(rows))
    rp, col, val = (t.cpu().numpy() for t in (A.row_ptr, A.col, A.val))
    so = oracle.sensitivity(rp, col, val, p.nvoxels)
    assert np.allclose(s.cpu().numpy(), so, rtol=1e-5, atol=1e-12)


@pytest.mark.parametrize("offset", [0, 1, 3])
def test_csrmv_ragged_rows_any_alignment(gpu_lib, oracle, offset):
    """Rows of every length from 0 up (starts at every residue mod 4), with the
    value and column streams starting 0, 4 or 12 bytes past a 16-byte boundary
    (the aligned form uses 16-byte loads, the others element loads)."""
    import ctypes as C
    from epetreco_gb300._lib import CscC, CsrC, check, lib
    rng = np.random.default_rng(31 + offset)
    n = 5000
    lens = np.concatenate([np.arange(0, 70), rng.integers(0, 400, 900), [0, 1, 2, 3, 5000]])
    rng.shuffle(lens)
    rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    nnz = int(rp[-1])
    col = np.concatenate([np.sort(rng.choice(n, l, replace=False)) for l in lens]).astype(np.int32)
    val = rng.random(nnz).astype(np.float32)
    x = rng.random(n).astype(np.float32)
    col_d = dev(np.concatenate([np.zeros(offset, np.int32), col]))
    val_d = dev(np.concatenate([np.zeros(offset, np.float32), val]))
    rp_d = dev(rp)
    a = CsrC(len(lens), n, nnz, rp_d.data_ptr(), col_d.data_ptr() + 4 * offset,
             val_d.data_ptr() + 4 * offset)
    y = torch.zeros(len(lens), device="cuda")
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    check(lib().epet_csrmv(0, C.byref(a), None, 1.0, C.c_void_p(dev(x).data_ptr()), 0.0,
                           C.c_void_p(y.data_ptr()), st))
    yo = oracle.csrmv_f64(0, rp, col, val, x.astype(np.float64), n)
    got = y.cpu().numpy()
    assert (got[lens == 0] == 0).all()
    nz = lens > 0
    assert np.abs(got[nz] - yo[nz]).max() <= 1e-5 * np.abs(yo[nz]).max()


@pytest.mark.parametrize("fmt", [0, api.BF16, api.FP16], ids=["fp32", "bf16", "fp16"])
def test_grouped_layout_equals_csc_layout(small_recon, fmt):
    """The one-pass grouped iteration against the CSR + column-major copy:
    FP32 images equal up to fp32 summation order, the 16-bit forms within
    1e-3 of FP32; the same grouped object iterated twice is bit-equal."""
    p, rows, y, s = small_recon
    a = api.Mlem(p, dev(rows), y, s, layout=api.LAYOUT_GROUPED, value_format=fmt)
    c = api.Mlem(p, dev(rows), y, s, layout=api.LAYOUT_GROUPED, value_format=fmt)
    b = api.Mlem(p, dev(rows), y, s, layout=api.LAYOUT_CSC)
    la, lb, lc = (r.iterate(6, loglik=True) for r in (a, b, c))
    xa, xb = a.image().double(), b.image().double()
    tol = 1e-6 if fmt == 0 else 1e-3
    assert float((xa - xb).norm() / xb.norm()) <= tol
    assert torch.equal(a.image(), c.image()) and la == lc
    assert abs(la - lb) <= (1e-6 if fmt == 0 else 1e-4) * abs(lb)


def test_grouped_layout_wide_rows(gpu_lib, oracle):
    """Rows wider than a group's shared table (1 mm voxels along 256 mm of
    the lines, 16 rays: thousands of entries a row) keep their own columns
    as their table; against the column-major layout and the FP64 oracle."""
    s = two_head_setup(2, 90.0, pos=0.25, n=3)
    g = VoxelGrid((-0.128, -0.008, -0.008), (0.001, 0.001, 0.001), (256, 16, 16))
    p = Problem(s, g, 16)
    rows = torch.arange(p.nchannels, dtype=torch.int32, device="cuda")
    A = api.systemMatrixCalculation(p, rows)
    lens = torch.diff(A.row_ptr)
    assert int(lens.max()) > 1536  # wider than the shared table
    y = torch.full((p.nchannels,), 50.0, device="cuda")
    sens = api.sensitivity(p)
    a = api.Mlem(p, rows, y, sens, layout=api.LAYOUT_GROUPED)
    b = api.Mlem(p, rows, y, sens, layout=api.LAYOUT_CSC)
    a.iterate(4)
    b.iterate(4)
    xa, xb = a.image().double(), b.image().double()
    assert float((xa - xb).norm() / xb.norm()) <= 1e-6
    rp, col, val = (t.cpu().numpy() for t in (A.row_ptr, A.col, A.val))
    s64 = oracle.csrmv_f64(1, rp, col, val, np.ones(p.nchannels), p.nvoxels)
    x64 = oracle.mlem_f64(rp, col, val, np.full(p.nchannels, 50.0), s64 / s64.sum(),
                          np.full(p.nvoxels, 1.0 / p.nvoxels), 4, p.nvoxels)
    assert np.linalg.norm(xa.cpu().numpy() - x64) / np.linalg.norm(x64) <= 1e-4


def test_grouped_layout_beyond_two_radix_passes(gpu_lib):
    """A grid above 2^18 voxels (65^3): the grouped layout's slot lists take
    three radix passes; its iteration against the column-major layout's."""
    s = two_head_setup(2, 90.0, pos=0.25, n=5)
    g = VoxelGrid((-0.065, -0.065, -0.065), (0.002, 0.002, 0.002), (65, 65, 65))
    p = Problem(s, g, 8)
    assert p.nvoxels > (1 << 18)
    rows = torch.arange(p.nchannels, dtype=torch.int32, device="cuda")
    y = torch.full((p.nchannels,), 20.0, device="cuda")
    sens = api.sensitivity(p)
    a = api.Mlem(p, rows, y, sens, layout=api.LAYOUT_GROUPED)
    b = api.Mlem(p, rows, y, sens, layout=api.LAYOUT_CSC)
    la, lb = a.iterate(3, loglik=True), b.iterate(3, loglik=True)
    xa, xb = a.image().double(), b.image().double()
    assert float((xa - xb).norm() / xb.norm()) <= 1e-6
    assert abs(la - lb) <= 1e-6 * abs(lb)
