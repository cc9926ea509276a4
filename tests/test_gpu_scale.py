"""Parity at the benchmark workloads' own sizes, not on samples.

* Small workload (32^3 voxels, all 228,488 channels, 10 rays): the whole
  system matrix of every channel against the oracle bit for bit; the
  sensitivity image over all channels; MLEM on the workload's measurement
  (1e6 counts, 5 iterations) from the stored and the matrix-free schedules
  against the FP64 oracle run on the oracle's own matrix (<= 1e-4 relative
  L2, the reference's image tolerance).
* Full workload (52^3 voxels, 5,140,980 channels, 100 rays): a few thousand
  rows at the library's default window capacity, including rows the walk
  redoes with a larger window and every row with an axis-parallel ray (the
  per-candidate path), bit for bit against the oracle.

The oracle gets the device's sin/cos table and cuRAND uniforms (dumped
through the library), so candidates and chords compare bit for bit."""
import numpy as np
import pytest
import torch

from epetreco_gb300 import api
from epetreco_gb300.problem import config

pytestmark = pytest.mark.gpu


def bits(a):
    return np.asarray(a, np.float32).view(np.uint32)


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def rows_of(rp, col, val, rows):
    """Rows `rows` of a CSR (numpy), as a new CSR."""
    lens = rp[rows + 1] - rp[rows]
    nrp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    idx = np.repeat(rp[rows] - nrp[:-1], lens) + np.arange(nrp[-1])
    return nrp, col[idx], val[idx]


def rel_l2(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def small_all(gpu_lib, oracle):
    """The small workload's matrix over all channels, from the library and
    from the oracle, and its measurement."""
    from epetreco_gb300.phantom import measurement
    cfg = config("small")
    p = cfg["problem"]
    allrows = np.arange(p.nchannels, dtype=np.int32)
    A = api.systemMatrixCalculation(p, dev(allrows))
    trig = api.trig_table(p).cpu().numpy()
    rnd = api.dump_uniforms(p, dev(allrows)).cpu().numpy()
    orp, ocol, oval = oracle.sm_build_csr(p, allrows, p.nrays, rnd, exact=True, trig=trig)
    rows, y, _ = measurement(p, cfg["counts"])
    return dict(p=p, cfg=cfg, A=A, orp=orp, ocol=ocol, oval=oval, rows=rows, y=y)


def test_small_workload_whole_matrix_bit_exact(small_all):
    d = small_all
    A = d["A"]
    assert A.m == 228_488
    assert (A.row_ptr.cpu().numpy() == d["orp"]).all()
    assert (A.col.cpu().numpy() == d["ocol"]).all()
    assert (bits(A.val.cpu().numpy()) == bits(d["oval"])).all()
    assert A.nnz > 30_000_000  # every channel's non-zeros, not a sample


def test_small_workload_sensitivity_all_channels(small_all, oracle):
    d = small_all
    p = d["p"]
    s, s64 = api.sensitivity(p, return_f64=True)
    ones = np.ones(p.nchannels)
    so = oracle.csrmv_f64(1, d["orp"], d["ocol"], d["oval"], ones, p.nvoxels)
    got = s64.cpu().numpy()
    assert np.abs(got - so).max() <= 1e-12 * np.abs(so).max() + 1e-300
    assert rel_l2(s.cpu().numpy(), so / so.sum()) <= 1e-6


@pytest.mark.parametrize("matrix_free", [False, True])
def test_small_workload_mlem_vs_fp64_oracle(small_all, oracle, matrix_free):
    """The workload as stated (all channels measured at 1e6 counts, measured
    rows = counts > 0, 5 iterations from a uniform image) against the FP64
    oracle's MLEM (reco.cu:209-281) on the oracle's own matrix."""
    d = small_all
    p, rows, y = d["p"], d["rows"], d["y"]
    nit = d["cfg"]["iterations"]
    s = api.sensitivity(p)
    R = api.Mlem(p, rows, y, s, matrix_free=matrix_free)
    R.iterate(nit)
    x = R.image().cpu().numpy()
    r = rows.cpu().numpy()
    rp, col, val = rows_of(d["orp"], d["ocol"], d["oval"], r)
    s_o = oracle.csrmv_f64(1, d["orp"], d["ocol"], d["oval"], np.ones(p.nchannels), p.nvoxels)
    x0 = np.full(p.nvoxels, 1.0 / p.nvoxels)
    x64 = oracle.mlem_f64(rp, col, val, y.cpu().numpy().astype(np.float64), s_o / s_o.sum(), x0,
                          nit, p.nvoxels)
    err = rel_l2(x, x64)
    assert err <= 1e-4, err
    assert abs(x.astype(np.float64).sum() - 1.0) < 1e-5
    assert len(r) > 100_000


def test_small_workload_matrix_free_equals_stored(small_all):
    """The reference's schedule (chords recomputed every iteration) and the
    stored matrix give the same images up to fp32 summation order."""
    d = small_all
    p, rows, y = d["p"], d["rows"], d["y"]
    s = api.sensitivity(p)
    a = api.Mlem(p, rows, y, s)
    b = api.Mlem(p, rows, y, s, matrix_free=True)
    la = a.iterate(5, loglik=True)
    lb = b.iterate(5, loglik=True)
    assert rel_l2(b.image().cpu().numpy(), a.image().cpu().numpy()) <= 1e-5
    assert abs(la - lb) <= 1e-6 * abs(la)


def test_matrix_free_pass_is_forward_then_transpose(small_all):
    """epet_project_mlem: A x bit-equal to the matrix-free forward
    projection, and c = A^T (y / A x) against the stored transpose."""
    d = small_all
    p = d["p"]
    rows = d["rows"][:20000].contiguous()
    y = d["y"][:20000].contiguous()
    x = torch.rand(p.nvoxels, device="cuda", generator=torch.Generator(device="cuda").manual_seed(1))
    c64, ybar = api.project_mlem(p, rows, x, y)
    assert torch.equal(ybar, api.project_forward(p, rows, x))
    A = api.systemMatrixCalculation(p, rows)
    e = torch.where(ybar > 0, y / ybar, torch.zeros_like(ybar))
    c = api.CSRmv(1, A, e, At=api.csr_to_csc(A))
    assert torch.allclose(c64.float(), c, rtol=1e-5, atol=1e-30)


def axis_parallel_rows(p, chunk=1 << 18):
    """Channels with a ray whose end points share a coordinate on one axis
    (not all three): the walk hands those rows to the per-candidate path."""
    out = []
    for c0 in range(0, p.nchannels, chunk):
        rows = torch.arange(c0, min(p.nchannels, c0 + chunk), dtype=torch.int32, device="cuda")
        r = api.rays(p, rows)
        eq = r[..., 0:3] == r[..., 3:6]
        n = eq.sum(-1)
        hit = ((n >= 1) & (n <= 2)).any(-1)
        out.append(rows[hit].cpu().numpy())
        del r, eq, n, hit
    return np.concatenate(out).astype(np.int32)


def test_full_workload_rows_at_default_capacity(gpu_lib, oracle):
    """Rows of the full workload built at the library's own window capacity
    (no artificial one): random rows (about 1 % of which the walk redoes with
    their exact window), the first and last channels, and every row with an
    axis-parallel ray; pattern and values bit-exact against the oracle, and
    within 1e-5 of the reference's sequential fp32 order."""
    p = config("full")["problem"]
    ex = axis_parallel_rows(p)
    assert len(ex) > 0
    rng = np.random.default_rng(2026)
    rows = np.unique(np.concatenate([rng.choice(p.nchannels, 3000, replace=False), ex,
                                     [0, 1, p.nchannels - 2, p.nchannels - 1]])).astype(np.int32)
    c0 = api.build_counters()
    A = api.systemMatrixCalculation(p, dev(rows))
    c1 = api.build_counters()
    # the sizing pass and the filling pass each walk every row once
    assert c1["exact_rows"] - c0["exact_rows"] == 2 * len(ex)
    assert c1["overflow_rows"] - c0["overflow_rows"] >= 2 * 5
    trig = api.trig_table(p).cpu().numpy()
    rnd = api.dump_uniforms(p, dev(rows)).cpu().numpy()
    rp, col, val = (t.cpu().numpy() for t in (A.row_ptr, A.col, A.val))
    orp, ocol, oval = oracle.sm_build_csr(p, rows, p.nrays, rnd, exact=True, trig=trig)
    assert (rp == orp).all()
    assert (col == ocol).all()
    assert (bits(val) == bits(oval)).all()
    srp, scol, sval = oracle.sm_build_csr(p, rows, p.nrays, rnd, exact=False, trig=trig)
    assert (srp == rp).all() and (scol == col).all()
    rel = np.abs(val.astype(np.float64) - sval) / np.abs(sval)
    assert rel.max() <= 1e-5, rel.max()
