"""Parity of the CUDA library with the oracle (a CPU restatement pinned to
the reference's own code).  Integer and index results must be bit-exact;
float results are compared bit-exactly where the arithmetic is defined to be
the same, else within the tolerance stated in each test.

The oracle receives the two inputs whose float values depend on the device:
the per-angle sin/cos table and the cuRAND uniforms (both dumped from the
library), so geometry, candidates and chord lengths can be compared bit for
bit."""
import numpy as np
import pytest
import torch

from epetreco_gb300 import api
from epetreco_gb300.problem import Problem, config, centred_grid, two_head_setup

pytestmark = pytest.mark.gpu


def bits(a):
    return np.asarray(a, np.float32).view(np.uint32)


def sample_rows(p: Problem, n: int, seed: int) -> np.ndarray:
    """Rows spread over all angles, plus the 90-degree (z-running) lines and
    the most oblique crystal pairs."""
    rng = np.random.default_rng(seed)
    per = p.nchannels // p.setup.na
    a90 = int(round(90.0 / p.setup.da)) % p.setup.na
    rows = set(rng.choice(p.nchannels, n, replace=False).tolist())
    rows |= {a90 * per, a90 * per + per - 1, 0, per - 1, p.nchannels - 1}
    rows |= {a90 * per + int(k) for k in rng.integers(0, per, 6)}
    return np.array(sorted(rows), np.int32)


def dev(a, dt=None):
    t = torch.from_numpy(np.ascontiguousarray(a))
    return (t.to(dt) if dt is not None else t).cuda()


@pytest.fixture(scope="module", params=["small", "full"])
def case(request, gpu_lib, oracle):
    p = config(request.param)["problem"]
    rows = sample_rows(p, 40 if request.param == "full" else 60, 17)
    trig = api.trig_table(p).cpu().numpy()
    rnd = api.dump_uniforms(p, dev(rows)).cpu().numpy()
    return dict(name=request.param, p=p, rows=rows, trig=trig, rnd=rnd)


def test_trig_table_close_to_host(case, oracle):
    host = oracle.trig_table(case["p"])
    ulps = np.abs(bits(case["trig"]).astype(np.int64) - bits(host).astype(np.int64))
    assert ulps.max() <= 2  # CUDA sinf/cosf: <= 2 ulp (documented bound)


def test_uniforms_in_unit_interval(case):
    u = case["rnd"]
    assert (u > 0).all() and (u <= 1).all()
    assert abs(u.mean() - 0.5) < 0.02


def test_rays_bit_exact(case, oracle):
    p, rows = case["p"], case["rows"]
    got = api.rays(p, dev(rows)).cpu().numpy()
    for i in range(0, len(rows), 7):
        want = oracle.rays(p, rows[i], case["rnd"][i], trig=case["trig"])
        assert (bits(got[i]) == bits(want)).all()


def test_workqueue_bit_exact(case, oracle):
    p, rows = case["p"], case["rows"]
    cnl, vxl, off = api.getWorkqueue(p, dev(rows))
    oc, ov, cnt = oracle.workqueue(p, rows, trig=case["trig"])
    assert cnl.numel() == len(oc)
    assert (cnl.cpu().numpy() == oc).all() and (vxl.cpu().numpy() == ov).all()
    assert (np.diff(off.cpu().numpy()) == cnt).all()


def test_values_bit_exact_reference_order(case, oracle):
    """getSystemMatrixFromWorkqueue semantics: fp32 sum in ray order."""
    p, rows = case["p"], case["rows"][:12]
    cnl, vxl, off = api.getWorkqueue(p, dev(rows))
    val = api.getSystemMatrixFromWorkqueue(p, dev(rows), off, vxl).cpu().numpy()
    row_of = np.searchsorted(rows, cnl.cpu().numpy()).astype(np.int32)
    want = oracle.sm_values_wq(p, rows, p.nrays, case["rnd"][:12], row_of, vxl.cpu().numpy(),
                               exact=False, trig=case["trig"])
    assert (bits(val) == bits(want)).all()
    assert (val > 0).mean() > 0.01


def test_sm_build_matches_oracle(case, oracle):
    """Fused build: non-zero pattern bit-exact; values bit-exact against the
    oracle's exact-sum mode and within (nrays-1)*2^-24 relative (1e-5) of the
    reference's sequential fp32 sum."""
    p, rows = case["p"], case["rows"]
    A = api.systemMatrixCalculation(p, dev(rows))
    rp, col, val = (t.cpu().numpy() for t in (A.row_ptr, A.col, A.val))
    orp, ocol, oval = oracle.sm_build_csr(p, rows, p.nrays, case["rnd"], exact=True,
                                          trig=case["trig"])
    assert (rp == orp).all()
    assert (col == ocol).all()
    assert (bits(val) == bits(oval)).all()
    srp, scol, sval = oracle.sm_build_csr(p, rows, p.nrays, case["rnd"], exact=False,
                                          trig=case["trig"])
    assert (srp == rp).all() and (scol == col).all()
    rel = np.abs(val.astype(np.float64) - sval) / np.abs(sval)
    assert rel.max() <= 1e-5, rel.max()
    # rows are sorted by voxel id
    for i in range(len(rows)):
        seg = col[rp[i]:rp[i + 1]]
        assert (np.diff(seg) > 0).all()


def test_sm_build_pattern_is_nonzero_workqueue(case):
    """The fused build keeps exactly the candidates whose value is non-zero."""
    p, rows = case["p"], case["rows"][:10]
    A = api.systemMatrixCalculation(p, dev(rows))
    cnl, vxl, off = api.getWorkqueue(p, dev(rows))
    val = api.getSystemMatrixFromWorkqueue(p, dev(rows), off, vxl)
    keep = (val != 0).cpu().numpy()
    assert (A.col.cpu().numpy() == vxl.cpu().numpy()[keep]).all()


def test_matrix_free_projections(case):
    p, rows = case["p"], case["rows"]
    A = api.systemMatrixCalculation(p, dev(rows))
    At = api.csr_to_csc(A)
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.rand(p.nvoxels, device="cuda", generator=g)
    y_mf = api.project_forward(p, dev(rows), x)
    y = api.CSRmv(api.NON_TRANSPOSE, A, x)
    assert torch.allclose(y_mf, y, rtol=2e-6, atol=0)
    e = torch.rand(len(rows), device="cuda", generator=g)
    c_mf = api.project_back(p, dev(rows), e)
    c = api.CSRmv(api.TRANSPOSE, A, e, At=At)
    assert torch.allclose(c_mf, c, rtol=2e-5, atol=1e-12)


def test_spmv_against_oracle(case, oracle):
    """y = A x and c = A^T e: fp32 accumulation vs the oracle's fp64-rounded
    result, relative 1e-5; both transpose paths (column-major copy, atomics)."""
    p, rows = case["p"], case["rows"]
    A = api.systemMatrixCalculation(p, dev(rows))
    At = api.csr_to_csc(A)
    rp, col, val = (t.cpu().numpy() for t in (A.row_ptr, A.col, A.val))
    rng = np.random.default_rng(5)
    x = rng.random(p.nvoxels).astype(np.float32)
    e = rng.random(len(rows)).astype(np.float32)
    y = api.CSRmv(0, A, dev(x)).cpu().numpy()
    yo = oracle.csrmv(0, rp, col, val, x, p.nvoxels)
    assert np.allclose(y, yo, rtol=1e-5, atol=0)
    c1 = api.CSRmv(1, A, dev(e), At=At).cpu().numpy()
    c2 = api.CSRmv(1, A, dev(e)).cpu().numpy()
    co = oracle.csrmv(1, rp, col, val, e, p.nvoxels)
    assert np.allclose(c1, co, rtol=1e-5, atol=1e-30)
    assert np.allclose(c2, co, rtol=1e-5, atol=1e-30)
    # alpha / beta
    y0 = rng.random(len(rows)).astype(np.float32)
    y2 = api.CSRmv(0, A, dev(x), alpha=2.0, beta=0.5, y=dev(y0)).cpu().numpy()
    assert np.allclose(y2, 2 * yo + 0.5 * y0, rtol=1e-5)


def test_csc_is_stable_transpose(case):
    p, rows = case["p"], case["rows"]
    A = api.systemMatrixCalculation(p, dev(rows))
    At = api.csr_to_csc(A)
    rp, col, val = (t.cpu().numpy() for t in (A.row_ptr, A.col, A.val))
    r = np.repeat(np.arange(len(rows)), np.diff(rp))
    order = np.lexsort((r, col))
    cp = np.zeros(p.nvoxels + 1, np.int64)
    np.add.at(cp, col + 1, 1)
    assert (At.col_ptr.cpu().numpy() == np.cumsum(cp)).all()
    assert (At.row.cpu().numpy() == r[order]).all()
    assert (bits(At.val.cpu().numpy()) == bits(val[order])).all()


def test_walk_division_is_correctly_rounded(gpu_lib):
    """The walk divides by a per-ray reciprocal (Markstein's correction);
    it must agree bit for bit with the IEEE division on the device."""
    import ctypes as C
    from epetreco_gb300._lib import check, lib
    bad = C.c_int64(-1)
    check(lib().epet_selftest_division(1 << 26, 20260512, C.byref(bad),
                                       C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    assert bad.value == 0


def test_rays_every_row_any_order(gpu_lib, oracle):
    """Rays of consecutive, gapped, repeated and descending channel lists:
    the generator of each row must be curand_init(seed, channel, 0), however
    the rays kernel reaches it."""
    p = config("small")["problem"]
    rng = np.random.default_rng(5)
    rows = np.concatenate([np.arange(1000, 1300), np.sort(rng.choice(p.nchannels, 200, False)),
                           [77, 77, 76, 3, 200000, 9]]).astype(np.int32)
    trig = api.trig_table(p).cpu().numpy()
    rnd = api.dump_uniforms(p, dev(rows)).cpu().numpy()
    got = api.rays(p, dev(rows)).cpu().numpy()
    for i in range(len(rows)):
        want = oracle.rays(p, rows[i], rnd[i], trig=trig)
        assert (bits(got[i]) == bits(want)).all(), i


def test_windows_over_capacity_are_redone(case):
    """With a window capacity (600 cells) below the channels' windows but
    above their non-zeros, nearly every row is measured again and rebuilt in
    the second launch with its exact window: the matrix must equal the
    default build bit for bit, and the matrix-free projections through the
    same path must agree."""
    p, rows = case["p"], case["rows"]
    cap = 600
    A = api.systemMatrixCalculation(p, dev(rows))
    c0 = api.build_counters()
    B = api.systemMatrixCalculation(p, dev(rows), max_row_nnz=cap)
    c1 = api.build_counters()
    # the sizing pass and the filling pass each redo the rows over capacity
    assert c1["overflow_rows"] - c0["overflow_rows"] >= len(rows) // 2
    assert torch.equal(A.row_ptr, B.row_ptr)
    assert torch.equal(A.col, B.col)
    assert torch.equal(A.val, B.val)
    x = torch.rand(p.nvoxels, device="cuda")
    y0 = api.project_forward(p, dev(rows), x)
    y1 = api.project_forward(p, dev(rows), x, max_row_nnz=cap)
    assert torch.equal(y0, y1)


def test_ray_steps_counts_cells_crossed(case):
    """epet_ray_steps (the walk's work measure): cells crossed per ray, from
    the entry and exit cells of each ray's grid interval (numpy, float64);
    rays that only graze a plane may count differently by one."""
    p, rows = case["p"], case["rows"]
    got = api.ray_steps(p, dev(rows))
    r = api.rays(p, dev(rows)).cpu().numpy().reshape(-1, 6).astype(np.float64)
    o = np.array(p.grid.origin, np.float64)
    d = np.array(p.grid.pitch, np.float64)
    n = np.array(p.grid.n)
    p0, dp = r[:, :3], r[:, 3:] - r[:, :3]
    with np.errstate(divide="ignore", invalid="ignore"):
        t0 = (o - p0) / dp
        t1 = (o + n * d - p0) / dp
    a_in = np.maximum(0, np.nanmax(np.minimum(t0, t1), axis=1))
    a_out = np.minimum(1, np.nanmin(np.maximum(t0, t1), axis=1))
    hit = a_in < a_out
    span = a_out - a_in
    c_in = np.clip(np.floor((p0 + (a_in + 1e-6 * span)[:, None] * dp - o) / d), 0, n - 1)
    c_out = np.clip(np.floor((p0 + (a_out - 1e-6 * span)[:, None] * dp - o) / d), 0, n - 1)
    want = int((1 + np.abs(c_out - c_in).sum(1))[hit].sum())
    assert abs(got - want) <= 1e-3 * want, (got, want)
    assert want > len(rows) * p.nrays  # every ray crosses several cells
