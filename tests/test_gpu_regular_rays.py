"""Regular rays (ReguRayGen, RayGenerators.hpp:46-66): all six box
coordinates of every ray are 0.5, so each ray joins the centres of the
channel's two crystals.  The oracle needs no uniforms dumped from the device
here, only the per-angle sin/cos table; the bars are those of the random
generator: rays and the non-zero pattern bit-exact, values bit-exact against
the oracle's exact-sum mode and within (nrays-1)*2^-24 relative of the
reference's sequential fp32 sum."""
from dataclasses import replace

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


@pytest.fixture(scope="module", params=["small", "full"])
def case(request, gpu_lib):
    p = config(request.param)["problem"].with_rays("regular")
    rng = np.random.default_rng(29)
    per = p.nchannels // p.setup.na
    a90 = int(round(90.0 / p.setup.da)) % p.setup.na
    rows = set(rng.choice(p.nchannels, 40, replace=False).tolist())
    rows |= {0, per - 1, a90 * per, a90 * per + per - 1, p.nchannels - 1}
    # centre lines with equal end coordinates on an axis (crystals at equal
    # height): the walk leaves these rows to the per-candidate path
    pool = np.sort(rng.choice(p.nchannels, 4000, replace=False)).astype(np.int32)
    r = api.rays(p, dev(pool))[:, 0, :].cpu().numpy()
    par = pool[(r[:, 1] == r[:, 4]) | (r[:, 2] == r[:, 5])]
    rows |= set(par[:8].tolist())
    rows = np.array(sorted(rows), np.int32)
    r = api.rays(p, dev(rows))[:, 0, :].cpu().numpy()
    parallel = (r[:, 1] == r[:, 4]) | (r[:, 2] == r[:, 5])
    trig = api.trig_table(p).cpu().numpy()
    half = np.full((len(rows), p.nrays, 6), 0.5, np.float32)
    return dict(p=p, rows=rows, trig=trig, half=half, parallel=parallel)


def test_uniforms_are_one_half(case):
    u = api.dump_uniforms(case["p"], dev(case["rows"])).cpu().numpy()
    assert (u == np.float32(0.5)).all()


def test_rays_join_crystal_centres(case, oracle):
    p, rows = case["p"], case["rows"]
    got = api.rays(p, dev(rows)).cpu().numpy()
    assert (got == got[:, :1, :]).all()  # every ray of a row is the same line
    for i in range(len(rows)):
        want = oracle.rays(p, rows[i], case["half"][i], trig=case["trig"])
        assert (bits(got[i]) == bits(want)).all()


def test_seed_is_unused(case):
    p, rows = case["p"], dev(case["rows"])
    a = api.rays(p, rows)
    b = api.rays(p.with_seed(7), rows)
    assert torch.equal(a, b)


def test_values_reference_order(case, oracle):
    p, rows = case["p"], case["rows"][:12]
    cnl, vxl, off = api.getWorkqueue(p, dev(rows))
    val = api.getSystemMatrixFromWorkqueue(p, dev(rows), off, vxl).cpu().numpy()
    row_of = np.searchsorted(rows, cnl.cpu().numpy()).astype(np.int32)
    want = oracle.sm_values_wq(p, rows, p.nrays, case["half"][:12], row_of,
                               vxl.cpu().numpy(), exact=False, trig=case["trig"])
    assert (bits(val) == bits(want)).all()
    assert (val > 0).any()


def test_sm_build_matches_oracle(case, oracle):
    p, rows = case["p"], case["rows"]
    A = api.systemMatrixCalculation(p, dev(rows))
    rp, col, val = (t.cpu().numpy() for t in (A.row_ptr, A.col, A.val))
    orp, ocol, oval = oracle.sm_build_csr(p, rows, p.nrays, case["half"], exact=True,
                                          trig=case["trig"])
    assert (rp == orp).all()
    assert (col == ocol).all()
    assert (bits(val) == bits(oval)).all()
    srp, scol, sval = oracle.sm_build_csr(p, rows, p.nrays, case["half"], exact=False,
                                          trig=case["trig"])
    assert (srp == rp).all() and (scol == col).all()
    rel = np.abs(val.astype(np.float64) - sval) / np.abs(sval)
    assert rel.max() <= (p.nrays - 1) * 2.0 ** -24 + 1e-12, rel.max()


def test_one_ray_gives_the_same_matrix(case):
    """nrays identical lines average to the line itself: nrays = 1 keeps the
    pattern, and the values agree up to three fp32 roundings (of the two
    fixed-point sums and of the division by nrays, 2^-22 relative together)
    plus one fixed-point unit of the nrays form (below 1e-15 m)."""
    p, rows = case["p"], dev(case["rows"])
    A = api.systemMatrixCalculation(p, rows)
    B = api.systemMatrixCalculation(replace(p, nrays=1), rows)
    assert torch.equal(A.row_ptr, B.row_ptr) and torch.equal(A.col, B.col)
    a, b = A.val.double(), B.val.double()
    assert ((a - b).abs() <= 2.0 ** -22 * b.abs() + 1e-15).all()


def test_regular_build_differs_from_random(case):
    """The generator reaches the walk: random rays cover the crystals'
    volume, so on the rows whose centre line is not axis-parallel their
    pattern is wider than the centre line's.  (An axis-parallel centre line
    gets a chord in every candidate along that axis, as the reference's slab
    test leaves the axis out, so those rows are longer instead.)"""
    p, rows = case["p"], dev(case["rows"])
    reg = api.systemMatrixCalculation(p, rows)
    rnd = api.systemMatrixCalculation(p.with_rays("random"), rows)
    keep = torch.from_numpy(~case["parallel"]).cuda()
    n_reg = reg.row_ptr.diff()[keep].sum().item()
    n_rnd = rnd.row_ptr.diff()[keep].sum().item()
    assert n_rnd > n_reg
    assert case["parallel"].sum() >= 8


def test_axis_parallel_rows(case, oracle):
    """Rows whose line has equal end coordinates on an axis go through the
    per-candidate path (the reference's slab test leaves that axis out, so
    such a row can be longer than the walk's window), with the fused build's
    exact sums.  With a window capacity of 600 cells nearly every row is also
    redone, and rows found axis-parallel only in the redo must reach the
    output too: the matrix equals the default build and the oracle's, and
    the matrix-free forward projection agrees."""
    p, rows = case["p"], case["rows"]
    c0 = api.build_counters()
    A = api.systemMatrixCalculation(p, dev(rows))
    c1 = api.build_counters()
    assert c1["exact_rows"] - c0["exact_rows"] >= 8
    B = api.systemMatrixCalculation(p, dev(rows), max_row_nnz=600)
    c2 = api.build_counters()
    assert c2["overflow_rows"] - c1["overflow_rows"] >= len(rows) // 2
    assert torch.equal(A.row_ptr, B.row_ptr)
    assert torch.equal(A.col, B.col)
    assert torch.equal(A.val, B.val)
    orp, ocol, oval = oracle.sm_build_csr(p, rows, p.nrays, case["half"], exact=True,
                                          trig=case["trig"])
    assert (B.row_ptr.cpu().numpy() == orp).all()
    assert (B.col.cpu().numpy() == ocol).all()
    assert (bits(B.val.cpu().numpy()) == bits(oval)).all()
    x = torch.rand(p.nvoxels, device="cuda")
    y0 = api.project_forward(p, dev(rows), x)
    y1 = api.project_forward(p, dev(rows), x, max_row_nnz=600)
    assert torch.equal(y0, y1)
