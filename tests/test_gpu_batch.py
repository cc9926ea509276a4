"""Batched reconstructions (one launch per iteration step over all problems,
one CUDA graph per iteration) and the autotuned launch shapes: each
problem's image against the FP64 oracle and against the same problem
reconstructed alone."""
import numpy as np
import pytest
import torch

from epetreco_gb300 import api
from epetreco_gb300.phantom import measurement, phantom_image
from epetreco_gb300.problem import batch_members

pytestmark = pytest.mark.gpu

NIT = 5


@pytest.fixture(scope="module")
def members(gpu_lib):
    ms = batch_members(5, seed=11, grids=(12, 16, 20), angles=(4, 6), rays=(8, 16),
                       counts=(2e4, 2e5))
    out = []
    for b in ms:
        p = b.problem
        x_true = phantom_image(p, b.phantom_seed, b.n_spheres)
        rows, y, _ = measurement(p, b.counts, seed=b.poisson_seed, x_true=x_true)
        s = api.sensitivity(p)
        out.append((p, rows, y, s))
    return out


def oracle_image(oracle, p, rows, y, s, nit):
    A = api.systemMatrixCalculation(p, rows)
    rp, col, val = (t.cpu().numpy() for t in (A.row_ptr, A.col, A.val))
    sn = s.cpu().numpy().astype(np.float64)
    sn /= sn.sum()
    x0 = np.full(p.nvoxels, 1.0 / p.nvoxels)
    return oracle.mlem_f64(rp, col, val, y.cpu().numpy().astype(np.float64), sn, x0, nit,
                           p.nvoxels)


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("autotune", [False, True])
def test_batch_matches_oracle_and_single(members, oracle, autotune):
    B = api.MlemBatch(members, autotune=autotune)
    B.iterate(NIT)
    st = B.stats()
    assert st["nnz"] > 0
    for G, U, grid in st["plan"].values():
        assert G in (4, 8, 16, 32) and U in (0, 1, 2, 4) and grid >= 0
    for i, (p, rows, y, s) in enumerate(members):
        xb = B.image(i).cpu().numpy()
        x64 = oracle_image(oracle, p, rows, y, s, NIT)
        assert rel(xb, x64) <= 1e-4
        R = api.Mlem(p, rows, y, s)
        R.iterate(NIT)
        assert rel(xb, R.image().cpu().numpy()) <= 1e-5


def test_batch_graph_equals_eager(members):
    a = api.MlemBatch(members, use_graph=True, autotune=False)
    b = api.MlemBatch(members, use_graph=False, autotune=False)
    a.iterate(3)
    b.iterate(3)
    for i in range(len(members)):
        assert torch.equal(a.image(i), b.image(i))


def test_batch_loglik_per_problem(members):
    B = api.MlemBatch(members, autotune=False)
    B.iterate(2)
    ll = B.iterate(1, loglik=True)
    for i, (p, rows, y, s) in enumerate(members):
        R = api.Mlem(p, rows, y, s)
        R.iterate(2)
        l1 = R.iterate(1, loglik=True)
        assert abs(ll[i] - l1) <= 1e-6 * abs(l1)


def test_batch_with_an_empty_problem(members):
    """A problem without measured rows keeps the others intact."""
    p0, rows0, y0, s0 = members[0]
    empty = (p0, rows0[:0], y0[:0], s0)
    B = api.MlemBatch([members[1], empty, members[2]], autotune=False)
    B.iterate(2)
    for k, i in ((0, 1), (2, 2)):
        p, rows, y, s = members[i]
        R = api.Mlem(p, rows, y, s)
        R.iterate(2)
        assert rel(B.image(k).cpu().numpy(), R.image().cpu().numpy()) <= 1e-5


def test_autotuned_single_matches_oracle(members, oracle):
    p, rows, y, s = members[-1]
    R = api.Mlem(p, rows, y, s, autotune=True)
    R.iterate(NIT)
    pl = R.plan()
    assert pl["forward"][0] in (4, 8, 16, 32) and pl["transpose"][1] in (0, 1, 2, 4)
    assert rel(R.image().cpu().numpy(), oracle_image(oracle, p, rows, y, s, NIT)) <= 1e-4


def test_batch_member_iterates_alone(members):
    """A member iterated alone runs the plain kernels on the batch's arrays."""
    B = api.MlemBatch(members[:3], autotune=False)
    B.member(1).iterate(NIT)
    p, rows, y, s = members[1]
    R = api.Mlem(p, rows, y, s)
    R.iterate(NIT)
    assert torch.equal(B.image(1), R.image())
    x0 = torch.full((members[0][0].nvoxels,), 1.0 / members[0][0].nvoxels, device="cuda")
    assert torch.equal(B.image(0), x0)
