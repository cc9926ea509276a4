"""The differentiable projector (libtorch C++ autograd Function): forward and
backward against the library's products, the gradient of the Poisson
negative log-likelihood against central finite differences in FP64, batched
phantoms, the matrix-free mode, and gradient-based reconstruction."""
import numpy as np
import pytest
import torch

from epetreco_gb300 import api
from epetreco_gb300.problem import config

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup(gpu_lib):
    from epetreco_gb300.autograd import Projector
    from epetreco_gb300.phantom import phantom_image
    p = config("small")["problem"]
    rng = np.random.default_rng(12)
    rows = torch.from_numpy(np.sort(rng.choice(p.nchannels, 3000, replace=False)).astype(
        np.int32)).cuda()
    proj = Projector(p, rows)
    x4 = torch.stack([torch.from_numpy(phantom_image(p, seed)) for seed in (1, 2, 3, 4)]).cuda()
    return p, rows, proj, x4


def test_forward_backward_are_the_library_products(setup):
    p, rows, proj, x4 = setup
    x = x4[0].clone().requires_grad_(True)
    y = proj(x)
    assert torch.equal(y, api.CSRmv(0, proj.A, x4[0]))
    g = torch.rand_like(y)
    y.backward(g)
    assert torch.equal(x.grad, api.CSRmv(1, proj.A, g, At=proj.At))


def test_batch_of_four(setup):
    p, rows, proj, x4 = setup
    xb = x4.clone().requires_grad_(True)
    yb = proj(xb)
    assert yb.shape == (4, rows.numel())
    for b in range(4):
        assert torch.equal(yb[b], proj(x4[b]))
    yb.sum().backward()
    ones = torch.ones(rows.numel(), device="cuda")
    for b in range(4):
        assert torch.equal(xb.grad[b], api.CSRmv(1, proj.A, ones, At=proj.At))


def test_poisson_gradient_finite_differences(setup):
    """dL/dx_v of L = sum(Ax - y log Ax) by autograd vs central differences
    (h = 1e-3) evaluated in FP64 on the host, on 64 voxels that the rows see."""
    from epetreco_gb300.autograd import poisson_nll
    p, rows, proj, x4 = setup
    x0 = (x4[0] + 0.5).double()
    y = torch.poisson(proj(x0.float()).double() * 20,
                      generator=torch.Generator(device="cuda").manual_seed(3)).float()
    x = x0.float().clone().requires_grad_(True)
    poisson_nll(proj(x), y).backward()
    grad = x.grad.double().cpu().numpy()
    rp, col, val = (t.cpu().numpy() for t in (proj.A.row_ptr, proj.A.col, proj.A.val))
    r = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
    yy = y.double().cpu().numpy()
    xh = x0.cpu().numpy()

    def L(xv):
        ax = np.zeros(len(rp) - 1)
        np.add.at(ax, r, val.astype(np.float64) * xv[col])
        return np.sum(ax - yy * np.log(ax))

    seen = np.unique(col)
    vox = np.random.default_rng(4).choice(seen, 64, replace=False)
    h = 1e-3
    for v in vox:
        xp, xm = xh.copy(), xh.copy()
        xp[v] += h
        xm[v] -= h
        fd = (L(xp) - L(xm)) / (2 * h)
        assert abs(grad[v] - fd) <= 1e-4 * max(1.0, abs(fd)), (v, grad[v], fd)


def test_matrix_free_mode_matches_stored(setup):
    from epetreco_gb300.autograd import Projector
    p, rows, proj, x4 = setup
    free = Projector(p, rows, mode="free")
    xs = x4[1].clone().requires_grad_(True)
    xf = x4[1].clone().requires_grad_(True)
    ys, yf = proj(xs), free(xf)
    assert torch.allclose(ys, yf, rtol=2e-6, atol=0)
    g = torch.rand_like(ys)
    ys.backward(g)
    yf.backward(g)
    assert torch.allclose(xs.grad, xf.grad, rtol=2e-5, atol=1e-9)


def test_gradient_reconstruction_decreases_nll(setup):
    from epetreco_gb300.autograd import reconstruct
    p, rows, proj, x4 = setup
    y = torch.poisson(proj(x4[0]) * 50, generator=torch.Generator(device="cuda").manual_seed(5))
    x, losses = reconstruct(proj, y, iters=30, lr=0.05)
    assert losses[-1] < losses[0]
    assert torch.isfinite(x).all() and (x > 0).all()


def test_matrix_free_keeps_a_64_bit_seed(gpu_lib):
    """A seed above 2^53 (not exact in float64) reaches the matrix-free
    projector unchanged: its forward equals the stored product built with
    the same seed."""
    from epetreco_gb300.autograd import Projector
    p = config("small")["problem"].with_seed(2**63 + 12345)
    rows = torch.arange(20000, 20400, dtype=torch.int32, device="cuda")
    free = Projector(p, rows, mode="free")
    A = api.systemMatrixCalculation(p, rows)
    x = torch.rand(p.nvoxels, device="cuda")
    assert torch.allclose(free(x), api.CSRmv(0, A, x), rtol=2e-6, atol=0)
    B = api.systemMatrixCalculation(p.with_seed(2**63 + 12344), rows)
    assert not torch.equal(A.val, B.val)  # the low bits of the seed matter
