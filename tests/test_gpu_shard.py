"""Row-sharded reconstruction kernels on one GPU: correction + update equals
one iteration bit for bit, and shards of the measured rows whose correction
images are summed between the two steps (what the all-reduce does across
GPUs) reproduce the single reconstruction.  Shards run one after another on
the one GPU; nothing waits on another rank."""
import numpy as np
import pytest
import torch

from epetreco_gb300 import api
from epetreco_gb300.problem import config
from epetreco_gb300.shard import partition, row_weights

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def recon(gpu_lib):
    from epetreco_gb300.phantom import measurement
    cfg = config("small")
    p = cfg["problem"]
    rows, y, _ = measurement(p, cfg["counts"])
    keep = torch.arange(0, rows.numel(), 3, device="cuda")  # a third of the measured rows
    rows, y = rows[keep].contiguous(), y[keep].contiguous()
    return p, rows, y, api.sensitivity(p)


@pytest.mark.parametrize("opts", [dict(), dict(value_format=api.BF16), dict(matrix_free=True)],
                         ids=["fp32", "bf16", "matrix_free"])
def test_correction_then_update_is_one_iteration(recon, opts):
    p, rows, y, s = recon
    a = api.Mlem(p, rows, y, s, use_graph=False, **opts)
    b = api.Mlem(p, rows, y, s, use_graph=False, **opts)
    for _ in range(3):
        a.iterate(1)
        b.update(b.correction())
        if opts.get("matrix_free"):
            # fp64 atomics in a different order may round c differently in
            # a rare voxel
            assert torch.allclose(a.image(), b.image(), rtol=1e-6, atol=0)
        else:
            assert torch.equal(a.image(), b.image())
    la, lb = a.iterate(0, loglik=True), b.loglik()
    assert abs(la - lb) <= (1e-9 * abs(la) if opts.get("matrix_free") else 0.0)


@pytest.mark.parametrize("nshards", [2, 3])
def test_shards_sum_to_the_single_reconstruction(recon, nshards):
    p, rows, y, s = recon
    w = row_weights(p, rows)
    assert w.numel() == rows.numel() and (w > 0).all()
    ranges = partition(w.cpu().numpy(), nshards)
    loads = [int(w[b:e].sum()) for b, e in ranges]
    assert max(loads) - min(loads) <= 2 * int(w.max())
    shards = [api.Mlem(p, rows[b:e].contiguous(), y[b:e].contiguous(), s) for b, e in ranges]
    full = api.Mlem(p, rows, y, s)
    for _ in range(5):
        c = torch.zeros(p.nvoxels, device="cuda")
        for sh in shards:
            c += sh.correction()
        for sh in shards:
            sh.update(c)
    full.iterate(5)
    xs = [sh.image() for sh in shards]
    assert all(torch.equal(xs[0], x) for x in xs[1:])  # the same update on every shard
    x, xf = xs[0].double(), full.image().double()
    assert float((x - xf).norm() / xf.norm()) <= 1e-6
    ll = sum(sh.loglik() for sh in shards)
    assert abs(ll - full.iterate(0, loglik=True)) <= 1e-6 * abs(ll)
