"""Row-sharded reconstruction on the host: the partition of the measured
rows and the exchange protocol of ShardedMlem (correction over the rank's
rows, all-reduce of c, identical update on every rank), run on two gloo
ranks on the CPU.  The rank-local reconstruction here computes in numpy
(FP64); on a GPU it is the library's reconstruction object and the
all-reduce runs over NCCL (tests/test_gpu_shard.py checks the kernels)."""
import os
import socket
import sys

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from epetreco_gb300.shard import partition  # noqa: E402


def synthetic(seed=3, m=400, V=300):
    """A seeded sparse system matrix with rows of uneven length, counts and a
    sensitivity with some zero voxels."""
    rng = np.random.default_rng(seed)
    lens = rng.integers(0, 40, m)
    rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    col = np.concatenate([np.sort(rng.choice(V, k, replace=False)) for k in lens]).astype(np.int64)
    val = rng.random(col.size)
    y = rng.poisson(20, m).astype(np.float64)
    s = np.bincount(col, val, V)
    return rp, col, val, y, s


class HostRecon:
    """MLEM over rows of the synthetic matrix (reco.cu:209-281), FP64."""

    def __init__(self, A, rows, y, s):
        rp, col, val = A
        rows = rows.numpy()
        self.V = s.numel()
        self.lens = rp[rows + 1] - rp[rows]
        idx = np.concatenate([np.arange(rp[r], rp[r + 1]) for r in rows] or [np.zeros(0, int)])
        self.col, self.val = col[idx], val[idx]
        self.rowid = np.repeat(np.arange(len(rows)), self.lens)
        self.y = y.numpy()
        sn = s.numpy()
        self.s = np.where(sn == 0, 1.0, sn / sn.sum())
        self.x = np.full(self.V, 1.0 / self.V)
        self.yb = None

    def correction(self, c=None):
        self.yb = np.bincount(self.rowid, self.val * self.x[self.col], len(self.y))
        e = np.where(self.yb > 0, self.y / np.where(self.yb > 0, self.yb, 1), 0.0)
        return torch.from_numpy(np.bincount(self.col, self.val * e[self.rowid], self.V))

    def update(self, c):
        self.x = self.x * c.numpy() / self.s
        self.x = self.x / self.x.sum()

    def loglik(self):
        k = self.yb > 0
        return float((self.y[k] * np.log(self.yb[k]) - self.yb[k]).sum())

    def image(self):
        return torch.from_numpy(self.x.copy())


def single_process(nit):
    rp, col, val, y, s = synthetic()
    R = HostRecon((rp, col, val), torch.arange(len(y)), torch.from_numpy(y), torch.from_numpy(s))
    for _ in range(nit):
        R.update(R.correction())
    R.correction()
    return R.x, R.loglik()


def _free_port() -> int:
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        return so.getsockname()[1]


def _worker(rank, world, port, nit, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    from epetreco_gb300.shard import ShardedMlem
    rp, col, val, y, s = synthetic()
    weights = np.diff(rp).astype(np.float64) + 1.0
    S = ShardedMlem(None, torch.arange(len(y)), torch.from_numpy(y), torch.from_numpy(s),
                    weights=weights, local=lambda p, r, yy, ss: HostRecon((rp, col, val), r, yy, ss))
    S.iterate(nit)
    x = S.image().numpy()
    S.local.correction()  # forward projection of the final image (for the likelihood)
    ll = S.loglik()
    q.put((rank, S.ranges, x, ll))
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_mlem_equals_single_process(world):
    nit = 6
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, nit, q)) for r in range(world)]
    for pr in procs:
        pr.start()
    out = sorted(q.get(timeout=180) for _ in procs)
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    x1, ll1 = single_process(nit)
    ranges = out[0][1]
    assert ranges[0][0] == 0 and ranges[-1][1] == 400
    assert all(a[1] == b[0] for a, b in zip(ranges, ranges[1:]))
    assert all(e > b for b, e in ranges)  # every rank holds rows
    for rank, rg, x, ll in out:
        assert rg == ranges
        assert np.array_equal(x, out[0][2])       # every rank keeps the same image
        assert np.linalg.norm(x - x1) / np.linalg.norm(x1) <= 1e-12
        assert abs(ll - ll1) <= 1e-9 * abs(ll1)


def test_partition_balances_contiguous_ranges():
    rng = np.random.default_rng(0)
    w = rng.integers(300, 600, 10_000).astype(float)
    for world in (1, 2, 3, 8):
        rg = partition(w, world)
        assert rg[0][0] == 0 and rg[-1][1] == len(w) and len(rg) == world
        assert all(a[1] == b[0] for a, b in zip(rg, rg[1:]))
        sums = [w[b:e].sum() for b, e in rg]
        assert max(sums) - min(sums) <= 2 * w.max()


def test_partition_edge_cases():
    assert partition([], 3) == [(0, 0), (0, 0), (0, 0)]
    assert partition([5.0], 2) in ([(0, 0), (0, 1)], [(0, 1), (1, 1)])
    assert partition([0.0, 0.0, 0.0], 2)[-1][1] == 3
    with pytest.raises(ValueError):
        partition([1.0, -1.0], 2)
    with pytest.raises(ValueError):
        partition([1.0], 0)
