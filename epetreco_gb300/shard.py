"""Row-sharded reconstruction: one MLEM problem spread over several ranks.

The reference deals its row chunks to the MPI ranks round-robin, each rank
back-projects its chunks into its own correction image c, the ranks sum c
with MPI_Allreduce and every rank applies the same update (reco.cu:216-260).
Here each rank owns one contiguous range of the measured-row list, balanced
by the chord walk's work (grid cells crossed by the rows' rays, which the
rows' non-zeros follow), holds that range's matrix in a reconstruction
object, and an iteration is

    c = A_rank^T (y / A_rank x)    (epet_mlem_correction, on the rank's GPU)
    c = sum over ranks of c        (torch.distributed all_reduce: NCCL for
                                    CUDA tensors, gloo on the host)
    x = x*c/s, x /= sum(x)         (epet_mlem_update, identical on every rank)

so every rank keeps the same image.  The collective is the path's only
exchange: V floats per iteration (0.56 MB at 52^3 voxels).
"""
from __future__ import annotations

import numpy as np
import torch


def partition(weights, world: int) -> list[tuple[int, int]]:
    """Contiguous ranges [begin, end) of a list whose weights sum to about
    the same per range (range k ends where the running sum first reaches
    k/world of the total)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    w = np.asarray(weights, np.float64)
    if (w < 0).any():
        raise ValueError("weights must be non-negative")
    pre = np.concatenate([[0.0], np.cumsum(w)])
    total = pre[-1]
    cuts = [0]
    for k in range(1, world):
        b = int(np.searchsorted(pre, total * k / world, side="left"))
        cuts.append(min(max(b, cuts[-1]), len(w)))
    cuts.append(len(w))
    return [(cuts[k], cuts[k + 1]) for k in range(world)]


def row_weights(p, rows: torch.Tensor) -> torch.Tensor:
    """Per-row work of the chord walk: grid cells crossed by each listed
    channel's rays (epet_ray_steps)."""
    from . import api
    _, w = api.ray_steps(p, rows, per_row=True)
    return w


class ShardedMlem:
    """One reconstruction whose measured rows are split over the ranks of a
    torch.distributed process group.

    ``local`` builds the rank's reconstruction from (p, rows, y, s); it
    defaults to ``api.Mlem`` with ``opts``.  Any object with ``correction``,
    ``update``, ``loglik`` and ``image`` methods over torch tensors serves
    (the host-side tests use one that computes on the CPU)."""

    def __init__(self, p, rows, y, s, group=None, weights=None, local=None, **opts):
        import torch.distributed as dist
        self.dist, self.group = dist, group
        self.rank = dist.get_rank(group)
        self.world = dist.get_world_size(group)
        if weights is None:
            weights = row_weights(p, rows)
        w = weights.cpu().numpy() if isinstance(weights, torch.Tensor) else np.asarray(weights)
        self.ranges = partition(w, self.world)
        b, e = self.ranges[self.rank]
        if local is None:
            from . import api

            def local(p_, r_, y_, s_):
                return api.Mlem(p_, r_, y_, s_, **opts)
        self.local = local(p, rows[b:e].contiguous(), y[b:e].contiguous(), s)
        self.c = None

    def iterate(self, nit: int) -> None:
        for _ in range(nit):
            self.c = self.local.correction(self.c)
            self.dist.all_reduce(self.c, op=self.dist.ReduceOp.SUM, group=self.group)
            self.local.update(self.c)

    def loglik(self) -> float:
        """Poisson log-likelihood of the last forward projection, summed over
        the ranks."""
        dev = self.c.device if self.c is not None else "cpu"
        t = torch.tensor([self.local.loglik()], dtype=torch.float64, device=dev)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM, group=self.group)
        return float(t.item())

    def image(self) -> torch.Tensor:
        return self.local.image()

    def close(self) -> None:
        close = getattr(self.local, "close", None)
        if close is not None:
            close()
