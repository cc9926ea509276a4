"""Differentiable projector: the system matrix as a torch autograd operator.

``Projector(p, rows)`` wraps the libtorch C++ ``torch::autograd::Function``s of
``csrc/autograd.cpp``: forward y = A x, backward A^T g -- computed by
libepet_gb300.  ``mode="stored"`` keeps the CSR and its column-major copy
(scatter-free transpose); ``mode="free"`` stores nothing and recomputes the
chords in every pass, for when the matrix does not fit.  ``x`` may carry
leading batch dimensions.

``poisson_nll`` and ``reconstruct`` give gradient-based Poisson-likelihood
reconstruction on top of it.
"""
from __future__ import annotations

import importlib

import torch

from . import api
from .problem import Problem


def _ext():
    try:
        return importlib.import_module("epetreco_gb300._autograd")
    except ImportError as e:  # the extension is part of the build
        raise RuntimeError("epetreco_gb300._autograd is not built: run "
                           "`python -m epetreco_gb300.build`") from e


def problem_vector(p: Problem) -> list:
    """The problem's float and int32 fields (exact in float64); the 64-bit
    seed travels as its own integer argument."""
    s, g = p.setup, p.grid
    return [float(v) for v in (s.pos0x, s.pos1x, s.na, s.n0z, s.n0y, s.n1z, s.n1y, s.da,
                               s.segx, s.segy, s.segz, *g.origin, *g.pitch, *g.n, p.nrays,
                               p.ray_mode)]


class Projector:
    def __init__(self, p: Problem, rows: torch.Tensor, mode: str = "stored"):
        if mode not in ("stored", "free"):
            raise ValueError("mode must be 'stored' or 'free'")
        self.p, self.mode = p, mode
        self.rows = rows.to(torch.int32).contiguous().cuda()
        self.ext = _ext()
        if mode == "stored":
            self.A = api.systemMatrixCalculation(p, self.rows)
            self.At = api.csr_to_csc(self.A)
        else:
            self.pvec = problem_vector(p)

    @property
    def shape(self):
        return (self.rows.numel(), self.p.nvoxels)

    def __call__(self, x: torch.Tensor) -> torch.Tensor:
        if self.mode == "stored":
            A, At = self.A, self.At
            return self.ext.project_stored(x, A.row_ptr, A.col.contiguous(), A.val.contiguous(),
                                           At.col_ptr, At.row.contiguous(),
                                           At.val.contiguous(), A.n)
        # the seed as a signed 64-bit value with the same bits (libtorch ints are int64)
        seed = int(self.p.seed) & (2**64 - 1)
        seed = seed - 2**64 if seed >= 2**63 else seed
        return self.ext.project_free(x, self.rows, self.pvec, seed)


def poisson_nll(ybar: torch.Tensor, y: torch.Tensor, eps: float = 1e-12) -> torch.Tensor:
    """sum ybar - y log(ybar) (the negative Poisson log-likelihood up to a
    constant), over the last dimension, summed over the batch."""
    return (ybar - y * torch.log(ybar.clamp_min(eps))).sum()


def reconstruct(proj: Projector, y: torch.Tensor, iters: int = 50, lr: float = 0.05,
                x0: torch.Tensor | None = None):
    """Gradient-based Poisson-likelihood reconstruction: x = exp(theta) (keeps
    the image positive), Adam on theta.  Returns (x, losses)."""
    V = proj.p.nvoxels
    if x0 is None:
        # the constant image whose projection has the measured total
        ones = torch.ones(V, device=y.device)
        a1 = float(proj(ones).sum())
        x0 = torch.full(y.shape[:-1] + (V,), float(y.sum(-1).mean()) / max(a1, 1e-30),
                        device=y.device)
    theta = torch.log(x0.clamp_min(1e-12)).clone().requires_grad_(True)
    opt = torch.optim.Adam([theta], lr=lr)
    losses = []
    for _ in range(iters):
        opt.zero_grad()
        loss = poisson_nll(proj(torch.exp(theta)), y)
        loss.backward()
        opt.step()
        losses.append(float(loss.detach()))
    return torch.exp(theta).detach(), losses
