"""Seeded synthetic phantoms and measurements.

The reference reconstructs HDF5 measurements that are not part of its
repository; the workloads here are synthetic: a uniform cylinder (axis = y,
the rotation axis) of activity 1 plus hot spheres of activity 4, scaled to
the grid, forward-projected with an independent ray seed (so the
reconstruction's own matrix does not generate its data), scaled to a total
count and Poisson-sampled.  Measured rows are the channels with y > 0, as the
reference's ``makeSparseVct`` keeps them (wrappers.hpp:271-281).
"""
from __future__ import annotations

import numpy as np
import torch

from . import api
from .problem import Problem

DATA_SEED = 7919  # ray seed of the data-generating projector (not 1251)


def phantom_image(p: Problem, seed: int = 1, n_spheres: int = 3) -> np.ndarray:
    """Cylinder r = 25/32 of the grid half-width (25 mm on the 64 mm grid)
    plus n_spheres hot spheres of radius 4-6 mm scaled likewise."""
    g = p.grid
    rng = np.random.default_rng(seed)
    half = 0.5 * g.n[0] * g.pitch[0]
    scale = half / 0.032
    cx, cy, cz = (g.centres(a).astype(np.float64) for a in range(3))
    X, Y, Z = np.meshgrid(cx, cy, cz, indexing="ij")  # voxel id order: x, y, z
    img = np.zeros(X.shape, np.float64)
    R = 0.025 * scale
    img[(X ** 2 + Z ** 2) <= R ** 2] = 1.0
    for _ in range(n_spheres):
        r = rng.uniform(0.004, 0.006) * scale
        rho = rng.uniform(0, R - r)
        phi = rng.uniform(0, 2 * np.pi)
        c = (rho * np.cos(phi), rng.uniform(-half + r, half - r) * 0.6, rho * np.sin(phi))
        img[((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2) <= r ** 2] = 4.0
    return img.reshape(-1).astype(np.float32)


def measurement(p: Problem, counts: float, seed: int = 2, phantom_seed: int = 1,
                x_true: np.ndarray | None = None):
    """Returns (rows int32 [m], y float32 [m], x_true float32 [V]) on the
    device: rows with y > 0 of Poisson(A' x_true scaled to `counts`), A' the
    system matrix with ray seed DATA_SEED."""
    if x_true is None:
        x_true = phantom_image(p, phantom_seed)
    x = torch.from_numpy(x_true).cuda()
    p_data = p.with_seed(DATA_SEED)
    nch = p.nchannels
    ybar = torch.empty(nch, dtype=torch.float32, device="cuda")
    step = 1 << 20
    for c0 in range(0, nch, step):
        rows = torch.arange(c0, min(nch, c0 + step), dtype=torch.int32, device="cuda")
        ybar[c0:c0 + rows.numel()] = api.project_forward(p_data, rows, x)
    total = float(ybar.double().sum().item())
    lam = (ybar.double() * (counts / total)).clamp_min(0)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    y = torch.poisson(lam, generator=gen).to(torch.float32)
    rows = torch.nonzero(y > 0).flatten().to(torch.int32)
    return rows, y[rows.long()].contiguous(), torch.from_numpy(x_true)
