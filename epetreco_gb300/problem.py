"""Geometry descriptors of the MLEM hot path.

``MeasurementSetup`` mirrors the reference's ``DefaultMeasurementSetup<T>``
(MeasurementSetup.hpp:124-164; constructor argument order
pos0x, pos1x, na, n0z, n0y, n1z, n1y, da, segx, segy, segz) and ``VoxelGrid``
mirrors ``DefaultVoxelGrid<T>`` (VoxelGrid.hpp:88-200; origin, pitch, count
per axis).  Units are metres and degrees, as in the reference's compiled
defaults (real_measurementsetup_defines.h, voxelgrid_defines.h).

The reference bakes one geometry into ``__constant__`` memory per process
(device_constant_memory.hpp:14-26); here a ``Problem`` is a value passed to
every call, so several geometries can live side by side (batched form).
"""
from __future__ import annotations

from dataclasses import dataclass, field, replace

import numpy as np


@dataclass(frozen=True)
class MeasurementSetup:
    """Two planar heads rotating about y (MeasurementSetup.hpp:124-164)."""
    pos0x: float
    pos1x: float
    na: int
    n0z: int
    n0y: int
    n1z: int
    n1y: int
    da: float
    segx: float
    segy: float
    segz: float

    @property
    def nchannels(self) -> int:
        return self.na * self.n0z * self.n0y * self.n1z * self.n1y

    def channel_id(self, ida, id0z, id0y, id1z, id1y):
        """Linear channel id (MeasurementSetupLinIndex.hpp:39-44): angle
        slowest, id1y fastest."""
        return (((ida * self.n0z + id0z) * self.n0y + id0y) * self.n1z + id1z) * self.n1y + id1y

    def channel_indices(self, cnl):
        """Inverse of :meth:`channel_id` (MeasurementSetupLinIndex.hpp:58-165)."""
        cnl = np.asarray(cnl)
        id1y = cnl % self.n1y
        t = cnl // self.n1y
        id1z = t % self.n1z
        t = t // self.n1z
        id0y = t % self.n0y
        t = t // self.n0y
        id0z = t % self.n0z
        ida = t // self.n0z
        return ida, id0z, id0y, id1z, id1y


@dataclass(frozen=True)
class VoxelGrid:
    """Axis-aligned grid (VoxelGrid.hpp:88-200); voxel id = ix*(ny*nz) +
    iy*nz + iz (VoxelGridLinIndex.hpp:33-35)."""
    origin: tuple
    pitch: tuple
    n: tuple

    @property
    def nvoxels(self) -> int:
        return int(self.n[0]) * int(self.n[1]) * int(self.n[2])

    def voxel_id(self, ix, iy, iz):
        return (ix * self.n[1] + iy) * self.n[2] + iz

    def voxel_indices(self, vxl):
        vxl = np.asarray(vxl)
        iz = vxl % self.n[2]
        t = vxl // self.n[2]
        return t // self.n[1], t % self.n[1], iz

    def centres(self, axis: int) -> np.ndarray:
        """Voxel centre coordinates along an axis, float32 as the reference
        forms them (o + (i + 0.5) * d)."""
        o = np.float32(self.origin[axis])
        d = np.float32(self.pitch[axis])
        i = np.arange(self.n[axis], dtype=np.float32)
        return (o + (i + np.float32(0.5)) * d).astype(np.float32)


RAY_GENERATORS = ("random", "regular")


@dataclass(frozen=True)
class Problem:
    """One reconstruction geometry plus its Monte-Carlo ray settings.

    ``rays`` picks the ray generator (RayGenerators.hpp): "random" is
    ``RandRayGen`` (six cuRAND uniforms per ray, generator seeded per channel
    with ``seed``), "regular" is ``ReguRayGen`` (every ray joins the two
    crystal centres; the seed is unused)."""
    setup: MeasurementSetup
    grid: VoxelGrid
    nrays: int
    seed: int = 1251  # RANDOM_SEED (getSystemMatrixFromWorkqueue.cu:22)
    rays: str = "random"

    def __post_init__(self):
        if self.rays not in RAY_GENERATORS:
            raise ValueError(f"rays must be one of {RAY_GENERATORS}")

    @property
    def ray_mode(self) -> int:
        """EPET_RAYS_RANDOM (0) or EPET_RAYS_REGULAR (1)."""
        return RAY_GENERATORS.index(self.rays)

    @property
    def nchannels(self) -> int:
        return self.setup.nchannels

    @property
    def nvoxels(self) -> int:
        return self.grid.nvoxels

    def with_seed(self, seed: int) -> "Problem":
        return replace(self, seed=seed)

    def with_rays(self, rays: str) -> "Problem":
        return replace(self, rays=rays)


def two_head_setup(na: int, da: float, pos: float = 0.25, n: int = 13,
                   seg=(0.020, 0.004, 0.004)) -> MeasurementSetup:
    """Two opposing heads of n x n crystals of seg (x, y, z) metres, centres
    at x = -pos and +pos, na angular steps of da degrees about y."""
    return MeasurementSetup(-pos, pos, na, n, n, n, n, da, *seg)


def centred_grid(n: int, pitch: float = 0.002) -> VoxelGrid:
    half = n * pitch / 2
    return VoxelGrid((-half,) * 3, (pitch,) * 3, (n,) * 3)


# Workloads.  "small" is the CPU-runnable case; "full" is the headline
# single-GPU case (52^3 voxels x 5,140,980 channels, 100 rays, 20 iterations).
CONFIGS = {
    "small": dict(problem=Problem(two_head_setup(8, 22.5), centred_grid(32), 10),
                  iterations=5, counts=1e6),
    "full": dict(problem=Problem(two_head_setup(180, 2.0), centred_grid(52), 100),
                 iterations=20, counts=5e8),
}


def config(name: str) -> dict:
    return dict(CONFIGS[name])


# Batched workload: independent reconstructions of uneven size.  Grids and
# angle counts are drawn uniformly from these sets; 8 angles step 22.5 deg
# (as the small workload), the others cover 360 deg (180 angles: 2 deg, as
# the full workload).
BATCH_GRIDS = (24, 32, 40, 52, 64)
BATCH_ANGLES = (8, 30, 60, 120, 180)


def batch_angle_step(na: int) -> float:
    return 22.5 if na == 8 else 360.0 / na


@dataclass(frozen=True)
class BatchMember:
    problem: Problem
    counts: float       # total Poisson counts of the measurement
    n_spheres: int      # hot spheres in the phantom
    phantom_seed: int
    poisson_seed: int


def batch_members(n: int = 64, seed: int = 4242, grids=BATCH_GRIDS, angles=BATCH_ANGLES,
                  rays=(20, 100), counts=(1e5, 1e8)) -> list[BatchMember]:
    """n seeded draws: grid and angle count uniform from the sets, rays
    uniform in [rays[0], rays[1]], counts log-uniform in [counts[0],
    counts[1]], 1-4 hot spheres."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        g = int(rng.choice(grids))
        na = int(rng.choice(angles))
        nr = int(rng.integers(rays[0], rays[1] + 1))
        c = float(10 ** rng.uniform(np.log10(counts[0]), np.log10(counts[1])))
        ns = int(rng.integers(1, 5))
        out.append(BatchMember(Problem(two_head_setup(na, batch_angle_step(na)),
                                       centred_grid(g), nr),
                               c, ns, 100 + i, 200 + i))
    return out
