"""The C++ driver built on the drop-in header (epet_reco: the reference's
reco.cu flow over include/epet_gb300_shim.hpp) against the library's
reconstruction object on the same inputs."""
import os
import subprocess

import numpy as np
import pytest
import torch

from epetreco_gb300 import api
from epetreco_gb300.problem import config

pytestmark = pytest.mark.gpu


def geometry_arg(p):
    s, g = p.setup, p.grid
    vals = [s.pos0x, s.pos1x, s.na, s.n0z, s.n0y, s.n1z, s.n1y, s.da, s.segx, s.segy, s.segz,
            *g.origin, *g.pitch, *g.n]
    return ",".join(repr(float(v)) if isinstance(v, float) else str(v) for v in vals)


@pytest.fixture(scope="module")
def inputs(gpu_lib, tmp_path_factory):
    from epetreco_gb300 import build
    from epetreco_gb300.phantom import measurement
    p = config("small")["problem"]
    rows, y, _ = measurement(p, 2e5)
    s = api.sensitivity(p)
    d = tmp_path_factory.mktemp("reco")
    dense = np.zeros(p.nchannels, np.float32)
    dense[rows.cpu().numpy()] = y.cpu().numpy()
    dense.tofile(d / "meas.f32")
    s.cpu().numpy().tofile(d / "sens.f32")
    return p, rows, y, s, d, build.RECO


def run_driver(exe, d, p, nit, extra=()):
    cmd = [exe, str(d / "meas.f32"), "img.f32", str(p.nrays), str(d / "sens.f32"), str(nit), "-",
           geometry_arg(p), *extra]
    r = subprocess.run(cmd, cwd=d, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return np.fromfile(d / f"{nit - 1}_img.f32", np.float32)


def test_driver_matrix_once_matches_library(inputs):
    p, rows, y, s, d, exe = inputs
    x_drv = run_driver(exe, d, p, 3, ["--matrix-once"])
    R = api.Mlem(p, rows, y, s)
    R.iterate(3)
    x = R.image().cpu().numpy()
    assert np.linalg.norm(x_drv - x) / np.linalg.norm(x) < 1e-5


def test_driver_reference_loop_matches_library(inputs):
    """The reference's loop (matrix rebuilt per chunk and iteration, atomics
    transpose) through the reference-named operators of the shim."""
    p, rows, y, s, d, exe = inputs
    x_drv = run_driver(exe, d, p, 2)
    R = api.Mlem(p, rows, y, s)
    R.iterate(2)
    x = R.image().cpu().numpy()
    assert np.linalg.norm(x_drv - x) / np.linalg.norm(x) < 1e-5


@pytest.mark.parametrize("mode", ["--matrix-free", "--csc-transpose"])
def test_driver_other_schedules_match_library(inputs, mode):
    """The reconstruction object without a stored matrix, and the reference's
    loop whose transposed products read each chunk's column-major copy
    (epetBuildTranspose) instead of scattering with atomics."""
    p, rows, y, s, d, exe = inputs
    x_drv = run_driver(exe, d, p, 2, [mode])
    R = api.Mlem(p, rows, y, s)
    R.iterate(2)
    x = R.image().cpu().numpy()
    assert np.linalg.norm(x_drv - x) / np.linalg.norm(x) < 1e-5


def test_driver_hdf5_files_match_raw_files(inputs):
    """The reference's file formats: the measurement as "messung", the
    sensitivity as a "density" file, each iteration's image written as a
    "density" file with the grid's attributes; the images equal the raw-file
    run's bit for bit."""
    from epetreco_gb300 import h5
    p, rows, y, s, d, exe = inputs
    dense = np.fromfile(d / "meas.f32", np.float32)
    h5.write_measurement(d / "meas.h5", dense)
    h5.writeHDF5_Density(s.cpu().numpy(), d / "sens.h5", p.grid)
    nit = 2
    cmd = [exe, str(d / "meas.h5"), "img.h5", str(p.nrays), str(d / "sens.h5"), str(nit), "-",
           geometry_arg(p), "--matrix-once"]
    r = subprocess.run(cmd, cwd=d, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    x_raw = run_driver(exe, d, p, nit, ["--matrix-once"])
    for it in range(nit):
        x, g = h5.read_density(d / f"{it}_img.h5")
        assert x.shape == tuple(p.grid.n) and g.n == tuple(p.grid.n)
        assert np.array_equal(np.float32(g.origin), np.float32(p.grid.origin))
    assert np.array_equal(x.ravel(), x_raw)
