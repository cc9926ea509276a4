"""Failure paths, with the failures made on the host (no GPU fault): device
allocations forced to fail at every point of a reconstruction's set-up
(the library's fault injection), checked to raise the library's error and
to leave the library usable; and restarts from checkpoint files, which must
continue a reconstruction exactly."""
import os
import subprocess

import numpy as np
import pytest
import torch

from epetreco_gb300 import _lib, api, h5
from epetreco_gb300.problem import config

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def recon(gpu_lib):
    from epetreco_gb300.phantom import measurement
    p = config("small")["problem"]
    rows, y, _ = measurement(p, 2e5)
    keep = torch.arange(0, rows.numel(), 4, device="cuda")
    return p, rows[keep].contiguous(), y[keep].contiguous(), api.sensitivity(p)


def test_allocation_failures_raise_and_recover(recon):
    p, rows, y, s = recon
    ref = api.Mlem(p, rows, y, s, use_graph=False)
    ref.iterate(2)
    x_ref = ref.image().clone()
    ref.close()
    failed = 0
    try:
        for after in range(0, 400, 7):
            api.debug_fail_allocations(after)
            try:
                R = api.Mlem(p, rows, y, s, use_graph=False)
            except _lib.EpetError as e:
                failed += 1
                assert e.status == 3, e  # EPET_ERR_CUDA (out of memory)
                continue
            finally:
                api.debug_fail_allocations(-1)
            R.iterate(2)
            assert torch.equal(R.image(), x_ref)
            R.close()
            break
    finally:
        api.debug_fail_allocations(-1)
    assert failed > 3  # the injected failures hit several set-up steps
    # the library works as before after every failure
    R = api.Mlem(p, rows, y, s, use_graph=False)
    R.iterate(2)
    assert torch.equal(R.image(), x_ref)
    R.close()


def test_allocation_failure_in_the_build(recon):
    p, rows, _, _ = recon
    api.debug_fail_allocations(0)
    try:
        with pytest.raises(_lib.EpetError):
            api.systemMatrixCalculation(p, rows)
    finally:
        api.debug_fail_allocations(-1)
    A = api.systemMatrixCalculation(p, rows)
    assert A.nnz > 0


def test_resume_from_checkpoint_is_exact(recon, tmp_path):
    p, rows, y, s = recon
    a = api.Mlem(p, rows, y, s)
    a.iterate(4)
    b = api.Mlem(p, rows, y, s)
    b.iterate(2)
    b.checkpoint(tmp_path / "ck.h5", 2)
    b.close()
    c = api.Mlem(p, rows, y, s)
    assert c.resume(tmp_path / "ck.h5") == 2
    c.iterate(2)
    assert torch.equal(c.image(), a.image())


def test_driver_resumes_from_its_own_output(recon, tmp_path):
    """epet_reco writes "<it>_<out>" HDF5 files carrying the iterations
    done; given one as the guess it continues the count and its later files
    equal the uninterrupted run's."""
    from epetreco_gb300 import build
    from test_gpu_driver import geometry_arg
    p, rows, y, s = recon
    dense = np.zeros(p.nchannels, np.float32)
    dense[rows.cpu().numpy()] = y.cpu().numpy()
    h5.write_measurement(tmp_path / "meas.h5", dense)
    h5.writeHDF5_Density(s.cpu().numpy(), tmp_path / "sens.h5", p.grid)
    common = [str(tmp_path / "meas.h5"), "img.h5", str(p.nrays), str(tmp_path / "sens.h5"), "4"]

    def run(d, guess):
        os.makedirs(d, exist_ok=True)
        r = subprocess.run([build.RECO, *common, guess, geometry_arg(p), "--matrix-once"],
                           cwd=d, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr
    run(tmp_path / "full", "-")
    assert h5.read_checkpoint(tmp_path / "full" / "1_img.h5")[2] == 2
    run(tmp_path / "resumed", str(tmp_path / "full" / "1_img.h5"))
    assert not os.path.exists(tmp_path / "resumed" / "0_img.h5")
    for it in (2, 3):
        xa = h5.read_checkpoint(tmp_path / "full" / f"{it}_img.h5")
        xb = h5.read_checkpoint(tmp_path / "resumed" / f"{it}_img.h5")
        assert xb[2] == it + 1 and np.array_equal(xa[0], xb[0])
