"""The oracle against the reference's own code built for the host, on fresh
seeded inputs (where the reference tree exists).  CPU only."""
import os

import numpy as np
import pytest

from epetreco_gb300.problem import config, Problem, two_head_setup, centred_grid

pyoracle = pytest.importorskip("pyoracle")
if not os.path.isdir(pyoracle.REF_SRC):
    pytest.skip("reference tree absent", allow_module_level=True)


@pytest.fixture(scope="module")
def ref():
    return pyoracle.RefHarness()


PROBLEMS = {
    "small": config("small")["problem"],
    "full": config("full")["problem"],
    # the reference's compiled default heads (real_measurementsetup_defines.h)
    # with its GRID32 grid (voxelgrid_defines.h)
    "refdefault": Problem(two_head_setup(180, 2.0, pos=0.457), 
                          type(centred_grid(32))((-0.030,) * 3, (0.001875,) * 3, (32,) * 3), 7),
}


@pytest.mark.parametrize("name", list(PROBLEMS))
def test_workqueue_and_values(oracle, ref, name):
    p = PROBLEMS[name]
    ref.setup(p)
    rng = np.random.default_rng(hash(name) % 1000)
    rows = np.sort(rng.choice(p.nchannels, 12, replace=False)).astype(np.int32)
    oc, ov, _ = oracle.workqueue(p, rows)
    rc, rv = ref.workqueue(rows)
    assert len(oc) == len(rc) and (oc == rc).all() and (ov == rv).all()
    rnd = rng.random((len(rows), p.nrays, 6)).astype(np.float32)
    rnd[rnd == 0] = 1
    row_of = np.searchsorted(rows, oc).astype(np.int32)
    sel = rng.choice(len(oc), min(800, len(oc)), replace=False)
    v = oracle.sm_values_wq(p, rows, p.nrays, rnd, row_of[sel], ov[sel])
    r = np.array([ref.lib.ref_sm_value(int(oc[i]), int(ov[i]), p.nrays,
                                       np.ascontiguousarray(rnd[row_of[i]].reshape(-1)))
                  for i in sel], np.float32)
    assert (v.view(np.uint32) == r.view(np.uint32)).all()


def test_bounded_workqueue_is_prefix(ref, oracle):
    """The reference's bounded scan yields a prefix of the full scan
    (test_getWorkqueue.cu:190-198)."""
    import ctypes as C
    p = PROBLEMS["small"]
    ref.setup(p)
    rows = np.array([5, 1000, 20000], np.int32)
    full_c, full_v, _ = oracle.workqueue(p, rows)
    lid, vid = C.c_int(0), C.c_int(0)
    oc = np.zeros(777, np.int32)
    ov = np.zeros(777, np.int32)
    n = ref.lib.ref_workqueue_bounded(rows, 3, C.byref(lid), C.byref(vid), 777, oc, ov)
    assert n == 777
    assert (oc == full_c[:777]).all() and (ov == full_v[:777]).all()


@pytest.mark.parametrize("name", ["small", "full"])
def test_regular_ray_values(oracle, ref, name):
    """ReguRayGen (RayGenerators.hpp:46-66) is every box coordinate 0.5; its
    operator() is device-only, so the reference's host-built transforms and
    value loop get those uniforms.  Rows whose centre line has equal end
    coordinates on an axis (crystals at equal height) are included: there the
    reference's slab test leaves that axis out, a case random rays never
    reach."""
    p = PROBLEMS[name]
    ref.setup(p)
    rng = np.random.default_rng(5)
    pool = np.sort(rng.choice(p.nchannels, 400, replace=False)).astype(np.int32)
    half = np.full(p.nrays * 6, 0.5, np.float32)
    par = [c for c in pool
           if (lambda r: r[1] == r[4] or r[2] == r[5])(oracle.rays(p, c, half[:6])[0])]
    assert len(par) >= 3
    rows = np.array(sorted(set(pool[:6].tolist()) | set(par[:4])), np.int32)
    oc, ov, _ = oracle.workqueue(p, rows)
    row_of = np.searchsorted(rows, oc).astype(np.int32)
    sel = rng.choice(len(oc), min(1200, len(oc)), replace=False)
    rnd = np.broadcast_to(half, (len(rows), p.nrays * 6))
    v = oracle.sm_values_wq(p, rows, p.nrays, rnd, row_of[sel], ov[sel])
    r = np.array([ref.lib.ref_sm_value(int(oc[i]), int(ov[i]), p.nrays, half) for i in sel],
                 np.float32)
    assert (v.view(np.uint32) == r.view(np.uint32)).all()
    # the axis-parallel rows reach candidates the centre line misses
    on_par = np.isin(oc[sel], par[:4])
    assert (v[on_par] > 0).mean() > (v[~on_par] > 0).mean()
