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


from epetreco_gb300.problem import MeasurementSetup, VoxelGrid  # noqa: E402

# Geometries off the two workloads: heads of different crystal counts at
# uneven distances, an angle step that is not a divisor of 360, a grid that is
# neither cubic nor centred nor of equal pitches, and quarter turns (lines along
# z at 90 and 270 degrees).
ODD = {
    "asymmetric": Problem(MeasurementSetup(-0.31, 0.19, 7, 5, 7, 9, 3, 13.0, 0.02, 0.004, 0.005),
                          VoxelGrid((-0.041, -0.023, -0.017), (0.003, 0.002, 0.0025),
                                    (24, 18, 14)), 9),
    "quarter_turns": Problem(MeasurementSetup(-0.2, 0.2, 4, 6, 4, 6, 4, 90.0, 0.01, 0.003, 0.003),
                             VoxelGrid((-0.02, -0.01, -0.015), (0.002, 0.002, 0.002),
                                       (20, 10, 15)), 5),
}


@pytest.mark.parametrize("name", list(ODD))
def test_odd_geometry_indices_and_transforms(oracle, ref, name):
    p = ODD[name]
    ref.setup(p)
    rng = np.random.default_rng(11)
    out5 = np.zeros(5, np.int32)
    for c in rng.choice(p.nchannels, 200, replace=False):
        ref.lib.ref_channel_decode(int(c), out5)
        assert (oracle.channel_decode(p, int(c)) == out5).all()
        assert ref.lib.ref_channel_encode(*[int(v) for v in out5]) == c
        assert p.setup.channel_id(*[int(v) for v in out5]) == c
    out3 = np.zeros(3, np.int32)
    for v in rng.choice(p.nvoxels, 200, replace=False):
        ref.lib.ref_voxel_decode(int(v), out3)
        assert (oracle.voxel_decode(p, int(v)) == out3).all()
        assert p.grid.voxel_id(*[int(x) for x in out3]) == v
    trig = oracle.trig_table(p)
    w_ref = np.zeros(3, np.float32)
    for c in rng.choice(p.nchannels, 100, replace=False):
        ida, i0z, i0y, i1z, i1y = (int(v) for v in oracle.channel_decode(p, int(c)))
        box = rng.random(3).astype(np.float32)
        sc = trig[2 * ida:2 * ida + 2]
        ref.lib.ref_trafo0(box, i0z, i0y, ida, w_ref)
        assert (oracle.trafo(p, sc, 0, i0z, i0y, box).view(np.uint32) == w_ref.view(np.uint32)).all()
        ref.lib.ref_trafo1(box, i1z, i1y, ida, w_ref)
        assert (oracle.trafo(p, sc, 1, i1z, i1y, box).view(np.uint32) == w_ref.view(np.uint32)).all()


@pytest.mark.parametrize("name", list(ODD))
@pytest.mark.parametrize("rays", ["random", "regular"])
def test_odd_geometry_workqueue_and_values(oracle, ref, name, rays):
    p = ODD[name]
    ref.setup(p)
    rng = np.random.default_rng(13)
    rows = np.sort(rng.choice(p.nchannels, 16, replace=False)).astype(np.int32)
    oc, ov, _ = oracle.workqueue(p, rows)
    rc, rv = ref.workqueue(rows)
    assert len(oc) > 0
    assert len(oc) == len(rc) and (oc == rc).all() and (ov == rv).all()
    if rays == "regular":
        rnd = np.full((len(rows), p.nrays * 6), 0.5, np.float32)
    else:
        rnd = rng.random((len(rows), p.nrays * 6)).astype(np.float32)
        rnd[rnd == 0] = 1
    row_of = np.searchsorted(rows, oc).astype(np.int32)
    sel = rng.choice(len(oc), min(1000, len(oc)), replace=False)
    v = oracle.sm_values_wq(p, rows, p.nrays, rnd, row_of[sel], ov[sel])
    r = np.array([ref.lib.ref_sm_value(int(oc[i]), int(ov[i]), p.nrays,
                                       np.ascontiguousarray(rnd[row_of[i]]))
                  for i in sel], np.float32)
    assert (v.view(np.uint32) == r.view(np.uint32)).all()
    assert (v > 0).any()
