"""The oracle against golden outputs of the reference's own code
(tests/golden/make_golden.py).  CPU only."""
import numpy as np
import pytest

from epetreco_gb300.problem import config


def bits(a):
    return np.asarray(a, np.float32).view(np.uint32)


def test_coosort_kat(oracle, golden):
    # test_cooSort.cu:17-33 inputs
    v, r, c = oracle.coo_sort([2, 6, 3, 4, 1, 5], [1, 3, 2, 2, 1, 3], [2, 2, 1, 2, 1, 1])
    assert (r == golden["coosort_row"]).all() and (c == golden["coosort_col"]).all()
    assert (v == golden["coosort_val"]).all()
    assert list(v) == [1, 2, 3, 4, 5, 6]


def test_coosort_random_stable(oracle, golden):
    row, col, val = golden["coosort_rand_in"]
    v, r, c = oracle.coo_sort(val.view(np.float32), row, col)
    ro, co, vo = golden["coosort_rand_out"]
    assert (r == ro).all() and (c == co).all() and (bits(v) == vo.view(np.uint32)).all()


def test_csr2ecsr_kat(oracle, golden):
    e = oracle.csr2ecsr(golden["ecsr_yrid"], golden["ecsr_csr"].astype(np.int64))
    assert list(e) == list(golden["ecsr_out"]) == [0, 3, 3, 5]


def test_coo2csr_kat(oracle, golden):
    assert list(oracle.coo2csr(golden["coo2csr_row"], 4)) == [0, 1, 4, 6, 9]


def test_mlem_ops_kat(oracle, golden):
    n = 10
    a = np.array([(i + 1) ** 2 for i in range(n)], np.float32)
    b = np.full(n, 10, np.float32)
    c = np.arange(1, n + 1, dtype=np.float32)
    assert (bits(oracle.divides(a, c)) == bits(golden["mlem_divides"])).all()
    d = oracle.divides_multiplies(a, b, c)
    assert (bits(d) == bits(golden["mlem_divmul"])).all()
    s = oracle.sum(d)
    assert np.float32(s) == golden["mlem_sum"] == 550
    assert (bits(oracle.scales(d, np.float32(1.0 / np.float32(s)))) == bits(golden["mlem_scales"])).all()


def test_divides_multiplies_zero_guard(oracle):
    r = oracle.divides_multiplies(np.array([2.0], np.float32), np.array([3.0], np.float32),
                                  np.array([0.0], np.float32))
    assert r[0] == 6.0


@pytest.mark.parametrize("name", ["small", "full"])
def test_index_maps(oracle, golden, name):
    p = config(name)["problem"]
    for c, d in zip(golden[f"{name}_chan"], golden[f"{name}_chan_dec"]):
        assert (oracle.channel_decode(p, c) == d).all()
        assert p.setup.channel_id(*[int(v) for v in d]) == c
    for v, d in zip(golden[f"{name}_vox"], golden[f"{name}_vox_dec"]):
        assert (oracle.voxel_decode(p, v) == d).all()
        assert p.grid.voxel_id(*[int(x) for x in d]) == v


@pytest.mark.parametrize("name", ["small", "full"])
def test_trafo(oracle, golden, name):
    p = config(name)["problem"]
    trig = golden[f"{name}_trig"]
    for box, cnl, t0, t1 in zip(golden[f"{name}_trafo_box"], golden[f"{name}_trafo_cnl"],
                                golden[f"{name}_trafo0"], golden[f"{name}_trafo1"]):
        ida, i0z, i0y, i1z, i1y = oracle.channel_decode(p, cnl)
        sc = trig[2 * ida:2 * ida + 2]
        assert (bits(oracle.trafo(p, sc, 0, i0z, i0y, box)) == bits(t0)).all()
        assert (bits(oracle.trafo(p, sc, 1, i1z, i1y, box)) == bits(t1)).all()


@pytest.mark.parametrize("name", ["small", "full"])
def test_workqueue(oracle, golden, name):
    p = config(name)["problem"]
    rows = golden[f"{name}_wq_rows"]
    cnl, vxl, cnt = oracle.workqueue(p, rows, trig=golden[f"{name}_trig"])
    assert (cnl == golden[f"{name}_wq_cnl"]).all()
    assert (vxl == golden[f"{name}_wq_vxl"]).all()


@pytest.mark.parametrize("name", ["small", "full"])
def test_values_sequential(oracle, golden, name):
    p = config(name)["problem"]
    rows = golden[f"{name}_wq_rows"]
    wc, wv = golden[f"{name}_wq_cnl"], golden[f"{name}_wq_vxl"]
    sel = golden[f"{name}_val_sel"]
    row_of = np.searchsorted(rows, wc[sel]).astype(np.int32)
    v = oracle.sm_values_wq(p, rows, p.nrays, golden[f"{name}_val_rnd"], row_of, wv[sel],
                            trig=golden[f"{name}_trig"])
    assert (bits(v) == bits(golden[f"{name}_val"])).all()


def test_intersection_length(oracle, golden):
    got = np.array([oracle.intersection_length(b, r)
                    for b, r in zip(golden["isect_box"], golden["isect_ray"])], np.float32)
    assert (bits(got) == bits(golden["isect_len"])).all()
    assert (got > 0).sum() > 100  # the fixture exercises real crossings


def test_chunk_helpers(oracle):
    from epetreco_gb300 import api
    for n_all, full in [(10, 3), (9, 3), (0, 5), (954 * 5 + 7, 954)]:
        nch = oracle.lib.eo_n_chunks(n_all, full)
        assert nch == api.nChunks(n_all, full)
        tot = 0
        for k in range(nch + 1):
            a = oracle.lib.eo_n_in_chunk(k, n_all, full)
            assert a == api.nInChunk(k, n_all, full)
            assert oracle.lib.eo_chunk_ptr(k, full) == api.chunkPtr(k, full)
            tot += a
        assert tot == n_all
