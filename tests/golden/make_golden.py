"""Generates tests/golden/ref_golden.npz from the reference's own code.

Run where the reference tree exists (it builds oracle/_ref/libepet_ref.so
from the reference headers, see oracle/Makefile):

    python tests/golden/make_golden.py

Everything stored is an output of the reference's code on seeded inputs
(geometry functors, candidate scan, per-element values, thrust-based
operators run on the host backend) plus the reference's own unit-test
inputs (test_cooSort.cu, test_convertCsr2Ecsr.cu, test_cusparseWrapper.cu,
test_mlemOperations.cu).  The trig table used by the transforms is stored
too, so checks do not depend on the platform's libm.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from epetreco_gb300.problem import config  # noqa: E402
from pyoracle import Oracle, RefHarness  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_golden.npz")


def main():
    ref = RefHarness()
    orc = Oracle()
    L = ref.lib
    g = {}
    # --- known answers from the reference's own unit tests, run through its code
    A = np.array([1, 3, 2, 2, 1, 3], np.int32)
    B = np.array([2, 2, 1, 2, 1, 1], np.int32)
    Cv = np.array([2, 6, 3, 4, 1, 5], np.float32)
    L.ref_coo_sort(Cv, A, B, 6)
    g["coosort_row"], g["coosort_col"], g["coosort_val"] = A, B, Cv
    yrid = np.array([2, 4, 6], np.int32)
    csr = np.array([0, 0, 0, 3, 3, 3, 3, 5], np.int32)
    ecsr = np.zeros(4, np.int32)
    L.ref_csr2ecsr(ecsr, yrid, 3, csr, 7)
    g["ecsr_yrid"], g["ecsr_csr"], g["ecsr_out"] = yrid, csr, ecsr
    # coo2csr input of test_cusparseWrapper.cu (the reference prints nothing;
    # the expected row pointer follows from the matrix drawn in its comment)
    g["coo2csr_row"] = np.array([0, 1, 1, 1, 2, 2, 3, 3, 3], np.int32)
    g["coo2csr_expect"] = np.array([0, 1, 4, 6, 9], np.int64)
    n = 10
    a = np.array([(i + 1) ** 2 for i in range(n)], np.float32)
    b = np.full(n, 10, np.float32)
    c = np.array([i + 1 for i in range(n)], np.float32)
    d = np.zeros(n, np.float32)
    L.ref_divides(d, a, c, n)
    g["mlem_divides"] = d.copy()
    L.ref_divides_multiplies(d, a, b, c, n)
    g["mlem_divmul"] = d.copy()
    norm = L.ref_sum(d, n)
    g["mlem_sum"] = np.float32(norm)
    L.ref_scales(d, C.c_float(1.0 / norm), n)
    g["mlem_scales"] = d.copy()
    # random cooSort case with duplicates (stability)
    rng = np.random.default_rng(3)
    nr = 2000
    row = rng.integers(0, 50, nr).astype(np.int32)
    col = rng.integers(0, 40, nr).astype(np.int32)
    val = rng.random(nr).astype(np.float32)
    g["coosort_rand_in"] = np.stack([row, col, val.view(np.int32)])
    r2, c2, v2 = row.copy(), col.copy(), val.copy()
    L.ref_coo_sort(v2, r2, c2, nr)
    g["coosort_rand_out"] = np.stack([r2, c2, v2.view(np.int32)])

    # --- geometry, candidates and values on both workload geometries
    for name in ("small", "full"):
        p = config(name)["problem"]
        ref.setup(p)
        trig = orc.trig_table(p)  # host sinf/cosf, same as the harness's
        g[f"{name}_trig"] = trig
        rng = np.random.default_rng(11)
        cn = rng.integers(0, p.nchannels, 200).astype(np.int32)
        dec = np.zeros((len(cn), 5), np.int32)
        for i, cc in enumerate(cn):
            L.ref_channel_decode(int(cc), dec[i])
        g[f"{name}_chan"], g[f"{name}_chan_dec"] = cn, dec
        vx = rng.integers(0, p.nvoxels, 200).astype(np.int32)
        vdec = np.zeros((len(vx), 3), np.int32)
        for i, vv in enumerate(vx):
            L.ref_voxel_decode(int(vv), vdec[i])
        g[f"{name}_vox"], g[f"{name}_vox_dec"] = vx, vdec
        # transforms
        nb = 300
        box = rng.random((nb, 3)).astype(np.float32)
        tc = rng.integers(0, p.nchannels, nb).astype(np.int32)
        t0 = np.zeros((nb, 3), np.float32)
        t1 = np.zeros((nb, 3), np.float32)
        for i in range(nb):
            ida, i0z, i0y, i1z, i1y = dec_of(L, tc[i])
            L.ref_trafo0(box[i], i0z, i0y, ida, t0[i])
            L.ref_trafo1(box[i], i1z, i1y, ida, t1[i])
        g[f"{name}_trafo_box"], g[f"{name}_trafo_cnl"] = box, tc
        g[f"{name}_trafo0"], g[f"{name}_trafo1"] = t0, t1
        # candidate workqueue of a few channels (one per angle quadrant and the
        # 90-degree direction, where lines run along z)
        per_angle = p.nchannels // p.setup.na
        picks = [int(rng.integers(0, p.nchannels)) for _ in range(4)]
        a90 = int(round(90.0 / p.setup.da)) % p.setup.na
        picks += [a90 * per_angle + int(rng.integers(0, per_angle)), a90 * per_angle]
        rows = np.array(sorted(set(picks)), np.int32)
        wc, wv = ref.workqueue(rows)
        g[f"{name}_wq_rows"], g[f"{name}_wq_cnl"], g[f"{name}_wq_vxl"] = rows, wc, wv
        # values with seeded uniforms in (0, 1]
        nr_ = p.nrays
        rnd = rng.random((len(rows), nr_, 6)).astype(np.float32)
        rnd[rnd == 0] = 1.0
        sel = np.sort(rng.choice(len(wc), min(1500, len(wc)), replace=False))
        row_of = np.searchsorted(rows, wc[sel]).astype(np.int32)
        vals = np.array([L.ref_sm_value(int(wc[i]), int(wv[i]), nr_,
                                        np.ascontiguousarray(rnd[row_of[k]].reshape(-1)))
                         for k, i in enumerate(sel)], np.float32)
        g[f"{name}_val_rnd"], g[f"{name}_val_sel"], g[f"{name}_val"] = rnd, sel.astype(np.int32), vals
    # slab chord lengths (both reference copies agree; stored once)
    rng = np.random.default_rng(5)
    nl = 3000
    rays = ((rng.random((nl, 6)) - 0.5) * 0.2).astype(np.float32)
    lo = ((rng.random((nl, 3)) - 0.5) * 0.04).astype(np.float32)
    boxes = np.concatenate([lo, lo + np.float32(0.002)], axis=1).astype(np.float32)
    # most rays through the boxes: a point inside the box +- a random direction
    k = (nl * 3) // 4
    inside = lo[:k] + np.float32(0.002) * rng.random((k, 3)).astype(np.float32)
    dirs = rng.normal(size=(k, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    rays[:k, :3] = (inside - 0.1 * dirs).astype(np.float32)
    rays[:k, 3:] = (inside + 0.1 * dirs).astype(np.float32)
    lens = np.array([L.ref_intersection_length(np.ascontiguousarray(boxes[i]),
                                               np.ascontiguousarray(rays[i])) for i in range(nl)],
                    np.float32)
    lens2 = np.array([L.ref_intersection_length_devonly(np.ascontiguousarray(boxes[i]),
                                                        np.ascontiguousarray(rays[i]))
                      for i in range(nl)], np.float32)
    assert (lens.view(np.uint32) == lens2.view(np.uint32)).all()
    g["isect_box"], g["isect_ray"], g["isect_len"] = boxes, rays, lens
    np.savez_compressed(OUT, **g)
    print(f"wrote {OUT} ({os.path.getsize(OUT)} bytes)")


def dec_of(L, cnl):
    out = np.zeros(5, np.int32)
    L.ref_channel_decode(int(cnl), out)
    return [int(v) for v in out]


if __name__ == "__main__":
    main()
