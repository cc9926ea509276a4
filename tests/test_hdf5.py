"""HDF5 files of the reference (measurement "messung", image "density"),
read and written by the library's own HDF5 code on the host (no GPU, no
libhdf5).  The reader is checked on a file libhdf5 wrote (a MATLAB v7.3 test
file shipped with scipy: superblock after a 512-byte user block, symbol-table
root group, old-style layout message, float64 data) and on variants of the
writer's files changed on the CPU (big-endian and integer element types, a
user block, chunked storage)."""
import os
import struct

import numpy as np
import pytest

from epetreco_gb300 import _lib
from epetreco_gb300.problem import VoxelGrid, centred_grid

SCIPY_H5 = os.path.join(os.path.dirname(np.__file__), "..", "scipy", "io", "matlab", "tests",
                        "data", "testhdf5_7.4_GLNX86.mat")


@pytest.fixture(scope="module", autouse=True)
def library():
    from epetreco_gb300 import build
    build.build()


def h5():
    from epetreco_gb300 import h5 as mod
    return mod


def test_measurement_round_trip(tmp_path):
    rng = np.random.default_rng(4)
    y = rng.poisson(0.7, 5000).astype(np.float32)
    assert (y == 0).any() and (y > 0).any()
    fn = tmp_path / "meas.h5"
    h5().write_measurement(fn, y)
    assert h5().dataset_shape(fn, "messung") == (5000,)
    assert np.array_equal(h5().read(fn, "messung"), y)
    rows, vals, nch = h5().readHDF5_MeasVct(fn)
    assert nch == 5000
    assert np.array_equal(rows, np.flatnonzero(y).astype(np.int32))
    assert np.array_equal(vals, y[y != 0])
    assert rows.dtype == np.int32 and vals.dtype == np.float32


def test_measurement_all_zero_and_empty(tmp_path):
    fn = tmp_path / "zero.h5"
    h5().write_measurement(fn, np.zeros(17, np.float32))
    rows, vals, nch = h5().readHDF5_MeasVct(fn)
    assert nch == 17 and rows.size == 0 and vals.size == 0
    fn = tmp_path / "empty.h5"
    h5().write_measurement(fn, np.zeros(0, np.float32))
    assert h5().dataset_shape(fn, "messung") == (0,)
    assert h5().read(fn, "messung").size == 0


def test_density_round_trip_and_attributes(tmp_path):
    g = VoxelGrid((-0.026, -0.03, 0.004), (0.001, 0.002, 0.0015), (5, 7, 3))
    x = np.random.default_rng(1).random(g.nvoxels).astype(np.float32)
    fn = tmp_path / "0_img.h5"
    h5().writeHDF5_Density(x, fn, g)
    assert h5().dataset_shape(fn, "density") == (5, 7, 3)
    xr, gr = h5().read_density(fn)
    assert xr.shape == (5, 7, 3)
    # voxel id = ix*(ny*nz) + iy*nz + iz is the file's row-major order
    assert np.array_equal(xr.ravel(), x)
    assert xr[2, 3, 1] == x[g.voxel_id(2, 3, 1)]
    assert np.array_equal(h5().readHDF5_Density(fn), x)
    assert gr.n == g.n
    assert np.array_equal(np.float32(gr.origin), np.float32(g.origin))
    # max = origin + n * pitch in float (H5DensityWriter.hpp:131-132); the
    # pitch read back is (max - min) / n
    o, d, n = np.float32(g.origin), np.float32(g.pitch), np.array(g.n)
    mx = (o + n.astype(np.float32) * d).astype(np.float32)
    assert np.allclose(gr.pitch, (mx.astype(np.float64) - o) / n, rtol=1e-6)
    assert np.allclose(gr.pitch, g.pitch, rtol=1e-5)


def attr_bytes(fn, name):
    """The 4 data bytes of scalar attribute `name` (located by its name in the
    file: the attribute messages this writer emits hold name, datatype and
    dataspace padded to 8 bytes, then the value)."""
    raw = open(fn, "rb").read()
    k = raw.find(name.encode() + b"\0")
    assert k > 0
    npad = (len(name) + 1 + 7) // 8 * 8
    tsz = struct.unpack_from("<H", raw, k - 4)[0]
    return raw[k + npad + (tsz + 7) // 8 * 8 + 8: k + npad + (tsz + 7) // 8 * 8 + 12]


def test_density_attribute_values(tmp_path):
    g = centred_grid(52)
    fn = tmp_path / "img.h5"
    h5().writeHDF5_Density(np.zeros(g.nvoxels, np.float32), fn, g)
    o, d = np.float32(g.origin[0]), np.float32(g.pitch[0])
    assert struct.unpack("<f", attr_bytes(fn, "xmin"))[0] == o
    assert struct.unpack("<f", attr_bytes(fn, "xmax"))[0] == np.float32(o + np.float32(52) * d)
    assert struct.unpack("<i", attr_bytes(fn, "znbin"))[0] == 52


def test_reads_file_written_by_libhdf5():
    if not os.path.exists(SCIPY_H5):
        pytest.skip("scipy's HDF5 test file is not installed")
    assert h5().dataset_shape(SCIPY_H5, "testdouble") == (9, 1)
    got = h5().read(SCIPY_H5, "/testdouble").ravel()
    want = (np.arange(9) * (np.pi / 4)).astype(np.float32)
    assert np.array_equal(got, want)


def patch(fn, out, edits):
    raw = bytearray(open(fn, "rb").read())
    for off, data in edits:
        raw[off:off + len(data)] = data
    open(out, "wb").write(bytes(raw))


def layout_and_type(fn):
    """File offsets of the dataset's datatype and layout messages and of its
    data (this writer: one dataset, version-1 object header)."""
    raw = open(fn, "rb").read()
    tree = struct.unpack_from("<Q", raw, 80)[0]
    snod = struct.unpack_from("<Q", raw, tree + 32)[0]
    oh = struct.unpack_from("<Q", raw, snod + 16)[0]
    size = struct.unpack_from("<I", raw, oh + 8)[0]
    p, out = oh + 16, {}
    while p < oh + 16 + size:
        t, s = struct.unpack_from("<HH", raw, p)
        out[t] = p + 8
        p += 8 + s
    data = struct.unpack_from("<Q", raw, out[0x08] + 2)[0]
    return out[0x03], out[0x08], data


def test_big_endian_and_integer_elements(tmp_path):
    y = np.array([0, 3, 1, 0, 250, 7], np.float32)
    fn = tmp_path / "m.h5"
    h5().write_measurement(fn, y)
    t, _, data = layout_and_type(fn)
    be = tmp_path / "be.h5"
    patch(fn, be, [(t + 1, bytes([0x21])), (data, y.astype(">f4").tobytes())])
    assert np.array_equal(h5().read(be, "messung"), y)
    # signed 32-bit integers, little- and big-endian
    ii = np.array([0, 3, -1, 0, 250, 7], np.int32)
    for order, code in (("<i4", 0x08), (">i4", 0x09)):
        f2 = tmp_path / f"int{code}.h5"
        patch(fn, f2, [(t, bytes([0x10, code, 0, 0])), (t + 8, struct.pack("<HH", 0, 32)),
                       (data, ii.astype(order).tobytes())])
        assert np.array_equal(h5().read(f2, "messung"), ii.astype(np.float32))
        rows, vals, _ = h5().readHDF5_MeasVct(f2)
        assert list(rows) == [1, 2, 4, 5] and list(vals) == [3, -1, 250, 7]


def test_user_block(tmp_path):
    """A file behind a 512-byte user block (addresses relative to the
    superblock, as libhdf5 writes such files)."""
    y = np.arange(1, 10, dtype=np.float32)
    fn = tmp_path / "m.h5"
    h5().write_measurement(fn, y)
    ub = tmp_path / "ub.h5"
    ub.write_bytes(b"\0" * 512 + fn.read_bytes())
    assert np.array_equal(h5().read(ub, "messung"), y)


def test_errors(tmp_path):
    fn = tmp_path / "m.h5"
    h5().write_measurement(fn, np.ones(8, np.float32))
    with pytest.raises(_lib.EpetError, match="no object"):
        h5().read(fn, "density")
    with pytest.raises(_lib.EpetError, match="cannot open"):
        h5().read(tmp_path / "missing.h5", "messung")
    bad = tmp_path / "bad.h5"
    bad.write_bytes(b"not an hdf5 file" * 64)
    with pytest.raises(_lib.EpetError, match="not an HDF5 file"):
        h5().read(bad, "messung")
    L = _lib.lib()
    out = np.zeros(4, np.float32)
    st = L.epet_h5_read_f32(os.fsencode(fn), b"messung", out.ctypes.data, 4)
    assert st == 2 and b"8 elements" in L.epet_last_error()  # EPET_ERR_CAPACITY
    _, lay, _ = layout_and_type(fn)
    ch = tmp_path / "chunked.h5"
    patch(fn, ch, [(lay + 1, bytes([2]))])
    with pytest.raises(_lib.EpetError, match="layout 2"):
        h5().read(ch, "messung")
    with pytest.raises(ValueError):
        h5().writeHDF5_Density(np.zeros(5, np.float32), tmp_path / "x.h5", centred_grid(2))
    rows = np.zeros(0, np.int32)
    st = L.epet_h5_read_measurement(os.fsencode(fn), rows.ctypes.data, rows.ctypes.data, 0,
                                    None, None)
    assert st == 2  # 8 measured channels, capacity 0


def test_checkpoint_carries_the_iteration(tmp_path):
    g = VoxelGrid((-0.01, -0.01, -0.01), (0.002, 0.002, 0.002), (4, 5, 6))
    x = np.random.default_rng(7).random(g.nvoxels).astype(np.float32)
    fn = tmp_path / "3_img.h5"
    h5().write_checkpoint(fn, x, g, 3)
    xr, gr, it = h5().read_checkpoint(fn)
    assert it == 3 and gr.n == g.n and np.array_equal(xr.ravel(), x)
    assert h5().read_attribute(fn, "density", "iteration") == 3.0
    assert h5().read_attribute(fn, "density", "znbin") == 6.0
    # still the reference's density file: its nine attributes and dataset
    assert np.array_equal(h5().readHDF5_Density(fn), x)
    plain = tmp_path / "img.h5"
    h5().writeHDF5_Density(x, plain, g)
    assert h5().read_checkpoint(plain)[2] == 0
    with pytest.raises(_lib.EpetError, match="no numeric attribute"):
        h5().read_attribute(plain, "density", "iteration")
    with pytest.raises(_lib.EpetError):
        h5().write_checkpoint(tmp_path / "bad.h5", x, g, -1)
