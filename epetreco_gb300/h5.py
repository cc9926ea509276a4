"""The reference's HDF5 files, read and written by the library's own HDF5
code (``csrc/hdf5_io.cpp``; libhdf5 is not needed).

* ``readHDF5_MeasVct`` (wrappers.hpp:311-333): the measurement dataset
  "messung" as the measured channels (value != 0) and their counts.
* ``readHDF5_Density`` (wrappers.hpp:452-464): the "density" dataset as a flat
  float array in file order.
* ``writeHDF5_Density`` (wrappers.hpp:398-403, H5DensityWriter.hpp:105-199):
  an image as the 3-D float dataset "density" [nx][ny][nz] with the grid's
  xmin/ymin/zmin, xmax/ymax/zmax and xnbin/ynbin/znbin attributes.

Host buffers only (numpy); errors raise ``EpetError`` with the library's
message.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib
from .problem import VoxelGrid


def _path(p) -> bytes:
    return os.fsencode(os.fspath(p))


def _grid_struct(g: VoxelGrid) -> _lib.Grid:
    return _lib.Grid((C.c_float * 3)(*g.origin), (C.c_float * 3)(*g.pitch),
                     (C.c_int32 * 3)(*g.n))


def dataset_shape(path, name: str) -> tuple:
    """Shape of dataset `name` ("group/name" for nested groups)."""
    nd = C.c_int32()
    dims = (C.c_int64 * 8)()
    _lib.check(_lib.lib().epet_h5_dataset_shape(_path(path), name.encode(), C.byref(nd), dims))
    return tuple(int(dims[i]) for i in range(nd.value))


def read(path, name: str) -> np.ndarray:
    """Dataset `name` as float32 with its shape (H5Reader::read,
    H5Reader.hpp:39-70, reads with NATIVE_FLOAT)."""
    shape = dataset_shape(path, name)
    out = np.empty(shape, np.float32)
    _lib.check(_lib.lib().epet_h5_read_f32(_path(path), name.encode(),
                                           out.ctypes.data_as(C.c_void_p), out.size))
    return out


def readHDF5_MeasVct(path):  # noqa: N802 - reference name
    """(row ids int32, counts float32, channels in the file): the channels of
    "messung" with a non-zero value, ascending."""
    L = _lib.lib()
    m, nch = C.c_int64(), C.c_int64()
    _lib.check(L.epet_h5_read_measurement(_path(path), None, None, 0, C.byref(m), C.byref(nch)))
    rows = np.empty(m.value, np.int32)
    y = np.empty(m.value, np.float32)
    _lib.check(L.epet_h5_read_measurement(_path(path), rows.ctypes.data_as(C.c_void_p),
                                          y.ctypes.data_as(C.c_void_p), m.value, C.byref(m),
                                          C.byref(nch)))
    return rows, y, int(nch.value)


def write_measurement(path, y) -> None:
    """A measurement file: the dense counts of every channel as the 1-D float
    dataset "messung"."""
    y = np.ascontiguousarray(np.asarray(y, np.float32).ravel())
    _lib.check(_lib.lib().epet_h5_write_measurement(_path(path), y.ctypes.data_as(C.c_void_p),
                                                    y.size))


def writeHDF5_Density(density, ofn, grid: VoxelGrid) -> None:  # noqa: N802 - reference name
    """The image (voxel id order, nx*ny*nz floats) as dataset "density"."""
    x = np.ascontiguousarray(np.asarray(density, np.float32).ravel())
    n = int(np.prod(grid.n))
    if x.size != n:
        raise ValueError(f"density holds {x.size} values, the grid {n}")
    g = _grid_struct(grid)
    _lib.check(_lib.lib().epet_h5_write_density(_path(ofn), x.ctypes.data_as(C.c_void_p),
                                                C.byref(g)))


def readHDF5_Density(ifn) -> np.ndarray:  # noqa: N802 - reference name
    """The "density" dataset as a flat float32 array in file order."""
    return read(ifn, "density").ravel()


def read_density(ifn):
    """(image [nx, ny, nz] float32, VoxelGrid from the file's attributes:
    origin = min, pitch = (max - min) / nbin)."""
    shape = dataset_shape(ifn, "density")
    x = np.empty(shape, np.float32)
    g = _lib.Grid()
    _lib.check(_lib.lib().epet_h5_read_density(_path(ifn), x.ctypes.data_as(C.c_void_p), x.size,
                                               C.byref(g)))
    return x, VoxelGrid(tuple(g.o), tuple(g.d), tuple(g.n))


def write_checkpoint(path, density, grid: VoxelGrid, iteration: int) -> None:
    """A "density" file with an int attribute "iteration" (a restart point)."""
    x = np.ascontiguousarray(np.asarray(density, np.float32).ravel())
    n = int(np.prod(grid.n))
    if x.size != n:
        raise ValueError(f"density holds {x.size} values, the grid {n}")
    g = _grid_struct(grid)
    _lib.check(_lib.lib().epet_h5_write_checkpoint(_path(path), x.ctypes.data_as(C.c_void_p),
                                                   C.byref(g), int(iteration)))


def read_attribute(path, name: str, attr: str) -> float:
    """Numeric scalar attribute `attr` of dataset `name`."""
    v = C.c_double()
    _lib.check(_lib.lib().epet_h5_read_attribute(_path(path), name.encode(), attr.encode(),
                                                 C.byref(v)))
    return v.value


def read_checkpoint(path):
    """(image [nx, ny, nz], VoxelGrid, iterations done; 0 for a "density"
    file without the "iteration" attribute)."""
    x, g = read_density(path)
    try:
        it = int(read_attribute(path, "density", "iteration"))
    except _lib.EpetError:
        it = 0
    return x, g, it

