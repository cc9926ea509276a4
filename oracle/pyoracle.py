"""ctypes wrappers for the CPU oracle and the host-built reference harness.

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline legs of ``bench.py``.  The product (``epetreco_gb300``) never
imports this module.

``Oracle`` wraps ``oracle/_build/libepet_oracle.so`` (the plain-C restatement
in ``epet_oracle.c``).  ``RefHarness`` wraps ``oracle/_ref/libepet_ref.so``,
the reference's own host-callable code built from the reference tree by
``make -C oracle ref``; it exists only where that tree exists.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libepet_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libepet_ref.so")


def _ref_src() -> str:
    """The reference's src/ tree: EPET_REF_SRC, else the recipe's default
    (``make -C oracle ref-src``)."""
    env = os.environ.get("EPET_REF_SRC")
    if env:
        return env
    try:
        return subprocess.run(["make", "-s", "-C", HERE, "ref-src"], capture_output=True,
                              text=True, check=True).stdout.strip()
    except (OSError, subprocess.CalledProcessError):
        return ""


REF_SRC = _ref_src()

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")


class EoSetup(C.Structure):
    _fields_ = [("pos0x", C.c_float), ("pos1x", C.c_float), ("na", C.c_int),
                ("n0z", C.c_int), ("n0y", C.c_int), ("n1z", C.c_int),
                ("n1y", C.c_int), ("da", C.c_float), ("segx", C.c_float),
                ("segy", C.c_float), ("segz", C.c_float)]


class EoGrid(C.Structure):
    _fields_ = [("o", C.c_float * 3), ("d", C.c_float * 3), ("n", C.c_int * 3)]


def build_oracle(force: bool = False) -> str:
    if force or not os.path.exists(ORACLE_SO) or (
            os.path.getmtime(ORACLE_SO) < max(
                os.path.getmtime(os.path.join(HERE, f))
                for f in ("epet_oracle.c", "epet_oracle.h"))):
        subprocess.check_call(["make", "-s", "-C", HERE, "all"])
    return ORACLE_SO


def build_ref() -> str | None:
    """Builds the reference harness when the reference tree is present."""
    if not os.path.isdir(REF_SRC):
        return None
    srcs = [os.path.join(HERE, "ref", f) for f in os.listdir(os.path.join(HERE, "ref"))]
    if not os.path.exists(REF_SO) or os.path.getmtime(REF_SO) < max(map(os.path.getmtime, srcs)):
        subprocess.check_call(["make", "-s", "-C", HERE, "ref", f"REF_SRC={REF_SRC}"])
    return REF_SO


def _setup_struct(p) -> EoSetup:
    s = p.setup
    return EoSetup(s.pos0x, s.pos1x, s.na, s.n0z, s.n0y, s.n1z, s.n1y, s.da,
                   s.segx, s.segy, s.segz)


def _grid_struct(p) -> EoGrid:
    g = p.grid
    return EoGrid((C.c_float * 3)(*g.origin), (C.c_float * 3)(*g.pitch),
                  (C.c_int * 3)(*g.n))


class Oracle:
    """The plain-C restatement.  ``p`` arguments are ``epetreco_gb300``-style
    problem descriptions (anything with ``.setup`` and ``.grid``)."""

    def __init__(self):
        lib = C.CDLL(build_oracle())
        self.lib = lib
        S, G = C.POINTER(EoSetup), C.POINTER(EoGrid)
        lib.eo_channel_decode.argtypes = [S, C.c_int, _i32p]
        lib.eo_channel_encode.argtypes = [S] + [C.c_int] * 5
        lib.eo_voxel_decode.argtypes = [G, C.c_int, _i32p]
        lib.eo_voxel_encode.argtypes = [G, C.c_int, C.c_int, C.c_int]
        lib.eo_trig_table.argtypes = [S, _f32p]
        lib.eo_trafo.argtypes = [S, _f32p, C.c_int, C.c_int, C.c_int, _f32p, _f32p]
        lib.eo_candidate.argtypes = [S, G, C.c_void_p, C.c_int, C.c_int]
        lib.eo_intersection_length.argtypes = [_f32p, _f32p]
        lib.eo_intersection_length.restype = C.c_float
        lib.eo_rays.argtypes = [S, C.c_void_p, C.c_int, C.c_int, _f32p, _f32p]
        lib.eo_sm_value.argtypes = [G, _f32p, C.c_int, C.c_int, C.c_int]
        lib.eo_sm_value.restype = C.c_float
        lib.eo_workqueue.argtypes = [S, G, C.c_void_p, _i32p, C.c_int64, _i32p, _i32p, C.c_int64]
        lib.eo_workqueue.restype = C.c_int64
        lib.eo_workqueue_counts.argtypes = [S, G, C.c_void_p, _i32p, C.c_int64, _i64p]
        lib.eo_workqueue_counts.restype = C.c_int64
        lib.eo_sm_values_wq.argtypes = [S, G, C.c_void_p, _i32p, C.c_int, _f32p, C.c_int64,
                                        _i32p, _i32p, C.c_int, _f32p]
        lib.eo_sm_build_csr.argtypes = [S, G, C.c_void_p, _i32p, C.c_int64, C.c_int, _f32p,
                                        C.c_int, _i64p, _i32p, _f32p, C.c_int64]
        lib.eo_sm_build_csr.restype = C.c_int64
        lib.eo_sm_build_start.argtypes = [S, G, C.c_void_p, _i32p, C.c_int64, C.c_int, _f32p,
                                          C.c_int, C.POINTER(C.c_int64)]
        lib.eo_sm_build_start.restype = C.c_void_p
        lib.eo_sm_build_finish.argtypes = [C.c_void_p, _i64p, _i32p, _f32p]
        lib.eo_mlem_f64_trace.argtypes = [C.c_int64, C.c_int64, _i64p, _i32p, _f32p, _f64p,
                                          _f64p, _f64p, C.c_int, _f64p]
        lib.eo_coo_sort.argtypes = [_f32p, _i32p, _i32p, C.c_int64]
        lib.eo_coo2csr.argtypes = [_i32p, C.c_int64, C.c_int64, _i64p]
        lib.eo_csr2ecsr.argtypes = [_i64p, _i32p, C.c_int64, _i64p, C.c_int64]
        lib.eo_csrmv.argtypes = [C.c_int, C.c_int64, C.c_int64, _i64p, _i32p, _f32p, C.c_float,
                                 _f32p, C.c_float, _f32p]
        lib.eo_csrmv_f64.argtypes = [C.c_int, C.c_int64, C.c_int64, _i64p, _i32p, _f32p,
                                     C.c_double, _f64p, C.c_double, _f64p]
        lib.eo_divides.argtypes = [_f32p, _f32p, _f32p, C.c_int64]
        lib.eo_divides_multiplies.argtypes = [_f32p, _f32p, _f32p, _f32p, C.c_int64]
        lib.eo_scales.argtypes = [_f32p, C.c_float, C.c_int64]
        lib.eo_sum.argtypes = [_f32p, C.c_int64]
        lib.eo_sum.restype = C.c_double
        lib.eo_mlem.argtypes = [C.c_int64, C.c_int64, _i64p, _i32p, _f32p, _f32p, _f32p, _f32p,
                                C.c_int]
        lib.eo_mlem_f64.argtypes = [C.c_int64, C.c_int64, _i64p, _i32p, _f32p, _f64p, _f64p,
                                    _f64p, C.c_int]
        lib.eo_sensitivity.argtypes = [C.c_int64, C.c_int64, _i64p, _i32p, _f32p, _f32p]
        lib.eo_poisson_loglik.argtypes = [C.c_int64, _f32p, _f32p]
        lib.eo_poisson_loglik.restype = C.c_double
        for f in ("eo_n_in_chunk", "eo_chunk_ptr", "eo_n_chunks", "eo_nchannels"):
            getattr(lib, f).restype = C.c_int64
        lib.eo_n_in_chunk.argtypes = [C.c_int64] * 3
        lib.eo_chunk_ptr.argtypes = [C.c_int64] * 2
        lib.eo_n_chunks.argtypes = [C.c_int64] * 2
        lib.eo_nchannels.argtypes = [S]

    # -- helpers
    @staticmethod
    def _trig_ptr(trig):
        if trig is None:
            return None
        trig = np.ascontiguousarray(trig, np.float32)
        return trig.ctypes.data_as(C.c_void_p), trig

    def trig_table(self, p) -> np.ndarray:
        s = _setup_struct(p)
        out = np.zeros(2 * s.na, np.float32)
        self.lib.eo_trig_table(C.byref(s), out)
        return out

    def channel_decode(self, p, cnl):
        out = np.zeros(5, np.int32)
        self.lib.eo_channel_decode(C.byref(_setup_struct(p)), int(cnl), out)
        return out

    def voxel_decode(self, p, vxl):
        out = np.zeros(3, np.int32)
        self.lib.eo_voxel_decode(C.byref(_grid_struct(p)), int(vxl), out)
        return out

    def trafo(self, p, trig_sc, det, iz, iy, box):
        out = np.zeros(3, np.float32)
        self.lib.eo_trafo(C.byref(_setup_struct(p)), np.asarray(trig_sc, np.float32), det, iz,
                          iy, np.asarray(box, np.float32), out)
        return out

    def candidate(self, p, cnl, vxl, trig=None):
        tp = self._trig_ptr(trig)
        return bool(self.lib.eo_candidate(C.byref(_setup_struct(p)), C.byref(_grid_struct(p)),
                                          tp[0] if tp else None, int(cnl), int(vxl)))

    def intersection_length(self, vxl6, ray6) -> float:
        return self.lib.eo_intersection_length(np.asarray(vxl6, np.float32),
                                               np.asarray(ray6, np.float32))

    def rays(self, p, cnl, rnd, trig=None):
        rnd = np.ascontiguousarray(rnd, np.float32).reshape(-1)
        nrays = rnd.size // 6
        out = np.zeros(nrays * 6, np.float32)
        tp = self._trig_ptr(trig)
        self.lib.eo_rays(C.byref(_setup_struct(p)), tp[0] if tp else None, int(cnl), nrays,
                         rnd, out)
        return out.reshape(nrays, 6)

    def workqueue(self, p, rows, trig=None):
        rows = np.ascontiguousarray(rows, np.int32)
        tp = self._trig_ptr(trig)
        S, G = C.byref(_setup_struct(p)), C.byref(_grid_struct(p))
        cnt = np.zeros(len(rows) + 1, np.int64)
        total = self.lib.eo_workqueue_counts(S, G, tp[0] if tp else None, rows, len(rows), cnt)
        oc = np.zeros(max(total, 1), np.int32)
        ov = np.zeros(max(total, 1), np.int32)
        self.lib.eo_workqueue(S, G, tp[0] if tp else None, rows, len(rows), oc, ov, total)
        return oc[:total], ov[:total], cnt[:len(rows)]

    def sm_values_wq(self, p, rows, nrays, rnd_rows, wq_row, wq_vxl, exact=False, trig=None):
        rows = np.ascontiguousarray(rows, np.int32)
        rnd_rows = np.ascontiguousarray(rnd_rows, np.float32).reshape(-1)
        wq_row = np.ascontiguousarray(wq_row, np.int32)
        wq_vxl = np.ascontiguousarray(wq_vxl, np.int32)
        out = np.zeros(max(len(wq_vxl), 1), np.float32)
        tp = self._trig_ptr(trig)
        self.lib.eo_sm_values_wq(C.byref(_setup_struct(p)), C.byref(_grid_struct(p)),
                                 tp[0] if tp else None, rows, nrays, rnd_rows, len(wq_vxl),
                                 wq_row, wq_vxl, 1 if exact else 0, out)
        return out[:len(wq_vxl)]

    def sm_build_csr(self, p, rows, nrays, rnd_rows, exact=False, trig=None):
        """Returns (row_ptr int64[m+1], col int32[nnz], val float32[nnz])."""
        rows = np.ascontiguousarray(rows, np.int32)
        rnd_rows = np.ascontiguousarray(rnd_rows, np.float32).reshape(-1)
        m = len(rows)
        tp = self._trig_ptr(trig)
        S, G = C.byref(_setup_struct(p)), C.byref(_grid_struct(p))
        nnz = C.c_int64(0)
        h = self.lib.eo_sm_build_start(S, G, tp[0] if tp else None, rows, m, nrays, rnd_rows,
                                       1 if exact else 0, C.byref(nnz))
        n = nnz.value
        rp = np.zeros(m + 1, np.int64)
        col = np.zeros(max(n, 1), np.int32)
        val = np.zeros(max(n, 1), np.float32)
        self.lib.eo_sm_build_finish(h, rp, col, val)
        return rp, col[:n], val[:n]

    def coo_sort(self, val, row, col):
        val = np.array(val, np.float32)
        row = np.array(row, np.int32)
        col = np.array(col, np.int32)
        self.lib.eo_coo_sort(val, row, col, len(val))
        return val, row, col

    def coo2csr(self, row, m):
        out = np.zeros(m + 1, np.int64)
        self.lib.eo_coo2csr(np.ascontiguousarray(row, np.int32), len(row), m, out)
        return out

    def csr2ecsr(self, yrow, csr):
        yrow = np.ascontiguousarray(yrow, np.int32)
        csr = np.ascontiguousarray(csr, np.int64)
        out = np.zeros(len(yrow) + 1, np.int64)
        self.lib.eo_csr2ecsr(out, yrow, len(yrow), csr, len(csr) - 1)
        return out

    def csrmv(self, trans, rp, col, val, x, n, alpha=1.0, beta=0.0, y=None):
        m = len(rp) - 1
        out_len = n if trans else m
        y = np.zeros(out_len, np.float32) if y is None else np.array(y, np.float32)
        self.lib.eo_csrmv(int(trans), m, n, np.ascontiguousarray(rp, np.int64),
                          np.ascontiguousarray(col, np.int32), np.ascontiguousarray(val, np.float32),
                          alpha, np.ascontiguousarray(x, np.float32), beta, y)
        return y

    def csrmv_f64(self, trans, rp, col, val, x, n, alpha=1.0, beta=0.0, y=None):
        m = len(rp) - 1
        out_len = n if trans else m
        y = np.zeros(out_len, np.float64) if y is None else np.array(y, np.float64)
        self.lib.eo_csrmv_f64(int(trans), m, n, np.ascontiguousarray(rp, np.int64),
                              np.ascontiguousarray(col, np.int32),
                              np.ascontiguousarray(val, np.float32), alpha,
                              np.ascontiguousarray(x, np.float64), beta, y)
        return y

    def divides(self, a, b):
        r = np.zeros(len(a), np.float32)
        self.lib.eo_divides(r, np.ascontiguousarray(a, np.float32),
                            np.ascontiguousarray(b, np.float32), len(a))
        return r

    def divides_multiplies(self, a, b, c):
        r = np.zeros(len(a), np.float32)
        self.lib.eo_divides_multiplies(r, *(np.ascontiguousarray(v, np.float32) for v in (a, b, c)),
                                       len(a))
        return r

    def scales(self, x, alpha):
        x = np.array(x, np.float32)
        self.lib.eo_scales(x, alpha, len(x))
        return x

    def sum(self, x) -> float:
        return self.lib.eo_sum(np.ascontiguousarray(x, np.float32), len(x))

    def mlem(self, rp, col, val, y, s, x0, nit, V):
        x = np.array(x0, np.float32)
        self.lib.eo_mlem(len(rp) - 1, V, np.ascontiguousarray(rp, np.int64),
                         np.ascontiguousarray(col, np.int32), np.ascontiguousarray(val, np.float32),
                         np.ascontiguousarray(y, np.float32), np.ascontiguousarray(s, np.float32),
                         x, nit)
        return x

    def mlem_f64(self, rp, col, val, y, s, x0, nit, V):
        x = np.array(x0, np.float64)
        self.lib.eo_mlem_f64(len(rp) - 1, V, np.ascontiguousarray(rp, np.int64),
                             np.ascontiguousarray(col, np.int32),
                             np.ascontiguousarray(val, np.float32),
                             np.ascontiguousarray(y, np.float64),
                             np.ascontiguousarray(s, np.float64), x, nit)
        return x

    def mlem_f64_trace(self, rp, col, val, y, s, x0, nit, V):
        """FP64 MLEM; returns the images after each iteration, [nit][V]."""
        x = np.array(x0, np.float64)
        tr = np.zeros((nit, V), np.float64)
        self.lib.eo_mlem_f64_trace(len(rp) - 1, V, np.ascontiguousarray(rp, np.int64),
                                   np.ascontiguousarray(col, np.int32),
                                   np.ascontiguousarray(val, np.float32),
                                   np.ascontiguousarray(y, np.float64),
                                   np.ascontiguousarray(s, np.float64), x, nit, tr)
        return tr

    def sensitivity(self, rp, col, val, V):
        s = np.zeros(V, np.float32)
        self.lib.eo_sensitivity(len(rp) - 1, V, np.ascontiguousarray(rp, np.int64),
                                np.ascontiguousarray(col, np.int32),
                                np.ascontiguousarray(val, np.float32), s)
        return s

    def poisson_loglik(self, y, ybar) -> float:
        return self.lib.eo_poisson_loglik(len(y), np.ascontiguousarray(y, np.float32),
                                          np.ascontiguousarray(ybar, np.float32))


class RefHarness:
    """The reference's own host-callable code (built from the reference tree)."""

    def __init__(self):
        so = build_ref()
        if so is None:
            raise FileNotFoundError("reference tree absent: harness unavailable")
        lib = C.CDLL(so)
        self.lib = lib
        lib.ref_setup.argtypes = [C.c_float, C.c_float] + [C.c_int] * 5 + [C.c_float] * 4 + \
            [C.c_float] * 6 + [C.c_int] * 3
        lib.ref_channel_decode.argtypes = [C.c_int, _i32p]
        lib.ref_channel_encode.argtypes = [C.c_int] * 5
        lib.ref_voxel_decode.argtypes = [C.c_int, _i32p]
        lib.ref_voxel_encode.argtypes = [C.c_int] * 3
        lib.ref_trafo0.argtypes = [_f32p, C.c_int, C.c_int, C.c_int, _f32p]
        lib.ref_trafo1.argtypes = [_f32p, C.c_int, C.c_int, C.c_int, _f32p]
        lib.ref_intersection_length.argtypes = [_f32p, _f32p]
        lib.ref_intersection_length.restype = C.c_float
        lib.ref_intersection_length_devonly.argtypes = [_f32p, _f32p]
        lib.ref_intersection_length_devonly.restype = C.c_float
        lib.ref_workqueue.argtypes = [_i32p, C.c_int, _i32p, _i32p, C.c_longlong,
                                      C.POINTER(C.c_longlong)]
        lib.ref_workqueue.restype = C.c_longlong
        lib.ref_workqueue_bounded.argtypes = [_i32p, C.c_int, C.POINTER(C.c_int),
                                              C.POINTER(C.c_int), C.c_int, _i32p, _i32p]
        lib.ref_sm_value.argtypes = [C.c_int, C.c_int, C.c_int, _f32p]
        lib.ref_sm_value.restype = C.c_float
        lib.ref_coo_sort.argtypes = [_f32p, _i32p, _i32p, C.c_int]
        lib.ref_csr2ecsr.argtypes = [_i32p, _i32p, C.c_int, _i32p, C.c_int]
        lib.ref_divides.argtypes = [_f32p] * 3 + [C.c_int]
        lib.ref_divides_multiplies.argtypes = [_f32p] * 4 + [C.c_int]
        lib.ref_scales.argtypes = [_f32p, C.c_float, C.c_int]
        lib.ref_sum.argtypes = [_f32p, C.c_int]
        lib.ref_sum.restype = C.c_float

    def setup(self, p):
        s, g = p.setup, p.grid
        self.lib.ref_setup(s.pos0x, s.pos1x, s.na, s.n0z, s.n0y, s.n1z, s.n1y, s.da, s.segx,
                           s.segy, s.segz, *g.origin, *g.pitch, *g.n)

    def workqueue(self, rows):
        rows = np.ascontiguousarray(rows, np.int32)
        tot = C.c_longlong(0)
        self.lib.ref_workqueue(rows, len(rows), np.zeros(1, np.int32), np.zeros(1, np.int32), 0,
                               C.byref(tot))
        n = tot.value
        oc = np.zeros(max(n, 1), np.int32)
        ov = np.zeros(max(n, 1), np.int32)
        self.lib.ref_workqueue(rows, len(rows), oc, ov, n, C.byref(tot))
        return oc[:n], ov[:n]
