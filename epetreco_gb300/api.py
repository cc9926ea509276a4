"""Host-side mirror of the reference's operator surface for the MLEM hot path.

Names, argument meaning and order follow the reference headers so drivers
read like ``reco.cu`` / ``backprojection.cu``; buffers are torch CUDA tensors
(device memory and streams only -- every computation runs in
``libepet_gb300.so``).  Errors raise ``EpetError`` (the reference throws
``cudaException`` from ``HANDLE_ERROR``, CUDA_HandleError.hpp:17-31).

  reference (file:line)                         here
  systemMatrixCalculation (wrappers.hpp:166-247)  systemMatrixCalculation
  getWorkqueue (getWorkqueue.hpp:187-223)         getWorkqueue
  getSystemMatrixFromWorkqueue (...Workqueue.cu)   getSystemMatrixFromWorkqueue
  cooSort (cooSort.hpp:53-71)                     cooSort
  convertCoo2Csr (cusparseWrapper.hpp:38-45)      convertCoo2Csr
  convertCsr2Ecsr (convertCsr2Ecsr.hpp:34-47)     convertCsr2Ecsr
  CSRmv<float> (csrmv.hpp:25-36)                  CSRmv
  divides/dividesMultiplies/scales/sum            same names
  (mlemOperations.hpp:22-139)
  nInChunk/chunkPtr/nChunks (wrappers.hpp:410-446) same names
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import torch

from . import _lib
from ._lib import (Csr16C, CscC, CsrC, EpetError, MlemOptions, ProblemC, check, lib,
                   problem_struct)

NON_TRANSPOSE = 0
TRANSPOSE = 1


def _ptr(t: torch.Tensor | None):
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError("expected a contiguous tensor")
    return C.c_void_p(t.data_ptr())


def _stream(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def _i32(t):
    return t.to(torch.int32).contiguous()


@dataclass
class Csr:
    """CSR over a measurement list (the reference's ECSR)."""
    row_ptr: torch.Tensor  # int64 [m+1]
    col: torch.Tensor      # int32 [nnz]
    val: torch.Tensor      # float32 [nnz]
    n: int                 # columns (voxels)

    @property
    def m(self) -> int:
        return self.row_ptr.numel() - 1

    @property
    def nnz(self) -> int:
        return self.col.numel()

    def cstruct(self) -> CsrC:
        return CsrC(self.m, self.n, self.nnz, self.row_ptr.data_ptr(),
                    self.col.data_ptr() if self.nnz else None,
                    self.val.data_ptr() if self.nnz else None)


@dataclass
class Csc:
    col_ptr: torch.Tensor
    row: torch.Tensor
    val: torch.Tensor
    m: int

    @property
    def n(self) -> int:
        return self.col_ptr.numel() - 1

    @property
    def nnz(self) -> int:
        return self.row.numel()

    def cstruct(self) -> CscC:
        return CscC(self.m, self.n, self.nnz, self.col_ptr.data_ptr(),
                    self.row.data_ptr() if self.nnz else None,
                    self.val.data_ptr() if self.nnz else None)


# ---------------------------------------------------------------- geometry

def trig_table(p) -> torch.Tensor:
    out = torch.empty(2 * p.setup.na, dtype=torch.float32, device="cuda")
    check(lib().epet_trig_table(C.byref(problem_struct(p)), _ptr(out), _stream()))
    return out


def dump_uniforms(p, rows: torch.Tensor) -> torch.Tensor:
    rows = _i32(rows)
    out = torch.empty((rows.numel(), p.nrays, 6), dtype=torch.float32, device="cuda")
    check(lib().epet_dump_uniforms(C.byref(problem_struct(p)), _ptr(rows), rows.numel(),
                                   _ptr(out), _stream()))
    return out


def rays(p, rows: torch.Tensor) -> torch.Tensor:
    rows = _i32(rows)
    out = torch.empty((rows.numel(), p.nrays, 6), dtype=torch.float32, device="cuda")
    check(lib().epet_rays(C.byref(problem_struct(p)), _ptr(rows), rows.numel(), _ptr(out),
                          _stream()))
    return out


# --------------------------------------------------------- system matrix

def getWorkqueue(p, rows: torch.Tensor):
    """All candidate (channel, voxel) pairs of the listed channels, list-major
    and voxel-minor.  Returns (cnl int32, vxl int32, row_ptr int64)."""
    rows = _i32(rows)
    m = rows.numel()
    cnt = torch.empty(m + 1, dtype=torch.int64, device="cuda")
    total = C.c_int64(0)
    PS = C.byref(problem_struct(p))
    check(lib().epet_workqueue_count(PS, _ptr(rows), m, _ptr(cnt), C.byref(total), _stream()))
    off = torch.zeros(m + 1, dtype=torch.int64, device="cuda")
    off[1:] = torch.cumsum(cnt[:m], 0)
    n = total.value
    cnl = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    vxl = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    check(lib().epet_workqueue_fill(PS, _ptr(rows), m, _ptr(off), _ptr(cnl), _ptr(vxl),
                                    _stream()))
    return cnl[:n], vxl[:n], off


def getSystemMatrixFromWorkqueue(p, rows: torch.Tensor, row_ptr: torch.Tensor,
                                 vxl: torch.Tensor) -> torch.Tensor:
    """Element values for a row-grouped workqueue, bit-identical to the
    reference's per-channel-seeded kernel."""
    rows = _i32(rows)
    val = torch.empty(max(vxl.numel(), 1), dtype=torch.float32, device="cuda")
    check(lib().epet_sm_values(C.byref(problem_struct(p)), _ptr(rows), rows.numel(),
                               _ptr(row_ptr.contiguous()), _ptr(_i32(vxl)), _ptr(val), None, 0,
                               _stream()))
    return val[:vxl.numel()]


def systemMatrixCalculation(p, rows: torch.Tensor, max_row_nnz: int = 0,
                            cap: int | None = None) -> Csr:
    """Fused build of the system matrix rows of the listed channels (CSR,
    columns ascending, zero values dropped).  Synchronous."""
    rows = _i32(rows)
    m = rows.numel()
    PS = C.byref(problem_struct(p))
    row_ptr = torch.empty(m + 1, dtype=torch.int64, device="cuda")
    nnz = C.c_int64(0)
    if cap is None:
        # first pass sizes the output
        cs = CsrC(m, p.nvoxels, 0, row_ptr.data_ptr(), None, None)
        st = lib().epet_sm_build(PS, _ptr(rows), m, C.byref(cs), 0, C.byref(nnz),
                                 int(max_row_nnz), None, 0, _stream())
        if st not in (_lib.EPET_OK, 2):
            check(st)
        cap = nnz.value
    col = torch.empty(max(cap, 1), dtype=torch.int32, device="cuda")
    val = torch.empty(max(cap, 1), dtype=torch.float32, device="cuda")
    cs = CsrC(m, p.nvoxels, 0, row_ptr.data_ptr(), col.data_ptr(), val.data_ptr())
    check(lib().epet_sm_build(PS, _ptr(rows), m, C.byref(cs), cap, C.byref(nnz),
                              int(max_row_nnz), None, 0, _stream()))
    n = nnz.value
    return Csr(row_ptr, col[:n], val[:n], p.nvoxels)


def project_forward(p, rows, x, max_row_nnz: int = 0) -> torch.Tensor:
    """Matrix-free y = A x (chords recomputed, nothing stored)."""
    rows = _i32(rows)
    y = torch.empty(rows.numel(), dtype=torch.float32, device="cuda")
    check(lib().epet_project_forward(C.byref(problem_struct(p)), _ptr(rows), rows.numel(),
                                     _ptr(x.contiguous()), _ptr(y), int(max_row_nnz), None, 0,
                                     _stream()))
    return y


def project_back(p, rows, e, c=None, max_row_nnz: int = 0) -> torch.Tensor:
    """Matrix-free c += A^T e."""
    rows = _i32(rows)
    if c is None:
        c = torch.zeros(p.nvoxels, dtype=torch.float32, device="cuda")
    check(lib().epet_project_back(C.byref(problem_struct(p)), _ptr(rows), rows.numel(),
                                  _ptr(e.contiguous()), _ptr(c), int(max_row_nnz), None, 0,
                                  _stream()))
    return c


def project_mlem(p, rows, x, y, c64=None, ybar=None, max_row_nnz: int = 0):
    """One matrix-free MLEM pass: ybar = A x, c64 += A^T (y / ybar) in fp64.
    Returns (c64, ybar)."""
    rows = _i32(rows)
    if c64 is None:
        c64 = torch.zeros(p.nvoxels, dtype=torch.float64, device="cuda")
    if ybar is None:
        ybar = torch.empty(rows.numel(), dtype=torch.float32, device="cuda")
    check(lib().epet_project_mlem(C.byref(problem_struct(p)), _ptr(rows), rows.numel(),
                                  _ptr(x.contiguous()), _ptr(y.to(torch.float32).contiguous()),
                                  _ptr(ybar), _ptr(c64), int(max_row_nnz), None, 0, _stream()))
    return c64, ybar


def sensitivity(p, rows=None, max_row_nnz: int = 0, return_f64: bool = False):
    """s = column sums of A over the listed channels (all channels by
    default), fp64 accumulation, normalised to sum 1."""
    if rows is None:
        rows = torch.arange(p.nchannels, dtype=torch.int32, device="cuda")
    rows = _i32(rows)
    s = torch.empty(p.nvoxels, dtype=torch.float32, device="cuda")
    s64 = torch.empty(p.nvoxels, dtype=torch.float64, device="cuda")
    check(lib().epet_sensitivity(C.byref(problem_struct(p)), _ptr(rows), rows.numel(), _ptr(s),
                                 _ptr(s64), int(max_row_nnz), None, 0, _stream()))
    return (s, s64) if return_f64 else s


# ------------------------------------------------------------ sparse formats

def cooSort(val: torch.Tensor, row: torch.Tensor, col: torch.Tensor) -> None:
    """In-place stable sort of COO triples by (row, col)."""
    for t, dt in ((val, torch.float32), (row, torch.int32), (col, torch.int32)):
        if t.dtype != dt or not t.is_contiguous():
            raise ValueError("cooSort expects contiguous float32 val, int32 row/col")
    check(lib().epet_coo_sort(_ptr(val), _ptr(row), _ptr(col), val.numel(), None, 0, _stream()))


def convertCoo2Csr(row: torch.Tensor, nnz: int, m: int) -> torch.Tensor:
    csr = torch.empty(m + 1, dtype=torch.int64, device="cuda")
    check(lib().epet_coo2csr(_ptr(_i32(row)), int(nnz), int(m), _ptr(csr), _stream()))
    return csr


def convertCsr2Ecsr(yRowId: torch.Tensor, nnzr: int, csr: torch.Tensor, m: int) -> torch.Tensor:
    ecsr = torch.empty(nnzr + 1, dtype=torch.int64, device="cuda")
    check(lib().epet_csr2ecsr(_ptr(ecsr), _ptr(_i32(yRowId)), int(nnzr),
                              _ptr(csr.to(torch.int64).contiguous()), int(m), _stream()))
    return ecsr


def csr_to_csc(a: Csr) -> Csc:
    col_ptr = torch.empty(a.n + 1, dtype=torch.int64, device="cuda")
    row = torch.empty(max(a.nnz, 1), dtype=torch.int32, device="cuda")
    val = torch.empty(max(a.nnz, 1), dtype=torch.float32, device="cuda")
    cc = CscC(a.m, a.n, a.nnz, col_ptr.data_ptr(), row.data_ptr(), val.data_ptr())
    ca = a.cstruct()
    check(lib().epet_csr_to_csc(C.byref(ca), C.byref(cc), None, 0, _stream()))
    return Csc(col_ptr, row[:a.nnz], val[:a.nnz], a.m)


# ---------------------------------------------------------------------- SpMV

def CSRmv(transA: int, A: Csr, x: torch.Tensor, alpha: float = 1.0, beta: float = 0.0,
          y: torch.Tensor | None = None, At: Csc | None = None) -> torch.Tensor:
    """y = alpha*op(A)*x + beta*y.  The transpose uses the column-major copy
    when given (scatter-free), else fp32 atomics."""
    out_len = A.n if transA else A.m
    if y is None:
        y = torch.zeros(out_len, dtype=torch.float32, device="cuda")
    ca = A.cstruct()
    cc = At.cstruct() if At is not None else None
    check(lib().epet_csrmv(int(transA), C.byref(ca), C.byref(cc) if cc else None, float(alpha),
                           _ptr(x.contiguous()), float(beta), _ptr(y), _stream()))
    return y


# ------------------------------------------------------ 16-bit value storage

BF16, FP16 = 1, 2
# layouts of a reconstruction's stored matrix (epet_mlem_options.layout)
LAYOUT_AUTO, LAYOUT_GROUPED, LAYOUT_CSC = 0, 1, 2


@dataclass
class Csr16:
    """16-bit storage of a CSR: rows in chunks of 8 entries with a 32-bit
    column base per chunk, 16-bit column offsets, BF16/FP16 values and an FP32
    scale per row (about 4.5 bytes per stored entry)."""
    row_ptr: torch.Tensor  # int64 [m+1], stored entries (multiples of 8)
    base: torch.Tensor     # int32 [capacity / 8]
    scale: torch.Tensor    # float32 [m]
    delta: torch.Tensor    # int16 [capacity]
    q: torch.Tensor        # int16 [capacity]
    n: int
    fmt: int
    stored: int            # entries written (escape entries included)

    @property
    def m(self) -> int:
        return self.row_ptr.numel() - 1

    def cstruct(self) -> Csr16C:
        return Csr16C(self.m, self.n, self.delta.numel(), self.row_ptr.data_ptr(),
                      self.base.data_ptr(), self.scale.data_ptr(), self.delta.data_ptr(),
                      self.q.data_ptr(), self.fmt)


def compress(A: Csr, fmt: int = BF16) -> Csr16:
    """The 16-bit form of A (epet_csr16_count + epet_csr_compress)."""
    m = A.m
    ca = A.cstruct()
    cnt = torch.empty(m + 1, dtype=torch.int64, device="cuda")
    n16 = C.c_int64(0)
    check(lib().epet_csr16_count(C.byref(ca), _ptr(cnt), C.byref(n16), _stream()))
    cap = max(n16.value, 8)
    out = Csr16(torch.empty(m + 1, dtype=torch.int64, device="cuda"),
                torch.empty(cap // 8, dtype=torch.int32, device="cuda"),
                torch.empty(max(m, 1), dtype=torch.float32, device="cuda"),
                torch.zeros(cap, dtype=torch.int16, device="cuda"),
                torch.zeros(cap, dtype=torch.int16, device="cuda"), A.n, int(fmt), n16.value)
    c16 = out.cstruct()
    check(lib().epet_csr_compress(C.byref(ca), int(fmt), C.byref(c16), _stream()))
    return out


def csr16_mv(A: Csr16, x: torch.Tensor, alpha: float = 1.0, beta: float = 0.0,
             y: torch.Tensor | None = None) -> torch.Tensor:
    """y = alpha * A x + beta * y over the 16-bit form (FP32 accumulation)."""
    if y is None:
        y = torch.zeros(A.m, dtype=torch.float32, device="cuda")
    c16 = A.cstruct()
    check(lib().epet_csr16_mv(C.byref(c16), float(alpha), _ptr(x.contiguous()), float(beta),
                              _ptr(y), _stream()))
    return y


def csc_as_csr(At: Csc) -> Csr:
    """The column-major copy viewed as the CSR of the transpose."""
    return Csr(At.col_ptr, At.row, At.val, At.m)


# ---------------------------------------------------------- MLEM operations

def divides(result, dividend, divisor, n: int | None = None) -> None:
    n = dividend.numel() if n is None else n
    check(lib().epet_divides(_ptr(result), _ptr(dividend), _ptr(divisor), n, _stream()))


def dividesMultiplies(result, a, b, c, n: int | None = None) -> None:
    n = a.numel() if n is None else n
    check(lib().epet_divides_multiplies(_ptr(result), _ptr(a), _ptr(b), _ptr(c), n, _stream()))


def scales(x, alpha: float, n: int | None = None) -> None:
    n = x.numel() if n is None else n
    check(lib().epet_scales(_ptr(x), float(alpha), n, _stream()))


def sum(x, n: int | None = None) -> float:  # noqa: A001 - reference name
    """Sum in fp64 on the device; returns a host value (synchronising), as the
    reference's thrust::reduce does."""
    n = x.numel() if n is None else n
    out = torch.empty(1, dtype=torch.float64, device="cuda")
    check(lib().epet_sum_f64(_ptr(x), n, _ptr(out), _stream()))
    return float(out.item())


# ------------------------------------------------------------ chunk helpers

def nInChunk(idChunk: int, nAll: int, nFullChunk: int) -> int:
    if idChunk < (nAll + nFullChunk - 1) // nFullChunk:
        if idChunk < nAll // nFullChunk:
            return nFullChunk
        return nAll % nFullChunk
    return 0


def chunkPtr(chunkId: int, nFullChunk: int) -> int:
    return chunkId * nFullChunk


def nChunks(maxNnz: int, maxNChunk: int) -> int:
    return (maxNnz + maxNChunk - 1) // maxNChunk


# --------------------------------------------------------------- MLEM driver

def trim_memory(keep_bytes: int = 0) -> None:
    """Returns the library's reserved device memory above keep_bytes."""
    check(lib().epet_trim_memory(int(keep_bytes)))


def debug_fail_allocations(after: int) -> None:
    """Fault injection for tests: after `after` more device allocations the
    library's allocations fail (EPET_ERR_CUDA) until called with -1."""
    check(lib().epet_debug_fail_allocations(int(after)))


def build_counters() -> dict:
    """Rows of system-matrix builds since load that were redone with their
    exact window size, and rows on the per-candidate path."""
    o, e = C.c_int64(0), C.c_int64(0)
    check(lib().epet_build_counters(C.byref(o), C.byref(e)))
    return {"overflow_rows": o.value, "exact_rows": e.value}


def ray_steps(p, rows, per_row: bool = False):
    """Grid cells crossed by all rays of the listed channels (the walk's
    work); with per_row, also the int64 count of each row."""
    rows = _i32(rows)
    n = C.c_int64(0)
    rs = torch.empty(rows.numel(), dtype=torch.int64, device="cuda") if per_row else None
    check(lib().epet_ray_steps(C.byref(problem_struct(p)), _ptr(rows), rows.numel(), _ptr(rs),
                               C.byref(n), _stream()))
    return (n.value, rs) if per_row else n.value


class Mlem:
    """One reconstruction on the device (reco.cu's loop): the system matrix
    of the measured rows is built once at construction.  The rows may come in
    any order; they are stored in crystal-pair order (a bijective key of the
    channel), so a shuffled list gives the same object."""

    def __init__(self, p, rows, y, s, use_graph: bool = True, max_row_nnz: int = 0,
                 value_format: int = 0, autotune: bool = False, matrix_free: bool = False,
                 layout: int = LAYOUT_AUTO):
        """``matrix_free=True`` stores no matrix: every iteration recomputes
        the chords in one walk per row (the reference's schedule of a matrix
        rebuilt in every iteration)."""
        self.p = p
        rows = _i32(rows)
        y = y.to(torch.float32).contiguous()
        s = s.to(torch.float32).contiguous()
        self._h = C.c_void_p()
        opt = MlemOptions(int(max_row_nnz), 1 if use_graph else 0, int(value_format),
                          1 if autotune else 0, 1 if matrix_free else 0, int(layout))
        check(lib().epet_mlem_create(C.byref(problem_struct(p)), _ptr(rows), _ptr(y),
                                     rows.numel(), _ptr(s), C.byref(opt), C.byref(self._h),
                                     _stream()))

    def iterate(self, nit: int, loglik: bool = False):
        ll = C.c_double(0.0)
        check(lib().epet_mlem_iterate(self._h, int(nit), C.byref(ll) if loglik else None,
                                      _stream()))
        return ll.value if loglik else None

    def correction(self, c: torch.Tensor | None = None) -> torch.Tensor:
        """c = A^T (y / A x) over this object's rows; the image is unchanged
        (row-sharded reconstructions sum c over the shards, then update)."""
        if c is None:
            c = torch.empty(self.p.nvoxels, dtype=torch.float32, device="cuda")
        check(lib().epet_mlem_correction(self._h, _ptr(c), _stream()))
        return c

    def update(self, c: torch.Tensor) -> None:
        """x = x*c/s (s == 0 -> 1), then x /= sum(x)."""
        check(lib().epet_mlem_update(self._h, _ptr(c.to(torch.float32).contiguous()), _stream()))

    def loglik(self) -> float:
        """FP64 Poisson log-likelihood of the last forward projection."""
        ll = C.c_double(0.0)
        check(lib().epet_mlem_loglik(self._h, C.byref(ll), _stream()))
        return ll.value

    def image(self) -> torch.Tensor:
        """A copy of the current image (float32, V)."""
        out = torch.empty(self.p.nvoxels, dtype=torch.float32, device="cuda")
        check(lib().epet_mlem_get_image(self._h, _ptr(out), _stream()))
        return out

    def set_image(self, x: torch.Tensor) -> None:
        check(lib().epet_mlem_set_image(self._h, _ptr(x.to(torch.float32).contiguous()),
                                        _stream()))

    def stats(self):
        nnz, b = C.c_int64(0), C.c_int64(0)
        check(lib().epet_mlem_stats(self._h, C.byref(nnz), C.byref(b)))
        return {"nnz": nnz.value, "bytes_per_iteration": b.value}

    def plan(self):
        """Launch shapes of the products: {"forward": (G, U, grid), "transpose": ...}."""
        pl = (C.c_int32 * 6)()
        check(lib().epet_mlem_plan(self._h, pl))
        return {"forward": tuple(pl[0:3]), "transpose": tuple(pl[3:6])}

    def checkpoint(self, path, iteration: int) -> None:
        """The image as the reference's "density" file (its grid attributes)
        plus an int attribute "iteration" (the iterations done), the restart
        point that reco.cu's "<it>_<out>" files are (reco.cu:284-291)."""
        from . import h5
        h5.write_checkpoint(path, self.image().cpu().numpy(), self.p.grid, iteration)

    def resume(self, path) -> int:
        """Sets the image from a checkpoint file and returns its iteration
        count (0 for a plain "density" file without one)."""
        import torch
        from . import h5
        x, _, it = h5.read_checkpoint(path)
        self.set_image(torch.from_numpy(x.ravel()).cuda())
        return it

    @property
    def layout(self) -> int:
        """LAYOUT_GROUPED or LAYOUT_CSC (-1 for a matrix-free object)."""
        v = C.c_int32(0)
        check(lib().epet_mlem_layout(self._h, C.byref(v)))
        return v.value

    def close(self):
        if self._h and getattr(self, "_owner", None) is None:
            lib().epet_mlem_destroy(self._h)
        self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MlemBatch:
    """Many independent reconstructions iterated together: each step of an
    iteration is one launch over all problems, the iteration one CUDA graph.
    ``problems`` is a list of (Problem, rows, y, s) with device tensors."""

    def __init__(self, problems, use_graph: bool = True, autotune: bool = True,
                 max_row_nnz: int = 0):
        n = len(problems)
        self.ps = [q[0] for q in problems]
        self._keep = []
        structs = (ProblemC * n)(*[problem_struct(q[0]) for q in problems])
        rows_p, m, y_p, s_p = (C.c_void_p * n)(), (C.c_int64 * n)(), (C.c_void_p * n)(), \
            (C.c_void_p * n)()
        for i, (p, rows, y, s) in enumerate(problems):
            rows, y, s = _i32(rows), y.to(torch.float32).contiguous(), \
                s.to(torch.float32).contiguous()
            self._keep += [rows, y, s]
            rows_p[i], y_p[i], s_p[i] = rows.data_ptr(), y.data_ptr(), s.data_ptr()
            m[i] = rows.numel()
        self._h = C.c_void_p()
        opt = MlemOptions(int(max_row_nnz), 1 if use_graph else 0, 0, 1 if autotune else 0)
        check(lib().epet_mlem_batch_create(n, C.byref(structs), rows_p, m, y_p, s_p,
                                           C.byref(opt), C.byref(self._h), _stream()))
        self._keep = []

    def iterate(self, nit: int, loglik: bool = False):
        ll = (C.c_double * len(self.ps))()
        check(lib().epet_mlem_batch_iterate(self._h, int(nit), ll if loglik else None,
                                            _stream()))
        return list(ll) if loglik else None

    def member(self, i: int) -> "Mlem":
        """Problem i as a single reconstruction (a view owned by the batch)."""
        h = lib().epet_mlem_batch_member(self._h, int(i))
        if not h:
            raise EpetError(lib().epet_last_error().decode())
        v = Mlem.__new__(Mlem)
        v.p, v._h, v._owner = self.ps[i], C.c_void_p(h), self
        return v

    def image(self, i: int) -> torch.Tensor:
        out = torch.empty(self.ps[i].nvoxels, dtype=torch.float32, device="cuda")
        check(lib().epet_mlem_batch_get_image(self._h, int(i), _ptr(out), _stream()))
        return out

    def stats(self):
        nnz, b = C.c_int64(0), C.c_int64(0)
        pl = (C.c_int32 * 6)()
        check(lib().epet_mlem_batch_stats(self._h, C.byref(nnz), C.byref(b), pl))
        return {"nnz": nnz.value, "bytes_per_iteration": b.value,
                "plan": {"forward": tuple(pl[0:3]), "transpose": tuple(pl[3:6])}}

    def close(self):
        if self._h:
            lib().epet_mlem_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
