"""The C-ABI library loads and exports every function declared in
include/*.h (no compute call; CPU only)."""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b(epet_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("epet_sm_build", "epet_workqueue_count", "epet_sm_values", "epet_coo_sort",
                 "epet_coo2csr", "epet_csr2ecsr", "epet_csrmv", "epet_divides",
                 "epet_divides_multiplies", "epet_scales", "epet_sum_f64", "epet_mlem_create"):
        assert must in names


def test_library_exports_all_declared():
    from epetreco_gb300 import build
    so = build.build()
    lib = ctypes.CDLL(so)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from epetreco_gb300 import _lib
    missing = [n for n in declared_functions() if n not in _lib.SIGNATURES]
    assert not missing, missing


def test_error_without_gpu_is_reported_not_raised():
    """Argument validation answers without touching the device."""
    from epetreco_gb300 import _lib
    from epetreco_gb300.problem import config
    L = _lib.lib()
    p = config("small")["problem"]
    ps = _lib.problem_struct(p)
    ps.nrays = 0
    assert L.epet_problem_validate(ctypes.byref(ps)) == 1
    assert b"nrays" in L.epet_last_error()
    ps.nrays = 10
    assert L.epet_problem_validate(ctypes.byref(ps)) == 0
