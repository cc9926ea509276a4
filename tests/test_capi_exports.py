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


STRUCTS = {"epet_setup": "Setup", "epet_grid": "Grid", "epet_problem": "ProblemC",
           "epet_csr": "CsrC", "epet_csc": "CscC", "epet_csr16": "Csr16C",
           "epet_mlem_options": "MlemOptions"}


def test_struct_layout_matches_header(tmp_path):
    """The ctypes mirrors have the size and field offsets the C compiler
    gives the header's structs (a C program built with gcc prints them)."""
    import shutil
    import subprocess
    from epetreco_gb300 import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "epet_gb300.h"',
             "int main(void) {"]
    for cname, pyname in STRUCTS.items():
        lines.append(f'  printf("{pyname} size %zu\\n", sizeof({cname}));')
        for f, _ in getattr(_lib, pyname)._fields_:
            lines.append(f'  printf("{pyname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                    str(exe)], check=True)
    got = {}
    for ln in subprocess.run([str(exe)], check=True, capture_output=True,
                             text=True).stdout.splitlines():
        k, v = ln.rsplit(" ", 1)
        got[k] = int(v)
    for pyname in STRUCTS.values():
        T = getattr(_lib, pyname)
        assert got[f"{pyname} size"] == ctypes.sizeof(T), pyname
        for f, _ in T._fields_:
            assert got[f"{pyname} {f}"] == getattr(T, f).offset, (pyname, f)


def test_problem_layout_keeps_ray_mode_in_padding():
    """ray_mode sits between nrays and the 8-byte seed, where a struct without
    it has padding: the size and the seed's offset are those of the
    four-field struct, and a zero-initialised problem is the random generator."""
    from epetreco_gb300 import _lib

    class Four(ctypes.Structure):
        _fields_ = [("setup", _lib.Setup), ("grid", _lib.Grid), ("nrays", ctypes.c_int32),
                    ("seed", ctypes.c_uint64)]
    assert ctypes.sizeof(_lib.ProblemC) == ctypes.sizeof(Four)
    assert _lib.ProblemC.seed.offset == Four.seed.offset
    assert _lib.ProblemC().ray_mode == 0


def test_ray_mode_validation():
    from epetreco_gb300 import _lib
    from epetreco_gb300.problem import Problem, config
    L = _lib.lib()
    p = config("small")["problem"]
    assert p.ray_mode == 0 and p.with_rays("regular").ray_mode == 1
    ps = _lib.problem_struct(p.with_rays("regular"))
    assert ps.ray_mode == 1
    assert L.epet_problem_validate(ctypes.byref(ps)) == 0
    ps.ray_mode = 2
    assert L.epet_problem_validate(ctypes.byref(ps)) == 1
    assert b"ray_mode" in L.epet_last_error()
    with pytest.raises(ValueError):
        Problem(p.setup, p.grid, p.nrays, rays="uniform")


def test_constant_geometry_threads():
    """epet_set/get_constant_geometry (the shim's stand-in for the reference's
    cudaMemcpyToSymbol of grid_const/setup_const/nrays_const) from several
    threads at once: every read returns one whole problem that some thread
    wrote (no CUDA call is involved)."""
    import threading
    from epetreco_gb300 import _lib
    from epetreco_gb300.problem import config
    L = _lib.lib()
    base = _lib.problem_struct(config("small")["problem"])
    errors = []

    def run(k):
        s, g = _lib.Setup(), _lib.Grid()
        ctypes.pointer(s)[0] = base.setup
        ctypes.pointer(g)[0] = base.grid
        s.na = 1 + k  # na and nrays tie each write together
        for it in range(2000):
            if L.epet_set_constant_geometry(ctypes.byref(s), ctypes.byref(g), 100 + k) != 0:
                errors.append("set")
            out = _lib.ProblemC()
            if L.epet_get_constant_geometry(ctypes.byref(out)) != 0:
                errors.append("get")
            elif out.nrays - 100 != out.setup.na - 1 or out.seed != 1251 or out.ray_mode != 0:
                errors.append((out.nrays, out.setup.na))

    ts = [threading.Thread(target=run, args=(k,)) for k in range(4)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errors, errors[:5]


def test_shim_maps_ray_generators(tmp_path):
    """The shim's RayGen argument mapping, compiled (no run): a generator
    template shaped like the reference's ReguRayGen, defined after the shim
    as a driver including RayGenerators.hpp would, maps to EPET_RAYS_REGULAR;
    any other type (RandRayGen) to EPET_RAYS_RANDOM."""
    import shutil
    import subprocess
    cxx = shutil.which("g++")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
    if cxx is None or not os.path.exists(os.path.join(cuda_inc, "cusparse.h")):
        pytest.skip("no C++ compiler or CUDA headers")
    src = tmp_path / "shim_rays.cpp"
    src.write_text(
        '#include "epet_gb300_shim.hpp"\n'
        "template <typename T, typename MSTrafo0_inplace, typename MSTrafo1_inplace>\n"
        "struct ReguRayGen { int unused; };\n"
        "template <typename T, typename A, typename B> struct RandRayGen { int unused; };\n"
        "static_assert(epet_shim::ray_mode_of<ReguRayGen<float, int, long>>::value ==\n"
        "              EPET_RAYS_REGULAR, \"regular\");\n"
        "static_assert(epet_shim::ray_mode_of<RandRayGen<float, int, long>>::value ==\n"
        "              EPET_RAYS_RANDOM, \"random\");\n"
        "int main() { return 0; }\n")
    subprocess.run([cxx, "-std=c++17", "-fsyntax-only", "-I", os.path.join(ROOT, "include"),
                    "-I", cuda_inc, str(src)], check=True)
