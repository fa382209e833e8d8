"""The C ABI library (no GPU needed): it loads, exports every symbol include/gd2d.h
declares, and rejects invalid configurations before touching the device."""
import ctypes
import os
import re
import subprocess

import pytest

import golikov_2d_gb300 as g

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "gd2d.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(gd_[a-z0-9_]+)\s*\(", txt)))


def test_header_and_python_mirror_agree():
    assert set(declared_symbols()) == set(g.EXPORTS)


def test_library_exports_every_declared_symbol(gdlib):
    out = subprocess.run(["nm", "-D", "--defined-only", g.lib_path()], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\bT (gd_[a-z0-9_]+)$", out, flags=re.M))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    for s in declared_symbols():
        assert hasattr(gdlib, s)


def test_abi_version_and_status_strings(gdlib):
    assert gdlib.gd_abi_version() == 3
    assert gdlib.gd_status_string(0) == b"ok"
    assert gdlib.gd_status_string(1) == b"invalid argument"


def base():
    return g.Config(N=16, M=16, dx=1 / 16, dy=1 / 16, x0=1 / 32, y0=1 / 32, gamma=1.4, krit=0.4)


@pytest.mark.parametrize("mutate", [
    lambda c: setattr(c, "N", 2),
    lambda c: setattr(c, "M", 0),
    lambda c: setattr(c, "dx", 0.0),
    lambda c: setattr(c, "dy", float("nan")),
    lambda c: setattr(c, "gamma", 1.0),
    lambda c: setattr(c, "krit", -0.1),
    lambda c: setattr(c, "order", 3),
    lambda c: setattr(c, "method", 3),              # HLLD with Euler physics
    lambda c: setattr(c, "bc", (0, 1, 1, 1)),       # periodic on one side only
    lambda c: setattr(c, "bc", (1, 1, 9, 1)),
    lambda c: (setattr(c, "geometry", g.AXISYM), setattr(c, "y0", 0.0)),
    lambda c: (setattr(c, "physics", g.MHD), setattr(c, "method", 1)),
    lambda c: setattr(c, "mode", 7),
])
def test_invalid_config_rejected_without_device(gdlib, mutate):
    c = base()
    mutate(c)
    h = ctypes.c_void_p()
    st = gdlib.gd_create(ctypes.byref(c.cstruct()), ctypes.byref(h))
    assert st == 1 and not h.value


def test_config_layout_matches_header(tmp_path):
    """sizeof(gd_config) and every field's offset, from the C compiler, equal the ctypes
    mirror's (the Hancock fields were appended in ABI 3)."""
    fields = [f for f, _ in g.gd_config._fields_]
    src = tmp_path / "layout.c"
    src.write_text('#include <stddef.h>\n#include <stdio.h>\n#include "gd2d.h"\n'
                   "int main(void) {\n"
                   '  printf("%zu\\n", sizeof(gd_config));\n' +
                   "".join(f'  printf("%zu\\n", offsetof(gd_config, {f}));\n' for f in fields) +
                   "  return 0;\n}\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                    str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    assert got[0] == ctypes.sizeof(g.gd_config)
    assert got[1:] == [getattr(g.gd_config, f).offset for f in fields]


def hancock_base():
    from golikov_2d_gb300 import problems
    return problems.hancock_config(16, 16)


@pytest.mark.parametrize("mutate,status", [
    (lambda c: setattr(c, "scheme", 3), 1),
    (lambda c: setattr(c, "scheme", -1), 1),
    (lambda c: setattr(c, "x_max", 0.0), 1),
    (lambda c: setattr(c, "y_max", float("inf")), 1),
    (lambda c: setattr(c, "geometry", g.CARTESIAN), 5),       # Kernel_GKR is axisymmetric
    (lambda c: setattr(c, "method", g.METHOD_HLLC_MHD), 5),   # its faces are HLLD (metod 3)
    (lambda c: setattr(c, "bc", (g.BC_MIRROR_X, g.BC_OUTFLOW, g.BC_AXIS, g.BC_AMBIENT)), 5),
    (lambda c: (setattr(c, "physics", g.EULER), setattr(c, "method", g.METHOD_HLLC)), 5),
])
def test_hancock_config_checks_without_device(gdlib, mutate, status):
    c = hancock_base()
    mutate(c)
    h = ctypes.c_void_p()
    st = gdlib.gd_create(ctypes.byref(c.cstruct()), ctypes.byref(h))
    assert st == status and not h.value


def test_null_arguments_rejected(gdlib):
    assert gdlib.gd_create(None, None) == 1
    assert gdlib.gd_advance(None, 1, 0, None) == 1
    assert gdlib.gd_set_dt_policy(None, 0) == 1
    assert gdlib.gd_set_floor_limit(None, 0) == 1
    assert gdlib.gd_advance_to(None, 1.0, 10, 0, None, None) == 1
    assert gdlib.gd_step_ref(None, None, None, None, None, None, None, None, None, 0, 0, None) == 1
    assert gdlib.gd_probe_fp64_peak(None) == 1


def test_every_allocation_goes_through_the_counted_helpers():
    """gd_alloc_counts counts what the library's helpers allocate; that is every allocation
    only if no source calls the CUDA allocators directly.  The helpers themselves live in
    gd_api.cu."""
    csrc = os.path.join(ROOT, "golikov_2d_gb300", "csrc")
    pat = re.compile(r"(?<![\w:])(cudaMalloc\w*|cudaHostAlloc|cudaFree\w*|cudaMallocAsync)\s*\(")
    found = []
    for name in sorted(os.listdir(csrc)):
        if not name.endswith((".cu", ".cuh", ".h", ".cpp")):
            continue
        text = open(os.path.join(csrc, name)).read()
        text = re.sub(r"//[^\n]*|/\*.*?\*/", "", text, flags=re.S)  # comments
        for m in pat.finditer(text):
            found.append((name, m.group(1)))
    allowed = [("gd_api.cu", "cudaMalloc"), ("gd_api.cu", "cudaMallocHost"),
               ("gd_api.cu", "cudaFree"), ("gd_api.cu", "cudaFreeHost")]
    assert sorted(found) == sorted(allowed), found
