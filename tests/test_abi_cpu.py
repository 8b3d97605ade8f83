"""CPU-side checks of the C ABI: the library builds for sm_103a, loads, and
exports every entry point include/*.h declares.  No kernel runs here."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import ROOT

HEADERS = [os.path.join(ROOT, "include", h) for h in sorted(os.listdir(os.path.join(ROOT, "include")))
           if h.endswith(".h")]


def declared_functions():
    names = set()
    for h in HEADERS:
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*(pdflow_[A-Za-z0-9_]+)\s*\(",
                             src, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_entry_points():
    names = declared_functions()
    for n in ("pdflow_create", "pdflow_push_frame", "pdflow_solve", "pdflow_read_flow", "pdflow_destroy"):
        assert n in names


def test_library_exports_every_declared_symbol(built_lib):
    missing = [n for n in declared_functions() if not hasattr(built_lib, n)]
    assert not missing, missing


def test_library_is_built_for_sm103a_only():
    from pdflow import build
    build.build()
    log = open(os.path.join(build.LIBDIR, "ptxas.log")).read() if os.path.exists(
        os.path.join(build.LIBDIR, "ptxas.log")) else ""
    if log:
        archs = set(re.findall(r"for '(sm_[0-9a-z]+)'", log))
        assert archs == {"sm_103a"}, archs


def test_default_params_are_the_reference_schedule(built_lib):
    from pdflow import default_params
    p = default_params(240)
    assert list(p.num_max_iter)[:5] == [40, 55, 70, 85, 100]
    p = default_params(480)
    assert list(p.num_max_iter) == [25, 40, 55, 70, 85, 100]
    assert abs(p.lambda_i - 0.04) < 1e-9 and abs(p.lambda_d - 0.35) < 1e-7 and p.mu == 75.0
    assert p.fovh == ctypes.c_float(3.141592653589793 * 62.5 / 180.0).value


def test_default_params_rejects_bad_rows(built_lib):
    from pdflow import _lib
    p = _lib.Params()
    assert built_lib.pdflow_default_params(100, ctypes.byref(p)) == _lib.ERR_ARG
    assert b"rows" in built_lib.pdflow_last_error()


def test_create_validates_arguments_before_touching_a_device(built_lib):
    from pdflow import _lib
    h = ctypes.c_void_p()
    assert built_lib.pdflow_create(100, 640, 480, None, ctypes.byref(h)) == _lib.ERR_ARG
    assert built_lib.pdflow_create(480, 320, 240, None, ctypes.byref(h)) == _lib.ERR_ARG   # rows > image
    assert built_lib.pdflow_create(240, 800, 600, None, ctypes.byref(h)) == _lib.ERR_ARG
    assert built_lib.pdflow_create(240, 320, 240, None, None) == _lib.ERR_ARG
    assert h.value is None


def test_null_handles_are_rejected(built_lib):
    from pdflow import _lib
    assert built_lib.pdflow_solve(None) == _lib.ERR_ARG
    assert built_lib.pdflow_read_flow(None, None, None, None) == _lib.ERR_ARG
    assert built_lib.pdflow_destroy(None) == _lib.OK
    assert built_lib.pdflow_debug_wait_timeout(None, 1000) == _lib.ERR_ARG


def test_cpp_host_class_compiles():
    """The C++ PD_flow class (the reference's PD_flow_opencv method names) builds
    against the C ABI."""
    src = os.path.join(ROOT, "pd-flow_gb300", "examples", "pd_flow_pair.cpp")
    out = os.path.join(ROOT, "pd-flow_gb300", "lib", "_build", "pd_flow_pair")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-fsyntax-only", "-I", os.path.join(ROOT, "include"),
                        "-I", os.path.join(ROOT, "pd-flow_gb300", "csrc"), src], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
