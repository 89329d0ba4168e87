"""The C-ABI library loads without a GPU, exports every symbol that
include/abie_gb300.h declares, and reports a missing device as an error
code instead of crashing or falling back to the CPU."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def _declared_functions():
    with open(os.path.join(ROOT, "include", "abie_gb300.h")) as fh:
        text = fh.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = "\n".join(l for l in text.splitlines() if not l.lstrip().startswith("#"))
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\([^;{]*\)\s*;", text)
    return sorted(set(n for n in names if n not in ("if", "while", "sizeof")))


def test_header_declares_reference_entry_points():
    names = set(_declared_functions())
    ref = {"initialize_code", "finalize_code", "set_state", "get_state", "get_model_time",
           "set_close_encounter_distance", "get_close_encounter_distance",
           "get_close_encounter_buffer", "get_collision_buffer", "reset_close_encounter_buffer",
           "reset_collision_buffer", "set_additional_forces", "integrator_gr", "integrator_wh",
           "integrator_rk", "calculate_energy", "ode_n_body_second_order",
           "calculate_accelerations", "integrator_gauss_radau15", "integrator_wisdom_holman"}
    assert ref <= names, ref - names


def test_library_exports_every_declared_symbol(built_lib):
    lib = ctypes.CDLL(built_lib)
    missing = [n for n in _declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_no_device_is_an_error_not_a_fallback(built_lib):
    import subprocess
    import sys
    # run in a child so this process keeps no CUDA state
    code = (
        "import ctypes,sys; lib=ctypes.CDLL(%r); "
        "rc=lib.initialize_code(ctypes.c_double(1.0),ctypes.c_double(0.0),ctypes.c_int(4),"
        "ctypes.c_int(1),ctypes.c_int(1),ctypes.c_int(-1)); print(rc)" % built_lib)
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120)
    assert out.stdout.strip() == "-1", out.stdout + out.stderr


def test_binding_reports_negative_codes():
    from abie_gb300.events import AbieError
    e = AbieError(-4, "x")
    assert e.code == -4 and "x" in str(e)
