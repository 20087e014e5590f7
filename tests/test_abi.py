"""CPU checks of the C ABI: the library builds, loads, exports every function that
include/nspipe_gb300.h declares, and rejects invalid parameters before it
touches a GPU (no compute calls here)."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "nspipe_gb300.h")


@pytest.fixture(scope="module")
def L():
    import importlib
    import sys
    sys.path.insert(0, os.path.join(ROOT, "nspipe-gpu_gb300"))
    import build as nbuild  # nspipe-gpu_gb300/build.py
    nbuild.build()
    nsp = importlib.import_module("nspipe_gb300")
    return nsp


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|long long|const char\*)\s+(nsp_\w+)\s*\(", text, re.M)))


def test_header_declares_expected_api():
    names = declared_functions()
    for n in ("nsp_create", "nsp_setup", "nsp_step", "nsp_nonlinear", "nsp_lusolve", "nsp_load_state",
              "nsp_save_state", "nsp_set_state_device", "nsp_diag", "nsp_last_error", "nsp_destroy"):
        assert n in names


def test_library_exports_every_declared_symbol(L):
    lib = L.lib()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", L.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (nsp_\w+)", out))
    assert set(declared_functions()) <= exported
    assert set(L.EXPORTS) == set(declared_functions())


def test_default_params_match_reference_header(L):
    p = L.default_params()
    assert (p.NR, p.NT, p.NZ) == (48, 64, 257)          # head.h:16-18
    assert p.LT == 6.283185307179586 and p.LZ == 100.0  # head.h:21-22
    assert p.Re == 1850.0 and p.dt == 0.01 and p.d_im == 0.51
    assert p.maxit == 10 and p.tol == 5e-8 and p.sten == 7 and p.Qdes == 0.5


@pytest.mark.parametrize("field,value,needle", [("NT", 33, "NT"), ("NZ", 64, "NZ"), ("sten", 5, "sten"),
                                                ("NZ", 11, "2^a 3^b"), ("Re", -1.0, "Re"), ("NR", 4, "NR")])
def test_invalid_parameters_rejected_before_device_use(L, field, value, needle):
    p = L.make_params(48, 32, 65, 2000.0, 0.01, 2 * L.PI2)
    setattr(p, field, value)
    arr = (L.NspParams * 1)(p)
    h = ctypes.c_void_p()
    rc = L.lib().nsp_create(arr, 1, L.NSP_FP64, 0, ctypes.byref(h))
    assert rc == L.NSP_ERR_ARG
    msg = L.lib().nsp_last_error(h).decode()
    assert needle in msg
    L.lib().nsp_destroy(h)


def test_null_and_range_arguments(L):
    lib = L.lib()
    assert lib.nsp_create(None, 1, 0, 0, None) == L.NSP_ERR_ARG
    p = L.make_params(48, 32, 65, 2000.0, 0.01, 2 * L.PI2)
    h = ctypes.c_void_p()
    assert lib.nsp_create((L.NspParams * 1)(p), 1, 7, 0, ctypes.byref(h)) == L.NSP_ERR_ARG  # bad precision
    assert lib.nsp_step(None, 1, None) == L.NSP_ERR_ARG
    assert lib.nsp_destroy(None) == L.NSP_OK
