"""The C-ABI library builds, loads without a GPU and exports every function that
include/grx.h declares (no compute call is made here)."""
import ctypes
import os
import re

from graspa_gb300 import build as B
from graspa_gb300 import grx

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "grx.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(grx_[a-z_0-9]+)\s*\(", src, flags=re.M)))


def test_header_lists_match_binding():
    assert set(declared_functions()) == set(grx.EXPORTS)


def test_library_exports_every_symbol():
    path = B.build()
    lib = ctypes.CDLL(path)
    missing = [f for f in declared_functions() if not hasattr(lib, f)]
    assert not missing, missing


def test_status_strings_without_gpu():
    L = grx.load()
    assert L.grx_status_string(0) == b"ok"
    assert L.grx_status_string(4) == b"device wait timed out"


def test_box_create_rejects_bad_desc():
    L = grx.load()
    d = grx.BoxDesc()
    d.ncomponents = 0
    h = ctypes.c_void_p()
    assert L.grx_box_create(ctypes.byref(d), ctypes.byref(h)) == 1
    assert b"ncomponents" in L.grx_last_error()
