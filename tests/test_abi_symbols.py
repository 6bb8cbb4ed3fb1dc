"""The C-ABI library builds for sm_103a, loads without a GPU, and exports
every entry point include/lsdtt_gb300.h declares; without a device every
entry point reports LSDTT_GPU_ENODEV instead of computing on the CPU."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", f) for f in sorted(os.listdir(os.path.join(ROOT, "include")))
           if f.endswith(".h")]


def declared_functions():
    names = []
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"\b(lsdtt_gpu_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


@pytest.fixture(scope="module")
def libpath():
    from lsdtt_gb300 import build as B
    return B.build()


def test_header_declares_entry_points():
    names = declared_functions()
    assert "lsdtt_gpu_flow_build" in names and "lsdtt_gpu_fill_pits" in names
    assert len(names) >= 10


def test_library_exports_every_declared_symbol(libpath):
    lib = ctypes.CDLL(libpath)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_no_device_is_an_error_not_a_fallback(libpath):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    lib = ctypes.CDLL(libpath)
    lib.lsdtt_gpu_last_error.restype = ctypes.c_char_p
    assert lib.lsdtt_gpu_device_available() == 0
    h = ctypes.c_void_p()

    class Grid(ctypes.Structure):
        _fields_ = [("n_rows", ctypes.c_int32), ("n_cols", ctypes.c_int32), ("cell_size", ctypes.c_double),
                    ("no_data_value", ctypes.c_double), ("boundary_conditions", ctypes.c_char * 4)]

    g = Grid(4, 4, 10.0, -9999.0, b"oooo")
    assert lib.lsdtt_gpu_flow_create(ctypes.byref(g), ctypes.byref(h)) == 1  # LSDTT_GPU_ENODEV
    assert b"no CUDA device" in lib.lsdtt_gpu_last_error()
