"""CPU-side checks of the C ABI: the library builds for sm_103a, loads, and
exports every entry point include/*.h declares (no GPU calls)."""
import ctypes
import glob
import os
import re

import pytest

from tramonto_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        with open(h) as f:
            txt = f.read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?\w[\w\s\*]*?\b((?:tgpu|dft)_\w+)\s*\(", txt, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    path = build.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "tgpu_fill" in names and "tgpu_schur_apply" in names and len(names) > 20
    assert "dft_linprobmgr_insertonematrixvalue" in names and "dft_hardsphere_lin_prob_mgr_create" in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_errors_without_gpu_are_status_codes(lib):
    # a null geometry is rejected before any CUDA call
    lib.tgpu_create.restype = ctypes.c_int
    lib.tgpu_last_error.restype = ctypes.c_char_p
    h = ctypes.c_void_p()
    assert lib.tgpu_create(None, 0, ctypes.byref(h)) == -1
    assert b"null" in lib.tgpu_last_error()
