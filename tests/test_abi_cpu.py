"""CPU checks of the C ABI: the library loads and exports every symbol the header declares."""
import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, 'include', 'hcipy_gb300.h')


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r'HX_API\s+[\w\s\*]+?\b(hx_\w+)\s*\(', text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert 'hx_mft_plan_create' in syms and 'hx_mft_execute' in syms and 'hx_last_error' in syms
    assert len(syms) >= 8


def test_library_exports_every_declared_symbol():
    from hcipy_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip('library not built (run __graft_entry__.build())')
    lib = ctypes.CDLL(_lib.LIB_PATH)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    # The Python binding covers exactly the declared entry points.
    assert sorted(_lib.SIGNATURES) == declared_symbols()


def test_status_calls_without_gpu():
    from hcipy_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip('library not built')
    lib = _lib.load()
    assert lib.hx_version() >= 100
    assert lib.hx_launch_count() >= 0
    # Argument validation happens before any CUDA call.
    handle = ctypes.c_void_p()
    rc = lib.hx_mft_plan_create(0, 1, 1, 1, None, None, None, None, None, None, None, None, 0, 0, None,
                                ctypes.byref(handle))
    assert rc == _lib.HX_ERR_INVALID
    assert b'dimensions' in lib.hx_last_error()
    with pytest.raises(ValueError):
        _lib.check(rc)
