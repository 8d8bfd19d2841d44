"""The C-ABI library loads and exports every symbol the header declares (CPU only)."""
import ctypes
import os
import re

from tianxin_gb300 import _lib

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")


def declared_symbols():
    names = set()
    for fn in os.listdir(HEADER):
        if fn.endswith(".h"):
            txt = open(os.path.join(HEADER, fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"^\s*(?:int|void|const char\*)\s+(tx_\w+)\s*\(", txt, flags=re.M))
    return names


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    names = declared_symbols()
    assert len(names) >= 20
    for n in sorted(names):
        assert hasattr(lib, n), n


def test_python_signatures_cover_header():
    assert declared_symbols() <= set(_lib.SIGNATURES)


def test_no_device_needed_to_describe_a_mesh():
    lib = _lib.load()
    from tianxin_gb300 import _abi
    d = _abi.mesh_desc((2, 2, 2))
    h = ctypes.c_void_p()
    assert lib.tx_mesh_create(ctypes.byref(d), ctypes.byref(h)) == 0
    lib.tx_destroy(h)
    bad = _abi.mesh_desc((2, 2, 2))
    bad.bx = 0
    assert lib.tx_mesh_create(ctypes.byref(bad), ctypes.byref(h)) == _abi.TX_EINVAL
