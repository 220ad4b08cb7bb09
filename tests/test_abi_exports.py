"""The C-ABI library builds for sm_103a, loads, and exports every function the header declares."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    src = open(os.path.join(ROOT, 'include', 'gwfast_gb300.h')).read()
    src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
    return sorted(set(re.findall(r'^\s*(?:int|const char\*|void)\s+(gwf_\w+)\s*\(', src, flags=re.M)))


def test_header_declares_entry_points():
    names = declared()
    for n in ('gwf_ctx_create', 'gwf_snr', 'gwf_fisher', 'gwf_cov', 'gwf_detector_add'):
        assert n in names


def test_library_exports_all_declared_symbols():
    from gwfast_gb300 import _build, _lib
    path = _build.build()
    lib = ctypes.CDLL(path)
    for n in declared():
        assert hasattr(lib, n), n
    assert set(_lib.SIGNATURES) <= set(declared())
