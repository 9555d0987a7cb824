"""The C-ABI library loads and exports every declared entry point (no
compute calls: there may be no GPU)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _declared():
    hdr = (ROOT / 'include' / 'pyfrb200.h').read_text()
    hdr = re.sub(r'/\*.*?\*/', '', hdr, flags=re.S)
    return sorted(set(re.findall(r'\b(b200_\w+)\s*\(', hdr)))


@pytest.fixture(scope='module')
def lib():
    import __graft_entry__ as ge
    ge.build_library()
    from pyfr_gb300.backend.lib import LIBPATH
    return ctypes.CDLL(str(LIBPATH))


def test_header_declares_entry_points():
    names = _declared()
    assert 'b200_mul_f64' in names and 'b200_rkvdh2_f64' in names
    assert len(names) > 40


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from pyfr_gb300.backend.lib import exported_symbols
    assert set(exported_symbols()) <= set(_declared())


def test_version_string(lib):
    lib.b200_version.restype = ctypes.c_char_p
    assert b'sm_103a' in lib.b200_version()
