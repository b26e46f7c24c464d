"""The C-ABI library loads and exports every symbol include/*.h declares (CPU only: no
compute call is made; the ctypes struct layouts are checked against the library's sizeof)."""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        names.update(re.findall(r"FF_API\s+[\w\s\*]+?\b(ff_\w+)\s*\(", text))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from factor_fields_gb300 import build
    from factor_fields_gb300 import _native as N
    build.build()
    return N.load()


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "ff_field_forward" in names and "ff_field_backward" in names and len(names) >= 8


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_bindings_cover_header(lib):
    from factor_fields_gb300 import _native as N
    assert set(declared_symbols()) == set(N.SIGNATURES), set(declared_symbols()) ^ set(N.SIGNATURES)


def test_struct_layouts_match(lib):
    from factor_fields_gb300 import _native as N
    assert lib.ff_abi_version() == 1
    for i, st in enumerate([N.FFField, N.FFMlp, N.FFMlpGrad, N.FFRender, N.FFProposal, N.FFAdamParam]):
        assert lib.ff_struct_size(i) == ctypes.sizeof(st), st.__name__
