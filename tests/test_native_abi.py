"""The C-ABI library builds, loads, and exports exactly the entry points include/fsgb300.h
declares -- no compute calls (CPU only)."""

import ctypes
import re
from pathlib import Path

import pytest

from fastsimus_gb300 import _native, build

HEADER = Path(__file__).resolve().parent.parent / "include" / "fsgb300.h"


def _declared():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fsg_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _native.load()


def test_header_declares_expected_entry_points():
    decl = _declared()
    assert "fsg_simus" in decl and "fsg_pfield" in decl and "fsg_last_error_string" in decl


def test_library_exports_every_declared_symbol(lib):
    for name in _declared():
        assert hasattr(lib, name), f"{name} declared in fsgb300.h but not exported"


def test_python_binding_covers_header(lib):
    assert sorted(_native.exported_symbols()) == _declared()


def test_abi_version(lib):
    assert lib.fsg_abi_version() == _native.ABI_VERSION


def test_struct_layouts_match_header():
    # offsets of the C structs (x86-64 / aarch64 LP64 alignment rules are the same)
    assert ctypes.sizeof(_native.FsgProbe) == 56
    assert _native.FsgProbe.baffle_impedance.offset == 48
    assert ctypes.sizeof(_native.FsgMedium) == 16
    assert ctypes.sizeof(_native.FsgFreqPlan) == 64
    assert ctypes.sizeof(_native.FsgMlpWeights) == 11 * 8
    assert _native.FsgFreqPlan.pulse_spectrum.offset == 48
    assert ctypes.sizeof(_native.FsgDasParams) == 48
    assert _native.FsgDasParams.method.offset == 40
