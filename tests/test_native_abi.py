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
    assert ctypes.sizeof(_native.FsgMlpWeights) == 12 * 8
    assert _native.FsgFreqPlan.pulse_spectrum.offset == 48
    assert ctypes.sizeof(_native.FsgDasParams) == 48
    assert _native.FsgDasParams.method.offset == 40


def test_struct_layouts_match_a_c_compiler(tmp_path):
    """Every struct the ctypes binding declares has the size and field offsets that a C
    compiler gives the declaration in include/fsgb300.h."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = [getattr(_native, n) for n in dir(_native)
               if n.startswith("Fsg") and isinstance(getattr(_native, n), type)
               and issubclass(getattr(_native, n), ctypes.Structure)]
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "fsgb300.h"', "int main(void) {"]
    for st in structs:
        lines.append(f'  printf("{st.__name__} %zu\\n", sizeof({st.__name__}));')
        for f in st._fields_:
            lines.append(f'  printf("{st.__name__}.{f[0]} %zu\\n", offsetof({st.__name__}, {f[0]}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    root = Path(__file__).resolve().parent.parent
    subprocess.run([cc, "-I", str(root / "include"), str(src), "-o", str(exe)], check=True)
    got = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                       check=True).stdout.splitlines())
    for st in structs:
        assert int(got[st.__name__]) == ctypes.sizeof(st), st.__name__
        for f in st._fields_:
            assert int(got[f"{st.__name__}.{f[0]}"]) == getattr(st, f[0]).offset, f"{st.__name__}.{f[0]}"
