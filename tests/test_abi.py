"""The C-ABI library: builds for sm_103a, loads, and exports every symbol that
include/meshopt_gb300.h declares (no compute calls: this runs without a GPU)."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib_path():
    from meshoptimizer_gb300 import LIB_PATH, build

    build.build()
    assert os.path.isfile(LIB_PATH)
    return LIB_PATH


def header_symbols():
    text = open(os.path.join(ROOT, "include", "meshopt_gb300.h")).read()
    return sorted(set(re.findall(r"MESHOPTGPU_API\s+[\w\s\*]+?\b(\w+)\s*\(", text)))


def test_header_declares_dropin_signatures():
    syms = header_symbols()
    for name in ("meshopt_simplify", "meshopt_simplifyWithAttributes", "meshopt_simplifyScale"):
        assert name in syms


def test_library_exports_every_declared_symbol(lib_path):
    import meshoptimizer_gb300 as mg

    lib = C.CDLL(lib_path)
    syms = header_symbols()
    assert sorted(syms) == sorted(mg.EXPORTS)
    for s in syms:
        assert hasattr(lib, s), s


def test_library_exports_nothing_else(lib_path):
    import subprocess

    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if " T " in l}
    assert exported == set(header_symbols())
