"""The drop-in at link time (no GPU needed): compiled callers resolve every simplifier symbol
from libmeshopt_gb300.so alone.

* a C99 program that includes only include/meshopt_gb300.h builds and links (the header is
  valid C and the library exports what it declares);
* a C++ program written against the reference's own meshoptimizer.h, calling its 32-bit
  entry points and its header-only 16-bit templates, links with libmeshopt_gb300.so in place
  of libmeshoptimizer (only where the reference checkout is present).
"""
import os
import shutil
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DROPIN = os.path.join(ROOT, "tests", "dropin")


@pytest.fixture(scope="module")
def libdir():
    from meshoptimizer_gb300 import LIB_PATH, build

    build.build()
    return os.path.dirname(LIB_PATH)


def _link(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_c_caller_links(libdir, tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    exe = str(tmp_path / "dropin_cases")
    _link([cc, "-std=c99", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), os.path.join(DROPIN, "dropin_cases.c"),
           "-L", libdir, "-lmeshopt_gb300", "-Wl,-rpath," + libdir, "-o", exe])
    assert os.path.isfile(exe)


def test_reference_header_caller_links(libdir, tmp_path):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    ref_src = os.path.join(oracle.reference_root(), "src")
    if not os.path.isfile(os.path.join(ref_src, "meshoptimizer.h")):
        pytest.skip("the reference checkout is not present")
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "ref_header_link")
    # the reference header first, then this library's; only libmeshopt_gb300 on the link line, so an
    # unresolved meshopt_* symbol fails the link
    _link([cxx, "-std=c++11", "-O2", "-Wall", "-Werror", "-I", ref_src, "-I", os.path.join(ROOT, "include"),
           os.path.join(DROPIN, "ref_header_link.cpp"), "-L", libdir, "-lmeshopt_gb300", "-Wl,-rpath," + libdir, "-o", exe])
    undefined = subprocess.run(["nm", "-u", exe], capture_output=True, text=True).stdout
    for sym in ("meshopt_simplify", "meshopt_simplifyWithAttributes", "meshopt_simplifyScale"):
        assert sym in undefined.split(), sym  # resolved from the library at load time
    exported = subprocess.run(["nm", "-D", "--defined-only", os.path.join(libdir, "libmeshopt_gb300.so")], capture_output=True, text=True).stdout
    for sym in ("meshopt_simplify", "meshopt_simplifyWithAttributes", "meshopt_simplifyScale"):
        assert sym in exported.split(), sym
