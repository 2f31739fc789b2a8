"""The drop-in run from a compiled C program: tests/dropin/dropin_cases.c includes only
include/meshopt_gb300.h, links only libmeshopt_gb300.so, and runs the reference's known-answer
cases (demo/tests.cpp, recorded through the reference library in tests/golden/known_answers.json)
through meshopt_simplify / meshopt_simplifyWithAttributes with host buffers, once with 32-bit
indices and once the way a 16-bit index caller goes through them. Its outputs must equal the
reference's bit for bit (result_error within 1e-6 relative)."""
import os
import shutil
import subprocess

import pytest

import fixtures

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REL_TOL = 1e-6


def _hex(x):
    return float(x).hex()


def _write_cases(path, cases):
    with open(path, "w") as f:
        f.write(f"{len(cases)}\n")
        for c in cases:
            vc = len(c["positions"]) * 4 // c["stride"]
            ac = 0 if c["weights"] is None else len(c["weights"])
            lock = c["lock"]
            na = 0 if c["attributes"] is None else len(c["attributes"])
            f.write(f"{c['name']} {len(c['indices'])} {vc} {c['stride']} {len(c['positions'])} {c['target']} {_hex(c['error'])} {c['options']} "
                    f"{ac} {c['attr_stride']} {na} {0 if lock is None else 1}\n")
            f.write(" ".join(str(int(i)) for i in c["indices"]) + "\n")
            f.write(" ".join(_hex(x) for x in c["positions"]) + "\n")
            if ac:
                f.write(" ".join(_hex(x) for x in c["weights"]) + "\n")
                f.write(" ".join(_hex(x) for x in c["attributes"]) + "\n")
            if lock is not None:
                f.write(" ".join(str(int(x)) for x in lock) + "\n")


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    from meshoptimizer_gb300 import LIB_PATH, build

    build.build()
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    libdir = os.path.dirname(LIB_PATH)
    exe = str(tmp_path_factory.mktemp("dropin") / "dropin_cases")
    r = subprocess.run([cc, "-std=c99", "-O2", "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "dropin", "dropin_cases.c"),
                        "-L", libdir, "-lmeshopt_gb300", "-Wl,-rpath," + libdir, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_program_known_answers(harness, tmp_path):
    cases = fixtures.known_answers()
    src, dst = str(tmp_path / "cases.txt"), str(tmp_path / "results.txt")
    _write_cases(src, cases)
    r = subprocess.run([harness, src, dst], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    by_name = {c["name"]: c for c in cases}
    seen = {32: set(), 16: set()}
    for line in open(dst):
        f = line.split()
        name, bits, status, count, err = f[0], int(f[1]), int(f[2]), int(f[3]), float.fromhex(f[4])
        out = [int(x) for x in f[5:]]
        c = by_name[name]
        assert status == 0, (name, bits, status)
        want = [int(x) for x in c["ref_output"]]
        if bits == 16:
            # the debug bit's output carries vertex kinds above bit 16, which no 16-bit buffer holds
            want = [x & 0xFFFF for x in want]
        assert out == want, (name, bits)
        assert count == len(c["ref_output"])
        ref = float(c["ref_error"])
        assert err == ref or abs(err - ref) <= REL_TOL * max(abs(err), abs(ref)), (name, bits, err, ref)
        seen[bits].add(name)
    assert seen[32] == set(by_name)
    assert seen[16] == set(by_name)  # every known-answer mesh has 16-bit indices
