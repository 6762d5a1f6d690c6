"""The table restatement of the x86 approximate reciprocal (rcpps) and
reciprocal square root (rsqrtss) that the reference's shaders normalise and
divide with (src/mcemath/vector.cpp:158-169,225-250): on an x86-64 host the
decoder in puresoft3d_gb300/csrc/x86_approx.h is compiled and compared with
the instructions themselves on all 2^32 inputs of each (about 20 s), which
pins the tables to the host they were generated on."""
import os
import platform
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GEN = os.path.join(ROOT, "puresoft3d_gb300", "csrc", "gen_x86_approx.c")
HDR = os.path.join(ROOT, "puresoft3d_gb300", "csrc", "x86_approx.h")


@pytest.mark.skipif(platform.machine() not in ("x86_64", "AMD64"), reason="needs the x86 instructions")
def test_tables_reproduce_the_instructions(tmp_path):
    exe = tmp_path / "check"
    subprocess.run(["gcc", "-O2", "-msse2", '-DX86_APPROX_HEADER="%s"' % HDR, "-o", str(exe), GEN], check=True)
    r = subprocess.run([str(exe), "--check"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("0 mismatches")


@pytest.mark.skipif(platform.machine() not in ("x86_64", "AMD64"), reason="needs the x86 instructions")
def test_generator_reproduces_the_committed_tables(tmp_path):
    exe = tmp_path / "gen"
    subprocess.run(["gcc", "-O2", "-msse2", "-o", str(exe), GEN], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    assert out == open(HDR).read()
