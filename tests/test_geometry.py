"""The lattice factory's geometry helpers against the reference's test/test_Geometry.cpp: builds
tests/geometry_kat.cpp with the host objects' flags (no floating-point contraction) and runs it
(no GPU)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_geometry_known_answers(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "geometry_kat"
    r = subprocess.run([cxx, "-std=c++17", "-O3", "-ffp-contract=off", "-Wall", "-Werror",
                        "-I", os.path.join(ROOT, "spinparser_gb300", "csrc", "host"),
                        os.path.join(ROOT, "tests", "geometry_kat.cpp"), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
