"""The C++ façade header compiles (syntax and types) with the host compiler."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_facade_header_compiles(tmp_path):
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "test_facade.cpp")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_ci_big_lines_follow_cisize():
    """CI_Big's kept block for a CISIZE budget in GB (CIMethod.cpp:596-598):
    numelements = CISIZE 2^30 3 / (64 5) 10 / 2, numlines = round((sqrt(1 + 8 ne) - 1) / 2)."""
    from ciflow_gb300.ciflow import ci_big_lines
    for gb in (0.001, 0.5, 1.0, 16.0):
        ne = int(gb * 1024.0 ** 3 * 3 / (64.0 * 5) * 10.0 / 2.0)
        assert ci_big_lines(gb) == int(round((-1 + (1 + 8 * ne) ** 0.5) / 2))
    assert ci_big_lines(1.0) == 10033  # 50,331,648 elements
