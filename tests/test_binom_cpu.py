"""The binomial and space-dimension helpers of the build (build.cuh), compiled for
the host with nvcc: every C(n, k) for n <= 130 equals the exact integer while it
fits in int64 and saturates at INT64_MAX beyond it (no overflow in between), and
space_dim refuses impossible electron counts and products beyond int64."""
import math
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
I64 = 2 ** 63 - 1


@pytest.fixture(scope="module")
def lines(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path_factory.mktemp("binom") / "test_binom")
    subprocess.run([nvcc, "-O2", "-std=c++17", "--expt-relaxed-constexpr", os.path.join(ROOT, "tests", "cpp", "test_binom.cu"),
                    "-o", exe], check=True)
    return subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split("\n")


def test_binomials_exact_or_saturated(lines):
    seen = 0
    for ln in lines:
        if not ln.startswith("b "):
            continue
        _, n, k, v = ln.split()
        exact = math.comb(int(n), int(k))
        assert int(v) == (exact if exact <= I64 else I64), (n, k, v)
        seen += 1
    assert seen == sum(n + 1 for n in range(131))


def test_space_dim(lines):
    got = {tuple(map(int, ln.split()[1:5])): int(ln.split()[5]) for ln in lines if ln.startswith("d ")}
    assert got[(0, 12, 6, 6)] == 853776
    assert got[(1, 24, 12, 12)] == 2704156
    assert math.comb(63, 31) ** 2 > I64 and got[(0, 63, 31, 31)] == -1
    assert got[(0, 64, 32, 32)] == -1  # beyond int64
    assert got[(0, 128, 64, 64)] == -1 and got[(1, 128, 64, 64)] == -1
    assert got[(0, 10, 11, 2)] == -1 and got[(0, 10, -1, 2)] == -1
