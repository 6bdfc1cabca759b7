"""The predicates and error-word records of the bounds-checked build
(ciflow_gb300/csrc/checked.cuh), compiled for the host with nvcc and checked on
valid and invalid values: an index is valid in [0, bound), a CRS row [s, e) of a
matrix n wide needs 0 <= s <= e and e - s <= n, and a record keeps its code in the
top byte and the low 56 bits of the index. (The GPU test runs valid inputs only.)"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
M56 = (1 << 56) - 1


@pytest.fixture(scope="module")
def lines(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path_factory.mktemp("checked") / "test_checked")
    subprocess.run([nvcc, "-O2", "-std=c++17", os.path.join(ROOT, "tests", "cpp", "test_checked.cu"), "-o", exe],
                   check=True)
    return subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split("\n")


def test_records_round_trip(lines):
    recs = [ln.split()[1:] for ln in lines if ln.startswith("rec ")]
    assert len(recs) == 36
    for code, idx, c2, i2 in recs:
        assert int(c2) == int(code) and int(i2) == int(idx) & M56


def test_index_predicate(lines):
    got = {(int(a), int(b)): int(v) for _, a, b, v in (ln.split() for ln in lines if ln.startswith("idx "))}
    for (i, bound), v in got.items():
        assert v == (1 if i < bound else 0), (i, bound)


def test_row_predicate(lines):
    got = [tuple(map(int, ln.split()[1:])) for ln in lines if ln.startswith("row ")]
    assert len(got) == 7
    for s, e, n, v in got:
        assert v == (1 if (s >= 0 and s <= e and e - s <= n) else 0), (s, e, n)
