"""The host eigensolver of the projected matrices (ciflow_gb300/csrc/small_eigh.h),
compiled with g++ and checked against numpy on random, graded, degenerate,
tridiagonal and arrowhead matrices up to 64 x 64: eigenvalues to 1e-12 |A|,
residuals |A z - w z| and orthonormality to 1e-12."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    out = str(tmp_path_factory.mktemp("eigh") / "test_small_eigh")
    subprocess.run([gxx, "-O2", "-std=c++17", os.path.join(ROOT, "tests", "cpp", "test_small_eigh.cpp"), "-o", out],
                   check=True)
    return out


def cases():
    rng = np.random.default_rng(0)
    out = []
    for n in (1, 2, 3, 5, 17, 31, 42, 64):
        a = rng.standard_normal((n, n)); out.append((a + a.T) / 2)
    a = np.diag(np.arange(8.0)); out.append(a)                          # already diagonal
    a = np.ones((6, 6)); out.append(a)                                  # rank one, degenerate
    t = np.diag(rng.standard_normal(40)) + np.diag(rng.standard_normal(39), 1); out.append(t + np.triu(t, 1).T)
    a = np.diag(rng.standard_normal(30) * 10); a[0, 1:] = a[1:, 0] = rng.standard_normal(29); out.append(a)
    a = rng.standard_normal((20, 20)); a = (a + a.T) * np.logspace(-8, 8, 20)[:, None] * np.logspace(-8, 8, 20)[None, :]
    out.append((a + a.T) / 2)                                           # graded
    a = np.eye(12) * 35.0 + 1e-9 * rng.standard_normal((12, 12)); out.append((a + a.T) / 2)  # clustered
    return out


def test_matches_numpy(exe):
    mats = cases()
    text = "".join(f"{m.shape[0]} " + " ".join(f"{x:.17g}" for x in m.ravel()) + "\n" for m in mats)
    res = subprocess.run([exe], input=text, capture_output=True, text=True, check=True).stdout.split("\n")
    for k, a in enumerate(mats):
        n = a.shape[0]
        w = np.array(res[2 * k].split(), dtype=float)
        z = np.array(res[2 * k + 1].split(), dtype=float).reshape(n, n)
        scale = max(1.0, np.abs(a).max())
        np.testing.assert_allclose(w, np.linalg.eigvalsh(a), atol=1e-12 * scale * n)
        assert np.all(np.diff(w) >= -1e-12 * scale)
        assert np.abs(a @ z - z * w).max() <= 1e-11 * scale * n
        assert np.abs(z.T @ z - np.eye(n)).max() <= 1e-12 * n
