"""CPU-side checks of the C ABI boundary: the library loads, exports every
symbol include/cigpu.h declares, and rejects invalid arguments before touching
a device. No compute call is made here."""
import ctypes
import os
import re

import numpy as np
import pytest

from ciflow_gb300 import _abi as A

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "cigpu.h")).read()
    return sorted(set(re.findall(r"\b(cigpu_[a-z_0-9]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(A.LIB_PATH):
        from ciflow_gb300 import build
        build.build()
    return A.lib()


def test_every_declared_symbol_is_exported(lib):
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) == set(A.SIGNATURES), "ctypes signatures must cover include/cigpu.h exactly"


def test_version_and_strerror(lib):
    assert lib.cigpu_get_version() == 1
    assert lib.cigpu_strerror(A.EINVAL) == b"invalid argument"
    assert lib.cigpu_strerror(A.ENOCONV).startswith(b"eigensolver")


def test_invalid_arguments_rejected_on_host(lib):
    out = ctypes.c_void_p()
    h = np.eye(4)
    e = np.zeros((4,) * 4)
    assert lib.cigpu_ham_create(0, 1, 1, 0.0, A.ptr(h), A.ptr(e), ctypes.byref(out)) == A.EINVAL
    assert lib.cigpu_ham_create(4, 5, 1, 0.0, A.ptr(h), A.ptr(e), ctypes.byref(out)) == A.EINVAL
    assert lib.cigpu_ham_create(70, 1, 1, 0.0, A.ptr(h), A.ptr(e), ctypes.byref(out)) == A.EINVAL
    bad = h.copy(); bad[0, 1] = 1.0
    assert lib.cigpu_ham_create(4, 1, 1, 0.0, A.ptr(bad), A.ptr(e), ctypes.byref(out)) == A.EINVAL
    nan = e.copy(); nan[0, 0, 0, 0] = np.nan
    assert lib.cigpu_ham_create(4, 1, 1, 0.0, A.ptr(h), A.ptr(nan), ctypes.byref(out)) == A.EINVAL
    asym = e.copy(); asym[0, 1, 2, 3] = 0.5
    assert lib.cigpu_ham_create(4, 1, 1, 0.0, A.ptr(h), A.ptr(asym), ctypes.byref(out)) == A.EINVAL
    assert lib.cigpu_build(None, 0, 0, None, ctypes.byref(out)) == A.EINVAL
    assert lib.cigpu_solve(None, 1e-8, 0, None, None, None) == A.EINVAL


def test_estimate_bytes(lib):
    b = ctypes.c_size_t()
    assert lib.cigpu_estimate_bytes(12, 6, 6, A.FCI, A.FP64, ctypes.byref(b)) == A.OK
    # full FP64 CRS of the L=12 FCI space alone is 853,776 x 1,819 x 12 bytes
    assert b.value > 853776 * 1819 * 12
    b32 = ctypes.c_size_t()
    lib.cigpu_estimate_bytes(12, 6, 6, A.FCI, A.MIXED, ctypes.byref(b32))
    assert b32.value < b.value
    assert lib.cigpu_estimate_bytes(12, 6, 6, 7, A.FP64, ctypes.byref(b)) == A.EINVAL


def test_server_arguments_checked_on_host(lib):
    out = ctypes.c_void_p()
    assert lib.cigpu_server_create(0, 0, 0, 16, ctypes.byref(out)) == A.EINVAL
    assert lib.cigpu_server_create(0, 0, 4, 0, ctypes.byref(out)) == A.EINVAL
    assert lib.cigpu_server_create(-1, 0, 4, 16, ctypes.byref(out)) in (A.ECUDA, A.EINVAL)
    assert lib.cigpu_server_submit(None, None, None) == A.EINVAL
    assert lib.cigpu_server_poll(None, 1, 0, None, None, None) == A.EINVAL
    assert lib.cigpu_server_cancel(None, 1) == A.EINVAL
    assert lib.cigpu_server_destroy(None) == A.OK
    if A.device_count() == 0:  # no GPU: refused, never a crash
        assert lib.cigpu_server_create(0, 0, 4, 16, ctypes.byref(out)) == A.ECUDA


def test_unitary_exp_matches_scipy(lib):
    import scipy.linalg
    from ciflow_gb300.ciflow import unitary_exp
    rng = np.random.default_rng(3)
    for L, sigma in ((1, 0.1), (6, 0.05), (12, 0.3), (24, 2.0)):
        k = np.triu(rng.normal(0, sigma, (L, L)), 1)
        X = k - k.T
        U = unitary_exp(X)
        np.testing.assert_allclose(U, scipy.linalg.expm(X), atol=1e-13 * max(1.0, np.abs(X).max()) * L)
        np.testing.assert_allclose(U @ U.T, np.eye(L), atol=1e-12 * L)
    bad = np.ones((3, 3))  # not antisymmetric
    assert lib.cigpu_unitary_exp(3, A.ptr(bad), A.ptr(np.empty((3, 3)))) == A.EINVAL
    assert lib.cigpu_ham_rotate(None, None, None, None) == A.EINVAL
    assert lib.cigpu_ham_export(None, None, None) == A.EINVAL


def test_checked_build_exports_and_flags(lib):
    """The bounds-checked build loads beside the regular one, exports the same
    symbols, and says which it is; the regular build has no error word."""
    if not os.path.exists(A.CHECKED_LIB_PATH):
        from ciflow_gb300 import build
        build.build()
    chk = A.checked_lib()
    for s in declared_symbols():
        assert hasattr(chk, s), s
    assert lib.cigpu_checked_build() == 0 and chk.cigpu_checked_build() == 1
    w = ctypes.c_uint64(7)
    assert lib.cigpu_check_word(ctypes.byref(w), 0) == A.ENOTSUP and w.value == 0
    assert chk.cigpu_check_word(None, 0) == A.EINVAL
