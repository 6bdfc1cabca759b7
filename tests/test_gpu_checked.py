"""The bounds-checked build (libcigpu_checked.so) on valid inputs: the FCI spaces
of L=8 4a4b and L=10 5a5b and a DOCI space, both forms (FP64 slot tiles, the
FP32/FP64 mixed tiles, the DOCI CRS and its matrix-free form), builds, solves,
matvecs and RDMs, with the device error word zero after every step and the
energies equal to the reference's. No invalid index is ever given to the GPU."""
import ctypes

import numpy as np
import pytest

import oracle as O
from ciflow_gb300 import _abi as A
from ciflow_gb300.synthetic import make_integrals
from tests.helpers import integrals, load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def chk():
    lib = A.checked_lib()
    assert lib.cigpu_checked_build() == 1
    w = ctypes.c_uint64()
    A.check(lib.cigpu_check_word(ctypes.byref(w), 1))  # start from a clear word
    return lib


def word(lib) -> int:
    w = ctypes.c_uint64()
    A.check(lib.cigpu_check_word(ctypes.byref(w), 0))
    return w.value


def run_case(lib, ints, method, precision, e_ref=None, rdm=True):
    h, e = np.ascontiguousarray(ints.h), np.ascontiguousarray(ints.eri)
    ham, crs = ctypes.c_void_p(), ctypes.c_void_p()
    A.check(lib.cigpu_ham_create(ints.L, ints.nup, ints.ndown, ints.econst, A.ptr(h), A.ptr(e), ctypes.byref(ham)))
    try:
        A.check(lib.cigpu_build(ham, method, precision, None, ctypes.byref(crs)))
        assert word(lib) == 0
        dim = ctypes.c_int64()
        lib.cigpu_crs_dims(crs, ctypes.byref(dim), None, None)
        c = np.empty(dim.value)
        info = A.SolveInfo()
        A.check(lib.cigpu_solve(crs, 1e-8, 0, None, A.ptr(c), ctypes.byref(info)))
        assert word(lib) == 0
        if e_ref is not None:
            assert abs(info.e0 - e_ref) <= (1e-8 if precision == A.FP64 else 1e-6)
        y = np.empty(dim.value)
        A.check(lib.cigpu_mvprod(crs, A.ptr(c), A.ptr(y), None))
        assert abs(float(c @ y) + ints.econst - info.e0) <= 1e-8
        if rdm:
            L = ints.L
            np_ = L * (L - 1) // 2
            r1, aa = np.empty((2, L, L)), np.empty((np_, np_))
            ab, bb = np.empty((L * L, L * L)), np.empty((np_, np_))
            A.check(lib.cigpu_rdm(crs, A.ptr(c), A.ptr(r1), A.ptr(aa), A.ptr(ab), A.ptr(bb)))
            assert abs(np.trace(r1[0]) + np.trace(r1[1]) - (ints.nup + ints.ndown)) < 1e-10
        assert word(lib) == 0
    finally:
        if crs:
            lib.cigpu_crs_destroy(crs)
        lib.cigpu_ham_destroy(ham)


@pytest.mark.parametrize("name", ["c0", "c4"])
@pytest.mark.parametrize("precision", [A.FP64, A.MIXED])
def test_checked_fci_word_stays_zero(chk, name, precision):
    meta, _ = load_golden(name)
    run_case(chk, integrals(name), A.FCI, precision, e_ref=meta["e0"])


@pytest.mark.parametrize("precision", [A.FP64, A.MIXED])
def test_checked_doci_word_stays_zero(chk, precision):
    ints = make_integrals(12, 6, 6, nchol=8, seed=21)
    ref = O.build_upper(O.DOCI, ints)
    e_ref, _ = O.lowest_eigenpair(ref, tol=1e-12)
    run_case(chk, ints, A.DOCI, precision, e_ref=e_ref + ints.econst)


def test_checked_sigma_word_stays_zero(chk, monkeypatch):
    """The mixed FCI form with its FP32 products from the factorised sigma vector
    (forced onto L=10 5a5b, whose grid is below the automatic threshold)."""
    monkeypatch.setenv("CIGPU_FP32_PRODUCT", "sigma")
    meta, _ = load_golden("c4")
    run_case(chk, integrals("c4"), A.FCI, A.MIXED, e_ref=meta["e0"])
