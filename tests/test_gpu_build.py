"""GPU CRS build parity (FCI::construct_CI_matrix / DOCI::construct_CI_matrix).

The device CRS, exported in the reference layout, must be bit-identical to the
reference CRS: same row pointers, same columns, same FP64 values (SHA-256 of the
uint32/uint32/float64 arrays, recorded from the reference itself by
tests/golden/make_golden.py), and identical to the oracle on cases without a
stored hash.
"""
import numpy as np
import pytest

import oracle as O
from ciflow_gb300 import _abi as A
from ciflow_gb300.ciflow import DOCI, FCI, Hamiltonian
from ciflow_gb300.synthetic import make_integrals
from tests.helpers import beh2_integrals, crs_sha256, integrals, load_golden

pytestmark = pytest.mark.gpu


def build(cls, ints, precision=A.FP64):
    return cls(Hamiltonian.from_integrals(ints), precision=precision)


@pytest.mark.parametrize("tag,cls", [("doci", DOCI), ("fci", FCI)])
def test_beh2_crs_bit_exact(tag, cls):
    ints, meta, _ = beh2_integrals()
    cim = build(cls, ints)
    m = cim.get_mat()
    assert m.getn() == meta[tag]["dim"]
    assert m.datasize() == meta[tag]["nnz"]
    assert crs_sha256(*m.upper()) == meta[tag]["crs_sha256"]


@pytest.mark.parametrize("name", ["c0", "c4"])
def test_config_crs_bit_exact(name):
    meta, _ = load_golden(name)
    ints = integrals(name)
    assert ints.checksum() == meta["integrals_sha"]
    m = build(FCI, ints).get_mat()
    assert (m.getn(), m.datasize()) == (meta["dim"], meta["nnz"])
    assert crs_sha256(*m.upper()) == meta["crs_sha256"]


def test_c1_crs_bit_exact():
    meta, _ = load_golden("c1")
    m = build(FCI, integrals("c1")).get_mat()
    assert (m.getn(), m.datasize()) == (meta["dim"], meta["nnz"])
    assert m.nnz_full == 2 * meta["nnz"] - meta["dim"]
    assert crs_sha256(*m.upper()) == meta["crs_sha256"]


def test_c2_doci_crs_bit_exact():
    meta, _ = load_golden("c2")
    m = build(DOCI, integrals("c2")).get_mat()
    assert (m.getn(), m.datasize()) == (meta["dim"], meta["nnz"])
    assert crs_sha256(*m.upper()) == meta["crs_sha256"]


@pytest.mark.parametrize("L,n,method", [(6, 3, O.DOCI), (10, 5, O.DOCI), (7, 2, O.FCI), (6, 3, O.FCI),
                                        (5, 1, O.FCI), (4, 2, O.DOCI)])
def test_small_spaces_match_oracle(L, n, method):
    ints = make_integrals(L, n, n, nchol=8, seed=100 + L + n)
    ref = O.build_upper(method, ints)
    cim = build(DOCI if method == O.DOCI else FCI, ints)
    row, col, val = cim.get_mat().upper()
    np.testing.assert_array_equal(row.astype(np.int64), ref.row)
    np.testing.assert_array_equal(col, ref.col)
    np.testing.assert_array_equal(val, ref.val)  # bit-exact FP64


def test_full_matrix_is_exact_mirror():
    ints = integrals("c0")
    m = build(FCI, ints).get_mat()
    row, col, val = m.full()
    import scipy.sparse as sp
    H = sp.csr_matrix((val, col.astype(np.int64), row), shape=(m.n, m.n))
    assert (H != H.T).nnz == 0
    # columns ascending within each row
    for r in range(0, m.n, 97):
        assert np.all(np.diff(col[row[r]:row[r + 1]].astype(np.int64)) > 0)
    ur, uc, uv = m.upper()
    U = sp.csr_matrix((uv, uc.astype(np.int64), ur.astype(np.int64)), shape=(m.n, m.n))
    assert abs(H - (U + U.T - sp.diags(U.diagonal()))).max() == 0


def test_mixed_build_same_pattern_fp32_values():
    ints = integrals("c0")
    m64 = build(FCI, ints).get_mat()
    m32 = build(FCI, ints, precision=A.MIXED).get_mat()
    r64, c64, v64 = m64.full()
    r32, c32, v32 = m32.full()
    np.testing.assert_array_equal(r64, r32)
    np.testing.assert_array_equal(c64, c32)
    np.testing.assert_array_equal(v64.astype(np.float32).astype(np.float64), v32)


@pytest.mark.parametrize("case", ["c0", "c4"])
def test_sigma_backed_mixed_build_defers_and_exports_the_same(case, monkeypatch):
    """A mixed build whose FP32 products come from the sigma operator stores FP64
    slot values and finishes its fill and row counts on a side stream: its counts
    and exported matrix equal those of the mixed build from stored FP32 values, and
    its FP64 product (which waits for the fill) equals the plain build's."""
    import ctypes

    ints = integrals(case)
    monkeypatch.setenv("CIGPU_FP32_PRODUCT", "slots")
    ref = build(FCI, ints, precision=A.MIXED).get_mat()
    monkeypatch.setenv("CIGPU_FP32_PRODUCT", "sigma")
    cim = build(FCI, ints, precision=A.MIXED)
    m = cim.get_mat()
    kind = ctypes.c_int()
    A.check(A.lib().cigpu_crs_fp32_product(m.handle, ctypes.byref(kind), None, None))
    assert kind.value == A.FP32_SIGMA
    x = np.random.default_rng(4).standard_normal(m.n)
    y = m.mvprod(x)  # FP64 product right after the build: waits for the deferred fill on the device
    y_ref = build(FCI, ints).get_mat().mvprod(x)
    assert np.abs(y - y_ref).max() <= 1e-12 * np.abs(y_ref).max()
    # the same build on compact FP64 tiles (the alpha-single x beta-single block left
    # out, its deferred fill counting it from histograms): the same counts, exports
    # and FP64 product, bit for bit
    monkeypatch.setenv("CIGPU_SLOTS64", "compact")
    comp = build(FCI, ints, precision=A.MIXED).get_mat()
    np.testing.assert_array_equal(comp.mvprod(x), y)
    s4, wp = _slot_widths(ints.L, ints.nup, ints.ndown)
    lay, stored = _layout(comp)
    assert lay == A.LAYOUT_SLOTS and stored % s4 == 0 and stored // s4 * wp == _layout(m)[1]
    assert (comp.nnz_upper, comp.nnz_full) == (ref.nnz_upper, ref.nnz_full)
    for a, b in zip(comp.full(), ref.full()):
        np.testing.assert_array_equal(a, b)
    assert (m.nnz_upper, m.nnz_full) == (ref.nnz_upper, ref.nnz_full)
    for a, b in zip(m.full(), ref.full()):
        np.testing.assert_array_equal(a, b)


def _slot_widths(L, nup, ndown):
    """(S4, Wp) of the FCI slot tiles: the start of the alpha-single x beta-single
    block and the padded row width (segments padded to multiples of 4)."""
    from math import comb

    def pad4(n):
        return (n + 3) & ~3

    nsa, nsb = nup * (L - nup), ndown * (L - ndown)
    nda, ndb = comb(nup, 2) * comb(L - nup, 2), comb(ndown, 2) * comb(L - ndown, 2)
    s4 = 4 + pad4(nsb) + pad4(ndb) + pad4(nsa + nda)
    return s4, s4 + pad4(nsa * nsb)


def _layout(m):
    import ctypes

    lay, stored = ctypes.c_int(), ctypes.c_int64()
    A.check(A.lib().cigpu_crs_layout(m.handle, ctypes.byref(lay), ctypes.byref(stored)))
    return lay.value, stored.value


@pytest.mark.parametrize("L,nup,ndown", [(10, 5, 5), (11, 5, 4), (10, 4, 5)])
def test_compact_fp64_tiles_equal_full_tiles(L, nup, ndown, monkeypatch):
    """FP64 slot tiles that leave out the alpha-single x beta-single block (the
    matvec forms it from the integrals) store S4 of the Wp values per row and give
    the full tiles' product bit for bit, the same row counts (the fill counts the
    block from per-pair histograms) and the same exported matrix. With 25 beta
    singles (10 orbitals, 5 beta electrons) quads of the block span two alpha
    singles."""
    ints = make_integrals(L, nup, ndown, nchol=8, seed=3 * L + 5 * nup + ndown)
    monkeypatch.setenv("CIGPU_SLOTS64", "full")
    full = build(FCI, ints).get_mat()
    monkeypatch.setenv("CIGPU_SLOTS64", "compact")
    comp = build(FCI, ints).get_mat()
    (lf, sf), (lc, sc) = _layout(full), _layout(comp)
    assert lf == lc == A.LAYOUT_SLOTS
    s4, wp = _slot_widths(L, nup, ndown)
    assert sf % wp == 0 and sc == sf // wp * s4
    x = np.random.default_rng(L + nup).standard_normal(full.n)
    np.testing.assert_array_equal(comp.mvprod(x), full.mvprod(x))
    assert (comp.nnz_upper, comp.nnz_full) == (full.nnz_upper, full.nnz_full)
    for a, b in zip(comp.full(), full.full()):
        np.testing.assert_array_equal(a, b)
    if full.n <= 70000:  # and the oracle's CRS (the larger case takes the oracle long)
        ref = O.build_upper(O.FCI, ints)
        row, col, val = comp.upper()
        np.testing.assert_array_equal(val, ref.val)
        np.testing.assert_array_equal(col, ref.col)


def test_symmetry_zeros_dropped_like_reference():
    # BeH2 in D2h: many elements are exactly zero and must be dropped (|v| <= 1e-14)
    ints, meta, _ = beh2_integrals()
    m = build(FCI, ints).get_mat()
    _, _, val = m.upper()
    assert np.all(np.abs(val) > 1e-14)
    assert m.datasize() < m.getn() * (m.getn() + 1) // 2


def test_zero_electron_and_tiny_spaces():
    ints = make_integrals(4, 0, 0, nchol=4, seed=5)
    m = build(FCI, ints).get_mat()
    assert m.getn() == 1
    ints = make_integrals(3, 1, 1, nchol=4, seed=6)
    ref = O.build_upper(O.FCI, ints)
    row, col, val = build(FCI, ints).get_mat().upper()
    np.testing.assert_array_equal(val, ref.val)


def test_launch_counter_advances():
    before = A.lib().cigpu_kernel_launches()
    build(FCI, integrals("c0"))
    assert A.lib().cigpu_kernel_launches() > before
