"""Determinant-list CI on the device (cigpu_build_dets), through the C ABI.

* The CRS of the reference's own determinant lists (BeH2 STO-3G, 1225
  determinants; Be cc-pVDZ, 100 GKCI determinants) is bit-identical to the
  reference's FCI_File CRS (SHA-256 of the upper triangle), and E0 matches the
  reference (1e-8 Eh plain, 1e-6 mixed) and the known answer of TestDetFile.cpp.
* The 70-orbital Be list of Testmp.cpp (128-bit strings) gives the CRS of the
  oracle's 128-bit restatement and the known answer -14.346369472944886.
* The full FCI list in the reference's determinant order gives the FCI CRS.
* CI_Big storage (no stored matrix): matvecs equal the CRS matvecs and E0 agrees.
"""
import ctypes

import numpy as np
import pytest

import oracle as O
from ciflow_gb300 import _abi as A
from ciflow_gb300.ciflow import CI_Big, FCI, FCI_File, Hamiltonian
from ciflow_gb300.synthetic import make_integrals

from .helpers import crs_sha256, dets_case

pytestmark = pytest.mark.gpu


def upper_sha(cim):
    row, col, val = cim.get_mat().upper()
    return crs_sha256(row, col, val)


@pytest.mark.parametrize("tag", ["beh2", "be_gkci", "be70"])
def test_dets_crs_and_energy(tag):
    ints, up, down, words, meta = dets_case(tag)
    ham = Hamiltonian.from_integrals(ints)
    cim = FCI_File(ham, up=up, down=down, words=words)
    assert cim.get_dim() == meta["dim"] and cim.get_mat().datasize() == meta["nnz"]
    assert upper_sha(cim) == meta["crs_sha256"]
    cim.solve(tol=1e-10)
    assert cim.get_ci_energy() == pytest.approx(meta["e0_oracle"], abs=1e-9)
    if "e0_known_answer" in meta:
        assert cim.get_ci_energy() == pytest.approx(meta["e0_known_answer"], abs=1e-9)
    mixed = FCI_File(ham, up=up, down=down, words=words, precision=A.MIXED)
    mixed.solve(tol=1e-7)
    assert mixed.get_ci_energy() == pytest.approx(meta["e0_oracle"], abs=1e-6)


def test_full_list_gives_the_fci_matrix():
    ints = make_integrals(8, 4, 3, nchol=16, seed=12)

    def strings(L, n):
        out, s = [], (1 << n) - 1
        while s < (1 << L):
            out.append(s)
            t = s | (s - 1)
            s = (t + 1) | (((~t & -~t) - 1) >> ((s & -s).bit_length()))
        return out
    ua, db = strings(8, 4), strings(8, 3)
    up = np.array([u for u in ua for d in db], np.uint64)
    down = np.array([d for u in ua for d in db], np.uint64)
    ham = Hamiltonian.from_integrals(ints)
    a, b = FCI_File(ham, up=up, down=down), FCI(ham)
    for x, y in zip(a.get_mat().upper(), b.get_mat().upper()):
        assert np.array_equal(x, y)
    # a shuffled list: the same matrix permuted
    perm = np.random.default_rng(1).permutation(len(up))
    c = FCI_File(ham, up=up[perm], down=down[perm])
    m = O.build_dets(ints, up[perm], down[perm])
    assert upper_sha(c) == crs_sha256(m.row, m.col, m.val)
    c.solve(tol=1e-10)
    b.solve(tol=1e-10)
    assert c.get_ci_energy() == pytest.approx(b.get_ci_energy(), abs=1e-10)


@pytest.mark.parametrize("tag", ["beh2", "be70"])
def test_onthefly_matches_stored(tag):
    ints, up, down, words, meta = dets_case(tag)
    ham = Hamiltonian.from_integrals(ints)
    stored = FCI_File(ham, up=up, down=down, words=words)
    fly = CI_Big(ham, up=up, down=down, words=words)
    layout, stored_n = ctypes.c_int(), ctypes.c_int64()
    A.check(A.lib().cigpu_crs_layout(fly.get_mat().handle, ctypes.byref(layout), ctypes.byref(stored_n)))
    assert layout.value == A.LAYOUT_ONTHEFLY and stored_n.value == 0
    x = np.random.default_rng(0).standard_normal(meta["dim"])
    y1, y2 = stored.get_mat().mvprod(x), fly.get_mat().mvprod(x)
    assert np.max(np.abs(y1 - y2)) <= 1e-12 * np.max(np.abs(y1))
    fly.solve(tol=1e-10)
    assert fly.get_ci_energy() == pytest.approx(meta["e0_oracle"], abs=1e-9)


@pytest.mark.parametrize("tag", ["beh2", "be70"])
@pytest.mark.parametrize("frac", [0.0, 0.3, 0.77, 1.0])
def test_ci_big_stored_block_matches_stored(tag, frac):
    """CI_Big with the block of its first `keep` determinants stored (CI_Big::mvprod,
    CIMethod.cpp:943-984): the matvec (stored block + every other element recomputed)
    equals the fully stored matrix's for keep = 0, a part of the list and all of it,
    the stored element count is the block's, and the energy is the known one."""
    ints, up, down, words, meta = dets_case(tag)
    ham = Hamiltonian.from_integrals(ints)
    n = meta["dim"]
    keep = int(round(frac * n))
    stored = FCI_File(ham, up=up, down=down, words=words)
    big = CI_Big(ham, up=up, down=down, words=words, keep=keep)
    layout, stored_n = ctypes.c_int(), ctypes.c_int64()
    A.check(A.lib().cigpu_crs_layout(big.get_mat().handle, ctypes.byref(layout), ctypes.byref(stored_n)))
    assert layout.value == A.LAYOUT_ONTHEFLY
    # the block's elements: those of the stored matrix with row and column below keep
    r, c, _ = stored.get_mat().full()
    rows = np.repeat(np.arange(n), np.diff(r.astype(np.int64)))
    assert stored_n.value == int(np.count_nonzero((rows < keep) & (c < keep)))
    x = np.random.default_rng(2).standard_normal(n)
    y1, y2 = stored.get_mat().mvprod(x), big.get_mat().mvprod(x)
    assert np.max(np.abs(y1 - y2)) <= 1e-12 * np.max(np.abs(y1))
    if frac in (0.3, 0.77):
        big.solve(tol=1e-10)
        assert big.get_ci_energy() == pytest.approx(meta["e0_oracle"], abs=1e-9)


def test_dets_rejections():
    ints, up, down, words, meta = dets_case("beh2")
    ham = Hamiltonian.from_integrals(ints)
    out = ctypes.c_void_p()
    lib = A.lib()
    bad = up.copy()
    u3 = int(up[3])
    bad[3] = np.uint64(u3 | (1 << next(o for o in range(7) if not (u3 >> o) & 1)))  # one electron too many
    assert lib.cigpu_build_dets(ham.device(), len(up), 1, A.ptr(bad), A.ptr(down), A.DETS_CRS, A.FP64, None,
                                ctypes.byref(out)) == A.EINVAL
    outside = up.copy()
    u0 = int(up[0])
    outside[0] = np.uint64((u0 ^ (u0 & -u0)) | (1 << 9))  # lowest electron moved to orbital 9
    assert lib.cigpu_build_dets(ham.device(), len(up), 1, A.ptr(outside), A.ptr(down), A.DETS_CRS, A.FP64, None,
                                ctypes.byref(out)) == A.EINVAL  # orbital 9 of a 7-orbital space
    assert lib.cigpu_build_dets(ham.device(), len(up), 1, A.ptr(up), A.ptr(down), A.DETS_ONTHEFLY, A.MIXED, None,
                                ctypes.byref(out)) == A.ENOTSUP


def rdms(cim_handle, L, c):
    np_ = L * (L - 1) // 2
    one, aa = np.zeros((2, L, L)), np.zeros((np_, np_))
    ab, bb = np.zeros((L * L, L * L)), np.zeros((np_, np_))
    c = np.ascontiguousarray(c)
    A.check(A.lib().cigpu_rdm(cim_handle, A.ptr(c), A.ptr(one), A.ptr(aa), A.ptr(ab), A.ptr(bb)))
    return one, aa, ab, bb


def test_dets_rdm_matches_reference_densfile():
    """The device DensFILE RDMs of the BeH2 list equal the reference's DensFILE
    (tests/golden/dets.npz) to 1e-13 and, as TestDensity.cpp checks, DensFCI's to
    1e-11; two runs are bit-identical (order-independent fixed-point sums)."""
    import json, os
    from .helpers import GOLDEN, beh2_integrals
    ints, up, down, words, meta = dets_case("beh2")
    g = np.load(os.path.join(GOLDEN, "dets.npz"))
    cim = FCI_File(Hamiltonian.from_integrals(ints), up=up, down=down, words=words)
    got = rdms(cim.get_mat().handle, ints.L, g["beh2_c"])
    for x, k in zip(got, ("rdm1", "aa", "ab", "bb")):
        assert np.max(np.abs(x - g[f"beh2_{k}"])) < 1e-13, k
    again = rdms(cim.get_mat().handle, ints.L, g["beh2_c"])
    assert all(np.array_equal(x, y) for x, y in zip(got, again))
    _, _, arr = beh2_integrals()
    for x, k in zip(got, ("rdm1", "aa", "ab", "bb")):
        assert np.max(np.abs(x - arr[f"fci_{k}"])) < 1e-11, k
    cim.solve(tol=1e-10)
    cim.construct_density()
    assert cim.cid.get_dens_energy() == pytest.approx(cim.get_ci_energy(), abs=1e-9)


def test_dets_rdm_matches_oracle_gkci():
    ints, up, down, words, meta = dets_case("be_gkci")
    cim = FCI_File(Hamiltonian.from_integrals(ints), up=up, down=down, words=words)
    cim.solve(tol=1e-10)
    c = cim.get_eigvec()
    got = rdms(cim.get_mat().handle, ints.L, c)
    ref = O.rdm_dets(ints.L, up, down, c)
    for x, y in zip(got, ref):
        assert np.max(np.abs(x - y)) < 1e-13

