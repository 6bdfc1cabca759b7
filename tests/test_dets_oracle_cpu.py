"""Determinant-list CI (FCI_File / CI_Big) on the CPU: the oracle's restatement of
FCI_File::construct_CI_matrix + get_ham_element (CIMethod.cpp:459-487, 890-914)
against the reference's own CRS and known answers (tests/golden/dets.*), and the
library's determinant-file reader (Permutator_File::read_file, Permutator.cpp:179-224).
CPU only: the reader is host code and needs no GPU."""
import ctypes
import os

import numpy as np
import pytest

import oracle as O
from ciflow_gb300 import _abi as A
from ciflow_gb300.synthetic import make_integrals

from .helpers import crs_sha256, dets_case


@pytest.mark.parametrize("tag", ["beh2", "be_gkci", "be70"])
def test_oracle_dets_build_matches_reference(tag):
    ints, up, down, words, meta = dets_case(tag)
    m = O.build_dets(ints, up, down, words)
    assert (m.n, m.nnz) == (meta["dim"], meta["nnz"])
    assert crs_sha256(m.row, m.col, m.val) == meta["crs_sha256"]
    if "crs_sha256_reference" in meta:  # the reference CRS itself (64-bit strings)
        assert meta["crs_sha256"] == meta["crs_sha256_reference"]
    w, _ = np.linalg.eigh(m.full_csr().toarray())
    e0 = w[0] + ints.econst
    assert e0 == pytest.approx(meta["e0_oracle"], abs=1e-10)
    if "e0_known_answer" in meta:  # TestDetFile.cpp:32, Testmp.cpp:39
        assert e0 == pytest.approx(meta["e0_known_answer"], rel=1e-12)


def test_full_list_in_reference_order_is_the_fci_matrix():
    ints = make_integrals(7, 3, 2, nchol=8, seed=3)

    def strings(L, n):
        out, s = [], (1 << n) - 1
        while s < (1 << L):
            out.append(s)
            t = s | (s - 1)
            s = (t + 1) | (((~t & -~t) - 1) >> ((s & -s).bit_length()))
        return out
    ua, db = strings(7, 3), strings(7, 2)
    up = np.array([u for u in ua for d in db], np.uint64)
    down = np.array([d for u in ua for d in db], np.uint64)
    a, b = O.build_dets(ints, up, down), O.build_upper(O.FCI, ints)
    assert np.array_equal(a.row, b.row) and np.array_equal(a.col, b.col) and np.array_equal(a.val, b.val)


def write_det_file(path, up, down, words, L):
    with open(path, "w") as f:
        f.write("#determinants written by the test\n#nup = ?\n")
        for i in range(len(up) // words):
            u = sum(int(up[i * words + w]) << (64 * w) for w in range(words))
            d = sum(int(down[i * words + w]) << (64 * w) for w in range(words))
            f.write(format(u, f"0{L}b") + "|" + format(d, f"0{L}b") + "\n")
        f.write("#all determinants with following seniorities are included = []\n")


@pytest.mark.parametrize("tag", ["be_gkci", "be70"])
def test_reader_round_trip(tmp_path, tag):
    from ciflow_gb300.ciflow import read_determinants
    ints, up, down, words, meta = dets_case(tag)
    path = str(tmp_path / "dets.txt")
    write_det_file(path, up, down, words, ints.L)
    u2, d2, w2 = read_determinants(path, ints.L)
    assert w2 == words and np.array_equal(u2, up) and np.array_equal(d2, down)


def test_reader_errors(tmp_path):
    lib = A.lib()
    n, nb = ctypes.c_int64(), ctypes.c_int()
    assert lib.cigpu_dets_read(str(tmp_path / "missing").encode(), 1, 0, None, None, ctypes.byref(n),
                               ctypes.byref(nb)) == A.ENOTFOUND
    bad = tmp_path / "bad.txt"
    bad.write_text("0011|01x1\n")
    assert lib.cigpu_dets_read(str(bad).encode(), 1, 0, None, None, ctypes.byref(n), ctypes.byref(nb)) == A.EINVAL
    long = tmp_path / "long.txt"
    long.write_text("1" * 70 + "|" + "1" * 3 + "\n")
    assert lib.cigpu_dets_read(str(long).encode(), 1, 0, None, None, ctypes.byref(n), ctypes.byref(nb)) == A.EINVAL
    assert lib.cigpu_dets_read(str(long).encode(), 2, 0, None, None, ctypes.byref(n), ctypes.byref(nb)) == A.OK
    assert (n.value, nb.value) == (1, 70)


def test_oracle_densfile_matches_reference():
    """The oracle's DensFILE restatement against the reference's DensFILE RDMs of the
    BeH2 list (tests/golden/dets.npz)."""
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "dets.npz"))
    ints, up, down, words, meta = dets_case("beh2")
    got = O.rdm_dets(ints.L, up, down, g["beh2_c"])
    for x, k in zip(got, ("rdm1", "aa", "ab", "bb")):
        assert np.max(np.abs(x - g[f"beh2_{k}"])) < 1e-14, k

