"""On-disk formats (host code, CPU only): the psi4 integral text dump read and
written like Hamiltonian::read_file / save_file (Hamiltonian.cpp:646-885), and the
CI-vector and RDM text dumps of the reference's output (Output.cpp:135-263,
CIDens.cpp:978-1026), compared byte for byte with text the reference itself wrote
(tests/golden/formats.json, made by tests/golden/make_golden.py)."""
import ctypes
import json
import os

import numpy as np
import pytest

import oracle as O
from ciflow_gb300 import _abi as A
from ciflow_gb300.ciflow import Hamiltonian

from .helpers import GOLDEN, beh2_integrals, dets_case

REF_DATA = os.path.join(O.REF_ROOT, "tests", "data")


@pytest.fixture(scope="module")
def formats():
    with open(os.path.join(GOLDEN, "formats.json")) as f:
        return json.load(f)


def write_civec(path, method, L, nup, ndown, c, threshold, up=None, down=None, words=1, name=None):
    c = np.ascontiguousarray(c, dtype=np.float64)
    st = A.lib().cigpu_write_civec(path.encode(), method, L, nup, ndown, len(c), A.ptr(c), 0.0, 0.0, threshold,
                                   A.ptr(up), A.ptr(down), words, name.encode() if name else None)
    assert st == A.OK
    return open(path).read()


def vector_block(text):
    return text[text.index("#CIMETHOD"):]


@pytest.mark.parametrize("tag", ["fci", "doci"])
def test_civec_text_matches_reference(tmp_path, formats, tag):
    ints, meta, arr = beh2_integrals()
    method = A.FCI if tag == "fci" else A.DOCI
    text = write_civec(str(tmp_path / "v.txt"), method, ints.L, ints.nup, ints.ndown, arr[f"{tag}_c"],
                       formats[f"nauw_{tag}"])
    assert vector_block(text) == formats[f"civec_{tag}"]


def test_civec_text_of_a_list_matches_reference(tmp_path, formats):
    ints, up, down, words, meta = dets_case("beh2")
    c = np.load(os.path.join(GOLDEN, "formats_dets_c.npy"))
    text = write_civec(str(tmp_path / "v.txt"), A.DETS, ints.L, ints.nup, ints.ndown, c, formats["nauw_dets"],
                       up, down, words, name="fcibeh2sto3gdeterminants")
    assert vector_block(text) == formats["civec_dets"]


@pytest.mark.parametrize("tag", ["fci", "doci"])
def test_rdm_text_matches_reference(tmp_path, formats, tag):
    ints, meta, arr = beh2_integrals()
    path = str(tmp_path / "r.txt")
    one, aa, ab, bb = (np.ascontiguousarray(arr[f"{tag}_{k}"]) for k in ("rdm1", "aa", "ab", "bb"))
    assert A.lib().cigpu_write_rdm(path.encode(), ints.L, A.ptr(one), A.ptr(aa), A.ptr(ab), A.ptr(bb)) == A.OK
    assert open(path).read() == formats[f"rdm_{tag}"]


@pytest.mark.parametrize("tag", ["beh2", "be70"])
def test_psi4_round_trip(tmp_path, tag):
    if tag == "beh2":
        ints = beh2_integrals()[0]
    else:
        ints = dets_case(tag)[0]
    H = Hamiltonian.from_integrals(ints)
    path = str(tmp_path / "ints.dat")
    H.save_file(path, hf_energy=-1.25)
    G = Hamiltonian.read_file(path)
    assert (G.L, G.nup, G.ndown) == (ints.L, ints.nup, ints.ndown)
    assert G.Econst == ints.econst and G.hf_energy == -1.25
    assert np.array_equal(G.h, ints.h) and np.array_equal(G.eri, ints.eri)


def test_psi4_errors(tmp_path):
    L, na, nb, ec = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
    args = (ctypes.byref(L), ctypes.byref(na), ctypes.byref(nb), ctypes.byref(ec), None, None, None, None)
    assert A.lib().cigpu_ham_read_psi4(str(tmp_path / "none").encode(), *args) == A.ENOTFOUND
    bad = tmp_path / "bad.dat"
    bad.write_text("no integrals here\n")
    assert A.lib().cigpu_ham_read_psi4(str(bad).encode(), *args) == A.EINVAL


@pytest.mark.skipif(not os.path.isdir(REF_DATA), reason="needs the reference tree (its data files and reader)")
@pytest.mark.parametrize("fname", ["beh2_sto3g_1_5.dat", "Be_ccpVDZ.dat", "mpbe5zmatrixelements.dat"])
def test_psi4_reader_matches_the_reference_reader(tmp_path, fname):
    path = os.path.join(REF_DATA, fname)
    ref = O.ref_read_file(path)
    ours = Hamiltonian.read_file(path)
    assert (ours.L, ours.nup, ours.ndown, ours.Econst) == (ref.L, ref.nup, ref.ndown, ref.econst)
    assert np.array_equal(ours.h, ref.h) and np.array_equal(ours.eri, ref.eri)
    # the reference reader reads what the library writes
    out = str(tmp_path / "ours.dat")
    ours.save_file(out)
    back = O.ref_read_file(out)
    assert np.array_equal(back.h, ref.h) and np.array_equal(back.eri, ref.eri) and back.econst == ref.econst
