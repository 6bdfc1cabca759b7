"""GPU RDM parity (CIDens::construct_density with DensFCI / DensDOCI).

The device RDMs of a state must equal the reference's for the same CI vector
(golden RDMs of the reference itself for BeH2 and the L=8 / L=10 synthetic
spaces; the oracle's restatement for the larger spaces), to FP64 round-off,
and satisfy CIDens::test_invariants (traces, E_dens == E_CI).
"""
import numpy as np
import pytest

import oracle as O
from ciflow_gb300 import _abi as A
from ciflow_gb300.ciflow import DOCI, FCI, Hamiltonian
from ciflow_gb300.synthetic import make_integrals
from tests.helpers import beh2_integrals, integrals, load_golden

pytestmark = pytest.mark.gpu


def rdm_via_abi(cim, c):
    L = cim.get_l()
    np_ = L * (L - 1) // 2
    r1 = np.empty((2, L, L))
    aa = np.empty((np_, np_))
    ab = np.empty((L * L, L * L))
    bb = np.empty((np_, np_))
    A.check(A.lib().cigpu_rdm(cim.get_mat().handle, A.ptr(np.ascontiguousarray(c)), A.ptr(r1), A.ptr(aa),
                              A.ptr(ab), A.ptr(bb)))
    return r1, aa, ab, bb


def assert_rdm_close(got, ref, atol):
    for g, r, name in zip(got, ref, ("rdm1", "aa", "ab", "bb")):
        err = np.abs(g - r).max()
        assert err <= atol, (name, err)


@pytest.mark.parametrize("tag,cls", [("doci", DOCI), ("fci", FCI)])
def test_beh2_rdm_matches_reference(tag, cls):
    ints, meta, a = beh2_integrals()
    cim = cls(Hamiltonian.from_integrals(ints))
    c = a[f"{tag}_c"]
    got = rdm_via_abi(cim, c)
    assert_rdm_close(got, (a[f"{tag}_rdm1"], a[f"{tag}_aa"], a[f"{tag}_ab"], a[f"{tag}_bb"]), 1e-13)
    assert abs(O.dens_energy(ints, *got) - meta[tag]["dens_energy"]) < 1e-11


@pytest.mark.parametrize("name", ["c0", "c4"])
def test_fci_rdm_of_solved_state(name):
    meta, a = load_golden(name)
    ints = integrals(name)
    cim = FCI(Hamiltonian.from_integrals(ints))
    cim.solve(tol=1e-9)
    c = cim.get_eigvec()
    got = rdm_via_abi(cim, c)
    ref = O.rdm(O.FCI, ints.L, ints.nup, ints.ndown, c)
    assert_rdm_close(got, ref, 1e-12)
    # against the reference's own RDMs of its own eigenvector (sign-invariant quantities)
    assert_rdm_close(got, (a["rdm1"], a["aa"], a["ab"], a["bb"]), 1e-7)
    # CIDens::test_invariants
    N = ints.nup + ints.ndown
    assert abs(np.trace(got[0][0]) + np.trace(got[0][1]) - N) < 1e-10
    assert abs(np.trace(got[1]) + np.trace(got[2]) + np.trace(got[3]) - N * (N - 1) / 2) < 1e-8
    assert abs(O.dens_energy(ints, *got) - cim.get_ci_energy()) < 1e-9


def test_fci_rdm_facade_and_unequal_spins():
    ints = make_integrals(7, 3, 2, nchol=6, seed=77)
    cim = FCI(Hamiltonian.from_integrals(ints))
    c = np.random.default_rng(5).standard_normal(cim.get_dim())
    c /= np.linalg.norm(c)
    got = rdm_via_abi(cim, c)
    ref = O.rdm(O.FCI, ints.L, ints.nup, ints.ndown, c, literal=True)
    assert_rdm_close(got, ref, 1e-13)


def test_c1_rdm_against_oracle():
    ints = integrals("c1")
    cim = FCI(Hamiltonian.from_integrals(ints), precision=A.MIXED)
    cim.solve(tol=1e-6)
    c = cim.get_eigvec()
    got = rdm_via_abi(cim, c)
    ref = O.rdm(O.FCI, ints.L, ints.nup, ints.ndown, c)
    assert_rdm_close(got, ref, 1e-11)
    assert abs(O.dens_energy(ints, *got) - cim.get_ci_energy()) < 1e-6


@pytest.mark.parametrize("L,n", [(8, 4), (10, 3)])
def test_doci_rdm_against_oracle(L, n):
    ints = make_integrals(L, n, n, nchol=8, seed=3 * L + n)
    cim = DOCI(Hamiltonian.from_integrals(ints))
    cim.solve(tol=1e-9)
    c = cim.get_eigvec()
    got = rdm_via_abi(cim, c)
    ref = O.rdm(O.DOCI, L, n, n, c)
    assert_rdm_close(got, ref, 1e-13)
    assert abs(O.dens_energy(ints, *got) - cim.get_ci_energy()) < 1e-9


def test_c2_doci_rdm():
    meta, a = load_golden("c2")
    ints = integrals("c2")
    cim = DOCI(Hamiltonian.from_integrals(ints), precision=A.MIXED)
    cim.solve(tol=1e-6)
    c = cim.get_eigvec()
    got = rdm_via_abi(cim, c)
    ref = O.rdm(O.DOCI, ints.L, ints.nup, ints.ndown, c)
    assert_rdm_close(got, ref, 1e-10)
    # reference RDMs of the reference eigenvector: agree to the eigenvector accuracy
    assert np.abs(got[0] - a["rdm1"]).max() < 1e-5


def test_python_facade_density():
    ints, meta, _ = beh2_integrals()
    cim = FCI(Hamiltonian.from_integrals(ints))
    cim.solve(tol=1e-10)
    cim.construct_density()
    d = cim.cid
    d.test_invariants()
    assert abs(d.get_dens_energy() - cim.get_ci_energy()) < 1e-10
    # antisymmetry of the same-spin block through the reference getter semantics
    assert d.get_two_rdm(0, 1, 2, 3, 4) == -d.get_two_rdm(0, 2, 1, 3, 4)
    assert d.get_two_rdm(0, 2, 2, 3, 4) == 0.0
