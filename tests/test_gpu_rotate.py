"""Orbital rotation on the device (cigpu_ham_rotate), the replacement of
OrbitalTransform::fillHamCI (OrbitalTransform.cpp:64-135).

Checks: the rotated integrals equal the numpy four-index transform to 1e-13
(relative to the largest integral) and are exactly 8-fold symmetric; the FCI
energy does not change under a rotation (FCI is invariant) while the DOCI
energy does, and matches DOCI on host-rotated integrals; a served request with
a rotation gives the same energy as the request with pre-rotated integrals.
Pinned to the reference: the rotated integrals equal those the reference's own
OrbitalTransform::fillHamCI produces for the same U (tests/golden/rotate.*,
made by tests/golden/make_golden.py from the compiled reference) to 1e-12 of
the largest integral.
"""
import numpy as np
import pytest
import scipy.linalg

from .helpers import load_golden

from ciflow_gb300 import _abi as A
from ciflow_gb300.ciflow import DOCI, FCI, Hamiltonian
from ciflow_gb300.server import Server
from ciflow_gb300.synthetic import Integrals, make_integrals, symmetrize_eri

pytestmark = pytest.mark.gpu


def generator(L, sigma, seed):
    rng = np.random.default_rng(seed)
    k = np.triu(rng.normal(0.0, sigma, (L, L)), 1)
    return k - k.T


def host_rotate(ints, U):
    h = U @ ints.h @ U.T
    eri = np.einsum("ap,bq,cr,ds,pqrs->abcd", U, U, U, U, ints.eri, optimize=True)
    return Integrals(ints.L, ints.nup, ints.ndown, ints.econst, 0.5 * (h + h.T), symmetrize_eri(eri))


@pytest.mark.parametrize("L", [4, 10, 24])
def test_rotated_integrals_match_numpy(L):
    ints = make_integrals(L, 2, 2, nchol=8, seed=L)
    U = scipy.linalg.expm(generator(L, 0.1, 7))
    H = Hamiltonian.from_integrals(ints).rotated(U)
    ref = host_rotate(ints, U)
    scale = np.abs(ints.eri).max()
    assert np.abs(H.eri - ref.eri).max() <= 1e-13 * scale * L
    assert np.abs(H.h - ref.h).max() <= 1e-13 * np.abs(ints.h).max() * L
    e = H.eri
    for perm in ((1, 0, 2, 3), (0, 1, 3, 2), (2, 3, 0, 1)):
        np.testing.assert_array_equal(e, e.transpose(perm))  # exact symmetry
    np.testing.assert_array_equal(H.h, H.h.T)


def test_fci_energy_invariant_doci_not():
    ints = make_integrals(8, 3, 3, nchol=16, seed=3)
    U = scipy.linalg.expm(generator(8, 0.2, 11))
    base = Hamiltonian.from_integrals(ints)
    rot = base.rotated(U)
    e_base, e_rot = FCI(base), FCI(rot)
    e_base.solve(tol=1e-10)
    e_rot.solve(tol=1e-10)
    assert abs(e_base.get_ci_energy() - e_rot.get_ci_energy()) <= 1e-9
    d_rot = DOCI(rot)
    d_rot.solve(tol=1e-10)
    d_ref = DOCI(Hamiltonian.from_integrals(host_rotate(ints, U)))
    d_ref.solve(tol=1e-10)
    assert abs(d_rot.get_ci_energy() - d_ref.get_ci_energy()) <= 1e-9
    d_base = DOCI(base)
    d_base.solve(tol=1e-10)
    assert abs(d_base.get_ci_energy() - d_rot.get_ci_energy()) > 1e-6  # DOCI depends on the orbitals


def test_served_rotation_matches_prerotated_integrals():
    ints = make_integrals(10, 5, 5, nchol=16, seed=4)
    U = scipy.linalg.expm(generator(10, 0.05, 1_000_001))
    with Server(max_inflight=2) as srv:
        a = srv.submit(ints, method=A.DOCI, precision=A.MIXED, tol=1e-8, rot=U)
        b = srv.submit(host_rotate(ints, U), method=A.DOCI, precision=A.MIXED, tol=1e-8)
        ra, rb = srv.wait(a), srv.wait(b)
        assert ra["status"] == A.OK and rb["status"] == A.OK
        assert abs(ra["e0"] - rb["e0"]) <= 1e-9
        with pytest.raises(A.CigpuError) as e:
            srv.submit(ints, rot=2.0 * U)  # not orthogonal
        assert e.value.status == A.EINVAL


@pytest.mark.parametrize("tag", ["L8", "L10", "L10_strong"])
def test_rotation_matches_reference_fillhamci(tag):
    from ciflow_gb300.synthetic import config_integrals
    meta, g = load_golden("rotate")
    m = meta[tag]
    ints = config_integrals(m["config"])
    assert ints.checksum() == m["integrals_sha"]
    H = Hamiltonian.from_integrals(ints).rotated(g[f"{tag}_U"])
    scale = np.abs(g[f"{tag}_eri"]).max()
    assert np.abs(H.eri - g[f"{tag}_eri"]).max() <= 1e-12 * scale
    assert np.abs(H.h - g[f"{tag}_h"]).max() <= 1e-12 * np.abs(g[f"{tag}_h"]).max()
