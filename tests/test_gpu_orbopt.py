"""Orbital optimisers on the device (cigpu_ham_jacobi, cigpu_doci_pair_scan,
cigpu_orbopt_*), through the C ABI, against the reference's outputs and the
oracle's restatement.

* Jacobi rotations: five rotations in sequence equal the reference's
  OrbitalTransform::do_jacobi_rotation result (tests/golden/orbopt.*) to 1e-13,
  exactly 8-fold symmetric.
* DOCI pair scan: angles, energies and kept pairs equal the reference's
  DensDOCI::find_min_angle / calc_rotate with scan_orbitals' selection (1e-9 in
  the angle, 1e-10 Eh in the energy, kept pairs exact), and every energy is the
  expectation value of the unrotated state in the rotated Hamiltonian.
* Simulated annealing and the local minimiser: the chain (accepted and rejected
  steps, final and best energies, final unitary) equals the oracle's chain with the
  same random streams; speculative evaluation of 8 proposals gives the same chain
  as one at a time.
* Natural orbitals: FCI energies are invariant; DOCI energies in natural orbitals
  match the oracle.
"""
import ctypes
import json
import os

import numpy as np
import pytest

from ciflow_gb300 import _abi as A
from ciflow_gb300.ciflow import DOCI, FCI, Hamiltonian
from ciflow_gb300.orbopt import LocalMinimizer, SimulatedAnnealing
from ciflow_gb300.synthetic import Integrals, make_integrals

import orbopt as OO  # the oracle restatement (oracle/orbopt.py)

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")
TOL = 1e-10


@pytest.fixture(scope="module")
def gold():
    with open(os.path.join(GOLD, "orbopt.json")) as f:
        meta = json.load(f)
    return meta, dict(np.load(os.path.join(GOLD, "orbopt.npz")))


def golden_ham(meta, h, eri):
    return Hamiltonian.from_integrals(Integrals(meta["L"], meta["nup"], meta["ndown"], meta["econst"], h, eri))


def create(ints, method, precision=A.FP64, seed=11, warm=True, tol=TOL):
    H = Hamiltonian.from_integrals(ints)
    cfg = A.OrboptConfig(method, precision, tol, 1 if warm else 0, 0, seed)
    out = ctypes.c_void_p()
    A.check(A.lib().cigpu_orbopt_create(H.device(), ctypes.byref(cfg), ctypes.byref(out)))
    return out.value


def get(opt, L, dim=None):
    U, Uo = np.zeros((L, L)), np.zeros((L, L))
    st = A.OrboptStats()
    c = np.zeros(dim) if dim else None
    A.check(A.lib().cigpu_orbopt_get(opt, A.ptr(U), A.ptr(Uo), A.ptr(c), ctypes.byref(st)))
    return U, Uo, c, st.as_dict()


def anneal(opt, steps, speculate=1, temp=0.4, change_temp=0.99, angle=1.4, change_angle=0.999):
    p = A.AnnealParams(temp, change_temp, angle, change_angle, steps, 2000, 1e-7, speculate, 0)
    e = ctypes.c_double()
    A.check(A.lib().cigpu_orbopt_anneal(opt, ctypes.byref(p), ctypes.byref(e)))
    return e.value


def test_jacobi_sequence_matches_reference(gold):
    meta, g = gold
    H = golden_ham(meta, g["h0"], g["eri0"])
    for k, l, th in meta["rotations"]:
        H = H.jacobi(k, l, th)
    assert np.max(np.abs(H.h - g["jac_h"])) < 1e-13
    assert np.max(np.abs(H.eri - g["jac_eri"])) < 1e-13
    e = H.eri
    for perm in [(1, 0, 2, 3), (0, 1, 3, 2), (2, 3, 0, 1), (3, 2, 1, 0)]:
        assert np.array_equal(e, np.transpose(e, perm)), "not exactly 8-fold symmetric"
    assert np.array_equal(H.h, H.h.T)


def test_jacobi_rejects_bad_arguments(gold):
    meta, g = gold
    H = golden_ham(meta, g["h0"], g["eri0"])
    out = ctypes.c_void_p()
    for k, l, th in [(1, 1, 0.2), (-1, 2, 0.2), (0, 8, 0.2), (0, 1, float("nan"))]:
        assert A.lib().cigpu_ham_jacobi(H.device(), k, l, th, None, ctypes.byref(out)) == A.EINVAL


@pytest.mark.parametrize("tag", ["scan0", "scan1"])
def test_doci_pair_scan_matches_reference(gold, tag):
    meta, g = gold
    L = meta["L"]
    h, eri = (g["h0"], g["eri0"]) if tag == "scan0" else (g["jac_h"], g["jac_eri"])
    cim = DOCI(golden_ham(meta, h, eri))
    np_ = L * (L - 1) // 2
    th, en, fd = np.zeros(np_), np.zeros(np_), np.zeros(np_, np.int32)
    c = np.ascontiguousarray(g[f"{tag}_c"])
    A.check(A.lib().cigpu_doci_pair_scan(cim.get_mat().handle, A.ptr(c), A.ptr(th), A.ptr(en), A.ptr(fd)))
    assert np.array_equal(fd, g[f"{tag}_found"])
    assert np.max(np.abs(th - g[f"{tag}_theta"])) < 1e-9
    assert np.max(np.abs(en - g[f"{tag}_energy"])) < 1e-10


def test_scan_energy_is_the_rotated_expectation_value(gold):
    """energy[k,l] = <Psi|H(theta)|Psi> with Psi the unrotated DOCI state, H(theta) the
    device Jacobi rotation, its DOCI CRS built and applied on the device."""
    meta, g = gold
    L = meta["L"]
    ham = golden_ham(meta, g["h0"], g["eri0"])
    cim = DOCI(ham)
    cim.solve(tol=1e-12)
    c = cim.get_eigvec()
    np_ = L * (L - 1) // 2
    th, en, fd = np.zeros(np_), np.zeros(np_), np.zeros(np_, np.int32)
    A.check(A.lib().cigpu_doci_pair_scan(cim.get_mat().handle, A.ptr(c), A.ptr(th), A.ptr(en), A.ptr(fd)))
    p = 0
    checked = 0
    for k in range(L):
        for l in range(k + 1, L):
            if fd[p] and checked < 8:
                rc = DOCI(ham.jacobi(k, l, th[p]))
                E = float(c @ rc.get_mat().mvprod(c))
                assert en[p] == pytest.approx(E, abs=1e-11)
                checked += 1
            p += 1
    assert checked == 8


@pytest.mark.parametrize("precision", [A.FP64, A.MIXED])
def test_anneal_chain_matches_oracle(precision):
    ints = make_integrals(8, 4, 4, nchol=16, seed=77)
    opt = create(ints, A.DOCI, precision, seed=11)
    try:
        e_gpu = anneal(opt, 80)
        U, Uo, _, st = get(opt, 8)
    finally:
        A.lib().cigpu_orbopt_destroy(opt)
    ref = OO.Optimizer(ints, OO.O.DOCI, seed=11)
    e_ref, acc, rej = ref.anneal(OO.AnnealParams(steps=80))
    tol_e = 1e-9 if precision == A.FP64 else 1e-8
    assert (st["accepted"], st["rejected"]) == (acc, rej)
    assert e_gpu == pytest.approx(e_ref, abs=tol_e)
    assert st["e_opt"] == pytest.approx(ref.e_opt, abs=tol_e)
    assert np.max(np.abs(U - ref.U)) < 1e-8
    assert np.max(np.abs(Uo - ref.U_opt)) < 1e-8
    assert acc > 3 and rej > 3, "the chain should both accept and reject"


def test_speculation_keeps_the_chain():
    ints = make_integrals(9, 4, 4, nchol=16, seed=5)
    out = {}
    for K in (1, 8):
        opt = create(ints, A.DOCI, A.FP64, seed=3)
        try:
            e1 = anneal(opt, 120, speculate=K, temp=0.05)
            # a second call continues the chain; near zero temperature most proposals
            # are rejected, so rounds grow towards K proposals
            e2 = anneal(opt, 150, speculate=K, temp=1e-6, angle=0.3)
            out[K] = (e1, e2) + get(opt, 9)
        finally:
            A.lib().cigpu_orbopt_destroy(opt)
    (a1, a2, Ua, Uoa, _, sa), (b1, b2, Ub, Uob, _, sb) = out[1], out[8]
    assert (sa["accepted"], sa["rejected"], sa["steps"]) == (sb["accepted"], sb["rejected"], sb["steps"])
    assert abs(a1 - b1) <= 1e-12 and abs(a2 - b2) <= 1e-12
    assert sa["e_opt"] == pytest.approx(sb["e_opt"], abs=1e-12)
    assert np.max(np.abs(Ua - Ub)) < 1e-12 and np.max(np.abs(Uoa - Uob)) < 1e-12
    assert sa["speculative_waste"] == 0 and sb["speculative_waste"] > 0
    assert sb["solves"] == sa["solves"] + sb["speculative_waste"]


@pytest.mark.parametrize("dist_choice", [0, 1])
def test_local_minimizer_matches_oracle(dist_choice):
    ints = make_integrals(8, 4, 4, nchol=16, seed=77)
    opt = create(ints, A.DOCI, A.FP64, seed=21)
    try:
        p = A.LocalParams(1e-6, 4, 40, dist_choice, 0)
        e = ctypes.c_double()
        A.check(A.lib().cigpu_orbopt_local(opt, ctypes.byref(p), ctypes.byref(e)))
        U, Uo, _, st = get(opt, 8)
    finally:
        A.lib().cigpu_orbopt_destroy(opt)
    ref = OO.Optimizer(ints, OO.O.DOCI, seed=21)
    e_ref, iters = ref.local(OO.LocalParams(conv_crit=1e-6, conv_steps=4, max_iters=40, dist_choice=bool(dist_choice)))
    assert st["steps"] == iters
    assert e.value == pytest.approx(e_ref, abs=1e-9)
    assert np.max(np.abs(U - ref.U)) < 1e-8
    assert e.value < OO.solve(OO.O.DOCI, 8, 4, 4, 0.0, ints.h, ints.eri)[0]


def test_local_minimizer_needs_doci():
    ints = make_integrals(6, 3, 3, nchol=8, seed=2)
    opt = create(ints, A.FCI, A.FP64)
    try:
        p = A.LocalParams(1e-6, 2, 10, 0, 0)
        assert A.lib().cigpu_orbopt_local(opt, ctypes.byref(p), None) == A.ENOTSUP
        bad = A.AnnealParams(0.0, 0.99, 1.4, 0.999, 10, 2000, 1e-7, 1, 0)
        assert A.lib().cigpu_orbopt_anneal(opt, ctypes.byref(bad), None) == A.EINVAL
    finally:
        A.lib().cigpu_orbopt_destroy(opt)


def test_natural_orbitals():
    ints = make_integrals(7, 3, 3, nchol=16, seed=9)
    e_fci = OO.solve(OO.O.FCI, 7, 3, 3, 0.0, ints.h, ints.eri)[0]
    # FCI is invariant under the rotation to its natural orbitals
    opt = create(ints, A.FCI, A.FP64)
    try:
        e = ctypes.c_double()
        A.check(A.lib().cigpu_orbopt_natural(opt, A.FCI, ctypes.byref(e)))
        U, _, _, _ = get(opt, 7)
        assert e.value == pytest.approx(e_fci, abs=1e-9)
        assert np.max(np.abs(U @ U.T - np.eye(7))) < 1e-12
        assert np.max(np.abs(U - np.eye(7))) > 1e-3
    finally:
        A.lib().cigpu_orbopt_destroy(opt)
    # DOCI in its own and in the FCI natural orbitals
    for dm in (A.DOCI, A.FCI):
        opt = create(ints, A.DOCI, A.FP64)
        try:
            e = ctypes.c_double()
            A.check(A.lib().cigpu_orbopt_natural(opt, dm, ctypes.byref(e)))
        finally:
            A.lib().cigpu_orbopt_destroy(opt)
        ref = OO.Optimizer(ints, OO.O.DOCI, seed=0)
        assert e.value == pytest.approx(ref.natural(dm), abs=1e-9)


def test_python_mirror_and_current_hamiltonian():
    ints = make_integrals(8, 4, 4, nchol=16, seed=77)
    cim = DOCI(Hamiltonian.from_integrals(ints))
    cim.solve(tol=1e-10)
    e0 = cim.get_ci_energy()
    sa = SimulatedAnnealing(cim, 0.4, 0.99, 1.4, 0.999, steps=40, speculate=4, tol=1e-10, seed=11)
    e_last = sa.optimize()
    assert cim.get_ci_energy() == pytest.approx(e_last, abs=1e-9)
    # the CIMethod's Hamiltonian is the start rotated by the optimiser's unitary
    h2, e2 = OO.rotate(ints.h, ints.eri, sa.get_unitary())
    assert np.max(np.abs(cim.get_ham().h - h2)) < 1e-12 and np.max(np.abs(cim.get_ham().eri - e2)) < 1e-12
    sa.set_cim_optimal()
    assert cim.get_ci_energy() == pytest.approx(sa.get_opt_ci_energy(), abs=1e-9)
    assert sa.get_opt_ci_energy() <= e0 + 1e-12
    lm = LocalMinimizer(cim, tol=1e-10, seed=1)
    rots = lm.scan_orbitals()
    P, D = OO.doci_pair_matrices(8, 4, cim.get_eigvec())
    th, en, fd = OO.scan(cim.get_ham().h, cim.get_ham().eri, P, D, 8)
    assert len(rots) == int(fd.sum())
    ref = [(k, l) for k in range(8) for l in range(k + 1, 8)]
    for k, l, t, e in rots:
        i = ref.index((k, l))
        assert t == pytest.approx(th[i], abs=1e-9) and e == pytest.approx(en[i], abs=1e-10)
    lm.set_conv_steps(3)
    e_loc = lm.optimize()
    assert e_loc <= cim.get_ci_energy() + 1e-9 and cim.get_ci_energy() == pytest.approx(e_loc, abs=1e-9)
    with pytest.raises(ValueError):
        LocalMinimizer(FCI(Hamiltonian.from_integrals(make_integrals(6, 3, 3, nchol=8, seed=2))))


def test_warm_start_far_above_the_ground_state():
    """Step 78 of an annealing chain (tests/golden/warm_chain.json, made by the
    oracle's chain): a 73-degree rotation leaves the current ground state 14 Eh
    above the proposal's. Warm-started from it, both methods reach the proposal's
    ground state (the oracle's energy) with converged residuals; the mixed method
    keeps its preconditioner's shift at or below the lowest diagonal element, without
    which its Davidson crawled to a stall at an excited energy."""
    with open(os.path.join(GOLD, "warm_chain.json")) as f:
        g = json.load(f)
    H = Hamiltonian.from_integrals(make_integrals(g["L"], g["pairs"], g["pairs"], nchol=g["nchol"], seed=g["seed"]))
    for i, j, a in g["accepted"]:
        H = H.jacobi(int(i), int(j), float(a))
    cur = DOCI(H, precision=A.FP64)
    cur.solve(tol=1e-10)
    assert abs(cur.get_ci_energy() - g["e_current"]) < 1e-8
    c0 = cur.get_eigvec()
    i, j, a = g["proposal"]
    Hp = H.jacobi(int(i), int(j), float(a))
    for prec in (A.MIXED, A.FP64):
        m = DOCI(Hp, precision=prec)
        m.solve(tol=1e-8, c0=c0)
        assert m.info["status"] == A.OK, (prec, m.info)
        assert abs(m.get_ci_energy() - g["e_proposal"]) < 1e-8, (prec, m.get_ci_energy(), g["e_proposal"])
        # the start lies far above: a solver that settles near it has not found the ground state
        assert m.info["matvecs_fp32"] + m.info["matvecs_fp64"] < 150
