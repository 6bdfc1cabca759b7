"""The orbital-optimiser restatement of the oracle against the reference's own
outputs (tests/golden/orbopt.*, made by tests/golden/make_golden.py from the
reference sources): Jacobi rotations with the accumulated unitary
(OrbitalTransform.cpp:278-414) and the DOCI pair scan (CIDens.cpp:1279-1464,
LocalMinimizer.cpp:89-118). CPU only."""
import json
import math
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import orbopt as OO  # noqa: E402

GOLD = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="module")
def gold():
    with open(os.path.join(GOLD, "orbopt.json")) as f:
        meta = json.load(f)
    return meta, dict(np.load(os.path.join(GOLD, "orbopt.npz")))


def test_jacobi_sequence_matches_reference(gold):
    meta, g = gold
    h, eri, U = g["h0"], g["eri0"], np.eye(meta["L"])
    for k, l, th in meta["rotations"]:
        h, eri = OO.jacobi(h, eri, k, l, th)
        U = OO.jacobi_unitary(U, k, l, th)
    assert np.max(np.abs(h - g["jac_h"])) < 1e-13
    assert np.max(np.abs(eri - g["jac_eri"])) < 1e-13
    assert np.max(np.abs(U - g["jac_U"])) < 1e-14
    # the accumulated unitary reproduces the sequence as one rotation of the start
    h2, e2 = OO.rotate(g["h0"], g["eri0"], U)
    assert np.max(np.abs(h2 - h)) < 1e-12 and np.max(np.abs(e2 - eri)) < 1e-12


@pytest.mark.parametrize("tag", ["scan0", "scan1"])
def test_doci_scan_matches_reference(gold, tag):
    meta, g = gold
    L, n = meta["L"], meta["nup"]
    if tag == "scan0":
        h, eri = g["h0"], g["eri0"]
    else:
        h, eri = g["jac_h"], g["jac_eri"]
    P, D = OO.doci_pair_matrices(L, n, g[f"{tag}_c"])
    th, en, fd = OO.scan(h, eri, P, D, 2 * n)
    assert np.array_equal(fd, g[f"{tag}_found"])
    assert np.max(np.abs(th - g[f"{tag}_theta"])) < 1e-9
    assert np.max(np.abs(en - g[f"{tag}_energy"])) < 1e-10
    pi = 0
    for k in range(L):
        for l in range(k + 1, L):
            t = OO.pair_terms(h, eri, P, D, 2 * n, k, l)
            for i, a in enumerate(meta["fixed_angles"]):
                assert OO.calc_rotate(t, a) == pytest.approx(g[f"{tag}_fixed"][pi, i], abs=1e-11)
            pi += 1


def test_calc_rotate_is_the_energy_of_the_rotated_hamiltonian(gold):
    """calc_rotate(k, l, t) = <Psi|H(t)|Psi> for the unrotated DOCI state: the DOCI
    CRS of the Jacobi-rotated integrals, applied to the same coefficients."""
    meta, g = gold
    L, n = meta["L"], meta["nup"]
    c = g["scan0_c"]
    P, D = OO.doci_pair_matrices(L, n, c)
    for k, l, a in [(0, 1, 0.3), (2, 7, -1.1), (3, 5, 2.4)]:
        t = OO.pair_terms(g["h0"], g["eri0"], P, D, 2 * n, k, l)
        h2, e2 = OO.jacobi(g["h0"], g["eri0"], k, l, a)
        m = OO.O.build_upper(OO.O.DOCI, OO._Ints(L, n, n, 0.0, h2, e2))
        E = float(c @ (m.full_csr() @ c))
        assert OO.calc_rotate(t, a) == pytest.approx(E, abs=1e-11)


def test_newton_derivatives_match_finite_differences(gold):
    meta, g = gold
    L, n = meta["L"], meta["nup"]
    P, D = OO.doci_pair_matrices(L, n, g["scan0_c"])
    t = OO.pair_terms(g["h0"], g["eri0"], P, D, 2 * n, 1, 4)
    for a in (-1.2, 0.0, 0.4, 2.9):
        d = 1e-5
        g1 = (OO.calc_rotate(t, a + d) - OO.calc_rotate(t, a - d)) / (2 * d)
        g2 = (OO.calc_rotate(t, a + d) - 2 * OO.calc_rotate(t, a) + OO.calc_rotate(t, a - d)) / d ** 2
        assert OO._gradient(t, a) == pytest.approx(g1, abs=1e-7)
        assert OO._hessian(t, a) == pytest.approx(g2, abs=1e-4)


def test_splitmix64_stream():
    """splitmix64 known answers (the 64-bit mix of Steele, Lea and Flood with the
    golden-ratio increment): outputs of seed 0 computed with arbitrary-precision
    integers from the definition, and the [0, 1) mapping."""
    r = OO.SplitMix64(0)
    z = 0x9E3779B97F4A7C15
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) % 2 ** 64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) % 2 ** 64
    assert r.next() == z ^ (z >> 31)
    r = OO.SplitMix64(12345)
    u = [r.uniform() for _ in range(1000)]
    assert 0.0 <= min(u) and max(u) < 1.0 and abs(np.mean(u) - 0.5) < 0.05
    r = OO.SplitMix64(7)
    assert all(0 <= r.below(5) < 5 for _ in range(1000))


def test_oracle_chain_is_deterministic_and_descends():
    """A short annealing chain and a local minimisation on the oracle: the same seed
    gives the same chain; the local minimiser lowers the DOCI energy."""
    from ciflow_gb300.synthetic import make_integrals
    ints = make_integrals(6, 3, 3, nchol=8, seed=5)
    p = OO.AnnealParams(steps=25)
    a = OO.Optimizer(ints, OO.O.DOCI, seed=3)
    b = OO.Optimizer(ints, OO.O.DOCI, seed=3)
    ra, rb = a.anneal(p), b.anneal(p)
    assert ra == rb and np.array_equal(a.U, b.U)
    assert a.e_opt <= OO.solve(OO.O.DOCI, 6, 3, 3, 0.0, ints.h, ints.eri)[0]
    lm = OO.Optimizer(ints, OO.O.DOCI, seed=3)
    e0 = lm.e
    e1, it = lm.local(OO.LocalParams(conv_steps=3, max_iters=40))
    assert e1 < e0 and it >= 3
    assert np.max(np.abs(lm.U @ lm.U.T - np.eye(6))) < 1e-12
    assert math.isfinite(e1)
