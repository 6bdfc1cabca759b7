"""Batched solves (cigpu_solve_batch) against one-at-a-time solves and dense references.

Problems below the batching limit run in lockstep FP64 Lanczos steps replayed as a
CUDA graph; every energy must match the dense eigensolve of the oracle matrix
(small spaces) or the single-problem FP64 solve (larger ones) to 1e-8 Eh, the
plain method's tolerance.
"""
import numpy as np
import pytest

import oracle as O
from ciflow_gb300 import _abi as A
from ciflow_gb300.batch import random_problems, solve_batch
from ciflow_gb300.ciflow import DOCI, FCI, Hamiltonian
from ciflow_gb300.synthetic import make_integrals

pytestmark = pytest.mark.gpu

E_TOL = 1e-8


def dense_e0(ints, method):
    H = O.build_upper(method, ints).full_csr()
    return np.linalg.eigvalsh(H.toarray())[0] + ints.econst


def single_e0(ints, method, tol=1e-10):
    cim = (DOCI if method == A.DOCI else FCI)(Hamiltonian.from_integrals(ints))
    cim.solve(tol=tol)
    return cim.get_ci_energy()


def test_batch_matches_dense_on_small_uneven_spaces():
    probs = random_problems(48, seed=3, max_L=8, min_L=4)
    probs += [(make_integrals(4, 0, 0, nchol=4, seed=5), A.FCI),  # one determinant
              (make_integrals(6, 2, 2, nchol=16, seed=7), A.DOCI),
              (make_integrals(7, 1, 1, nchol=16, seed=1123), A.FCI)]  # weak overlap with the lowest diagonal
    e0, infos, status, stats = solve_batch(probs, tol=1e-9)
    assert stats["batched"] == len(probs) and stats["individual"] == 0
    assert stats["graph_launches"] > 0 and stats["lanes"] in (4, 8, 16, 32)
    for (ints, m), e, inf, st in zip(probs, e0, infos, status):
        assert st == A.OK, (ints.L, ints.nup, m, inf)
        assert inf["residual"] <= 1e-9
        assert abs(e - dense_e0(ints, m)) <= E_TOL, (ints.L, ints.nup, m)


def test_batch_matches_single_solves_and_splits_by_size():
    probs = random_problems(24, seed=11, max_L=10, min_L=6)
    # limit 5000: the larger problems take the single-problem path (MIXED requested)
    probs = [(ints, m, A.MIXED) for ints, m in probs]
    e0, infos, status, stats = solve_batch(probs, tol=1e-7, max_batched_dim=5000)
    assert stats["batched"] + stats["individual"] == len(probs)
    assert stats["batched"] > 0 and stats["individual"] > 0
    for (ints, m, _), e, st, inf in zip(probs, e0, status, infos):
        assert st == A.OK
        assert abs(e - single_e0(ints, m)) <= 1e-6  # mixed single solves: |dE0| <= 1e-6
        n = O.dim(O.DOCI if m == A.DOCI else O.FCI, ints.L, ints.nup, ints.ndown)
        # the lockstep solves FP64; the problems above the limit keep MIXED
        assert inf["precision"] == (A.FP64 if n <= 5000 else A.MIXED)
        if n <= 20000:  # against the oracle's ARPACK eigenpair of the reference CRS
            e_ref, _ = O.lowest_eigenpair(O.build_upper(O.DOCI if m == A.DOCI else O.FCI, ints), tol=1e-12)
            assert abs(e - (e_ref + ints.econst)) <= 1e-6


def test_batch_twice_same_result_and_rejects_bad_requests():
    probs = random_problems(16, seed=5, max_L=9, min_L=5)
    a, _, _, s1 = solve_batch(probs, tol=1e-8)
    b, _, _, s2 = solve_batch(probs, tol=1e-8)
    np.testing.assert_array_equal(a, b)  # deterministic kernels, cached shape
    assert s2["tuned"] == 0
    bad = make_integrals(6, 3, 3, nchol=8, seed=6)
    bad.eri[0, 1, 2, 3] += 1e-3
    with pytest.raises(A.CigpuError) as e:
        solve_batch([(bad, A.FCI)] + probs[:2], tol=1e-8)
    assert e.value.status == A.EINVAL
    with pytest.raises(A.CigpuError) as e:
        solve_batch(probs[:2], tol=0.0)
    assert e.value.status == A.EINVAL
    e0, _, _, st = solve_batch([], tol=1e-8)
    assert len(e0) == 0 and st["batched"] == 0
