"""Batched lowest eigenpairs of many independent problems (cigpu_solve_batch).

    e0, infos, status, stats = solve_batch(problems, tol=1e-6)

`problems` is a list of (Integrals, method) or (Integrals, method, precision);
problems up to `max_batched_dim` determinants are solved together in lockstep
FP64 Lanczos steps launched as CUDA graphs, larger ones one by one.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _abi as A


def solve_batch(problems, tol: float = 1e-6, max_batched_dim: int = 0):
    n = len(problems)
    keep = []  # keep the integral arrays alive during the call
    reqs = (A.Request * max(n, 1))()
    for i, pr in enumerate(problems):
        ints, method = pr[0], pr[1]
        precision = pr[2] if len(pr) > 2 else A.FP64
        hh = np.ascontiguousarray(ints.h, dtype=np.float64)
        ee = np.ascontiguousarray(ints.eri, dtype=np.float64)
        keep += [hh, ee]
        reqs[i] = A.Request(ints.L, ints.nup, ints.ndown, method, precision, 0, ints.econst, tol,
                            A.ptr(hh), A.ptr(ee), None)
    e0 = np.full(max(n, 1), np.nan)
    infos = (A.SolveInfo * max(n, 1))()
    status = np.zeros(max(n, 1), dtype=np.int32)
    stats = A.BatchStats()
    st = A.lib().cigpu_solve_batch(n, reqs, max_batched_dim, A.ptr(e0), infos, A.ptr(status), ctypes.byref(stats))
    A.check(st, "cigpu_solve_batch")
    return e0[:n], [infos[i].as_dict() for i in range(n)], status[:n], stats.as_dict()


def random_problems(count: int, seed: int = 0, max_L: int = 12, min_L: int = 6):
    """The uneven batch: L uniform in [min_L, max_L]; FCI with 1..L/2 electrons per
    spin or DOCI with 2..L/2 pairs (coin flip); integrals seeded per problem."""
    from .synthetic import make_integrals

    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        L = int(rng.integers(min_L, max_L + 1))
        if rng.random() < 0.5:
            ne = int(rng.integers(1, L // 2 + 1))
            out.append((make_integrals(L, ne, ne, nchol=16, seed=1000 + i), A.FCI))
        else:
            p = int(rng.integers(2, L // 2 + 1))
            out.append((make_integrals(L, p, p, nchol=16, seed=1000 + i), A.DOCI))
    return out
