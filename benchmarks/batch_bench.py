"""Batched uneven solves: 512 problems in one cigpu_solve_batch call against the
same 512 solved one at a time (cigpu_ham_create + cigpu_build + cigpu_solve each).

The batch: L uniform in 6..12; FCI with 1..L/2 electrons per spin or DOCI with
2..L/2 pairs; integrals seeded per problem (15 to 853,776 determinants). Both
paths use the plain FP64 method, so they compute the same quantity; every result
carries |dE0| between the two.

    python -m benchmarks.batch_bench --count 512
"""
from __future__ import annotations

import argparse
import ctypes
import json
import time
from math import comb

import numpy as np

from ciflow_gb300 import _abi as A
from ciflow_gb300.batch import random_problems, solve_batch


def one_at_a_time(problems, tol: float):
    """E0 and wall seconds of each problem solved alone through the C ABI."""
    lib = A.lib()
    e0 = np.empty(len(problems))
    secs = np.empty(len(problems))
    for i, (ints, method) in enumerate(problems):
        t0 = time.perf_counter()
        hh = np.ascontiguousarray(ints.h)
        ee = np.ascontiguousarray(ints.eri)
        ham, crs = ctypes.c_void_p(), ctypes.c_void_p()
        A.check(lib.cigpu_ham_create(ints.L, ints.nup, ints.ndown, ints.econst, A.ptr(hh), A.ptr(ee),
                                     ctypes.byref(ham)))
        A.check(lib.cigpu_build(ham, method, A.FP64, None, ctypes.byref(crs)))
        info = A.SolveInfo()
        st = lib.cigpu_solve(crs, tol, 0, None, None, ctypes.byref(info))
        if st not in (A.OK, A.ENOCONV):
            A.check(st)
        e0[i] = info.e0
        lib.cigpu_crs_destroy(crs)
        lib.cigpu_ham_destroy(ham)
        secs[i] = time.perf_counter() - t0
    return e0, secs


def run(count: int = 512, seed: int = 0, tol: float = 1e-6, max_batched_dim: int = 0):
    problems = random_problems(count, seed=seed)
    dims = np.array([comb(i.L, i.nup) * (comb(i.L, i.ndown) if m == A.FCI else 1) for i, m in problems])
    lim = max_batched_dim or 65536
    small = dims <= lim
    solve_batch(problems[: min(8, count)], tol=tol, max_batched_dim=max_batched_dim)  # warm-up
    one_at_a_time(problems[: min(8, count)], tol)
    t0 = time.perf_counter()
    e_b, infos, status, stats = solve_batch(problems, tol=tol, max_batched_dim=max_batched_dim)
    t_batch = time.perf_counter() - t0
    e_s, secs = one_at_a_time(problems, tol)
    t_single = float(secs.sum())
    small_probs = [p for p, f in zip(problems, small) if f]
    t0 = time.perf_counter()
    e_bs, infos_s, _, stats_small = solve_batch(small_probs, tol=tol, max_batched_dim=max_batched_dim)
    t_batch_small = time.perf_counter() - t0
    t_single_small = float(secs[small].sum())
    mv = np.array([i["matvecs_fp64"] for i in infos_s]) if small_probs else np.zeros(1)
    de = np.abs(e_b - e_s)
    return {
        "problems": count, "dims": {"min": int(dims.min()), "max": int(dims.max()), "sum": int(dims.sum())},
        "batched_below": lim, "n_batched": int(small.sum()), "n_individual": int((~small).sum()),
        "tol": tol, "precision": "fp64 (both arms)",
        "batch_s": t_batch, "one_at_a_time_s": t_single,
        "solves_per_s_batch": count / t_batch, "solves_per_s_one_at_a_time": count / t_single,
        "speedup": t_single / t_batch,
        "small_only": {"problems": int(small.sum()), "batch_s": t_batch_small, "one_at_a_time_s": t_single_small,
                       "speedup": t_single_small / t_batch_small,
                       "matvecs_p50_p100": [float(np.percentile(mv, 50)), float(mv.max())], "stats": stats_small},
        "max_abs_dE0_batch_vs_single": float(de.max()),
        "not_converged": int(sum(1 for s in status if s != A.OK)),
        "stats": stats,
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--count", type=int, default=512)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--tol", type=float, default=1e-6)
    ap.add_argument("--max-batched-dim", type=int, default=0)
    a = ap.parse_args()
    print(json.dumps(run(a.count, a.seed, a.tol, a.max_batched_dim)))


if __name__ == "__main__":
    main()
