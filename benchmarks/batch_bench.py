"""Batched uneven solves: 512 problems in one cigpu_solve_batch call against the
same 512 solved one at a time (cigpu_ham_create + cigpu_build + cigpu_solve each).

The batch: L uniform in 6..12; FCI with 1..L/2 electrons per spin or DOCI with
2..L/2 pairs; integrals seeded per problem (15 to 853,776 determinants). Every
request asks for the mixed form, in both arms: one at a time each problem is a
MIXED build + solve; the batch solves the problems up to the batching limit in
lockstep FP64 Lanczos steps (their reported precision) and the larger ones MIXED
on three concurrent streams. Both arms reach |dE0| <= 1e-6; the line carries the
largest |dE0| between them and, for a seeded sample of problems up to 20,000
determinants, against the oracle's ARPACK eigenpair of the reference CRS.

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


def one_at_a_time(problems, tol: float, precision: int):
    """E0 and wall seconds of each problem solved alone through the C ABI."""
    lib = A.lib()
    e0 = np.empty(len(problems))
    secs = np.empty(len(problems))
    for i, (ints, method, *_) in enumerate(problems):
        t0 = time.perf_counter()
        hh = np.ascontiguousarray(ints.h)
        ee = np.ascontiguousarray(ints.eri)
        ham, crs = ctypes.c_void_p(), ctypes.c_void_p()
        A.check(lib.cigpu_ham_create(ints.L, ints.nup, ints.ndown, ints.econst, A.ptr(hh), A.ptr(ee),
                                     ctypes.byref(ham)))
        A.check(lib.cigpu_build(ham, method, precision, None, ctypes.byref(crs)))
        info = A.SolveInfo()
        st = lib.cigpu_solve(crs, tol, 0, None, None, ctypes.byref(info))
        if st not in (A.OK, A.ENOCONV):
            A.check(st)
        e0[i] = info.e0
        lib.cigpu_crs_destroy(crs)
        lib.cigpu_ham_destroy(ham)
        secs[i] = time.perf_counter() - t0
    return e0, secs


def run(count: int = 512, seed: int = 0, tol: float = 1e-6, max_batched_dim: int = 0, oracle=None,
        oracle_sample: int = 24):
    """oracle: the oracle module (given by the caller) for the sample check, or None."""
    prec = A.MIXED
    problems = [(i, m, prec) for i, m in random_problems(count, seed=seed)]
    dims = np.array([comb(i.L, i.nup) * (comb(i.L, i.ndown) if m == A.FCI else 1) for i, m, _ in problems])
    lim = max_batched_dim or 65536
    small = dims <= lim
    solve_batch(problems[: min(8, count)], tol=tol, max_batched_dim=max_batched_dim)  # warm-up
    one_at_a_time(problems[: min(8, count)], tol, prec)
    t0 = time.perf_counter()
    e_b, infos, status, stats = solve_batch(problems, tol=tol, max_batched_dim=max_batched_dim)
    t_batch = time.perf_counter() - t0
    e_s, secs = one_at_a_time(problems, tol, prec)
    t_single = float(secs.sum())
    small_probs = [p for p, f in zip(problems, small) if f]
    t0 = time.perf_counter()
    e_bs, infos_s, _, stats_small = solve_batch(small_probs, tol=tol, max_batched_dim=max_batched_dim)
    t_batch_small = time.perf_counter() - t0
    t_single_small = float(secs[small].sum())
    mv = np.array([i["matvecs_fp64"] for i in infos_s]) if small_probs else np.zeros(1)
    de = np.abs(e_b - e_s)
    check = None
    if oracle is not None:  # a seeded sample against the oracle's ARPACK eigenpair
        O = oracle
        cand = [k for k in range(count) if dims[k] <= 20000]
        pick = np.random.default_rng(seed + 7).choice(cand, size=min(oracle_sample, len(cand)), replace=False)
        errs = []
        t0 = time.perf_counter()
        for k in pick:
            ints, m, _ = problems[int(k)]
            e_ref, _ = O.lowest_eigenpair(O.build_upper(O.DOCI if m == A.DOCI else O.FCI, ints), tol=1e-12)
            errs.append(max(abs(e_b[k] - (e_ref + ints.econst)), abs(e_s[k] - (e_ref + ints.econst))))
        check = {"problems": len(pick), "max_abs_dE0_vs_oracle": float(max(errs)) if errs else None,
                 "oracle_s": time.perf_counter() - t0}
    precisions = {"fp64": sum(1 for i in infos if i["precision"] == A.FP64),
                  "mixed": sum(1 for i in infos if i["precision"] == A.MIXED)}
    return {
        "problems": count, "dims": {"min": int(dims.min()), "max": int(dims.max()), "sum": int(dims.sum())},
        "batched_below": lim, "n_batched": int(small.sum()), "n_individual": int((~small).sum()),
        "tol": tol, "requested_precision": "mixed (both arms)", "batch_precision_used": precisions,
        "batch_s": t_batch, "one_at_a_time_s": t_single,
        "solves_per_s_batch": count / t_batch, "solves_per_s_one_at_a_time": count / t_single,
        "speedup": t_single / t_batch,
        "small_only": {"problems": int(small.sum()), "batch_s": t_batch_small, "one_at_a_time_s": t_single_small,
                       "speedup": t_single_small / t_batch_small,
                       "matvecs_p50_p100": [float(np.percentile(mv, 50)), float(mv.max())], "stats": stats_small},
        "max_abs_dE0_batch_vs_single": float(de.max()),
        "oracle_sample": check,
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
