"""Determinant-list CI throughput (FCI_File / CI_Big): a CISD determinant list.

Workload: the reference determinant (the nup / ndown lowest orbitals) and all its
single and double excitations, seeded synthetic integrals (the reference reads such
lists from files, e.g. its CISD and GKCI lists). Reported: the device build of the
CRS (two pair scans of the whole list), the stored FP64 / FP32 matvecs, the
on-the-fly matvec (CI_Big: every pair rescanned and its element recomputed), the
solves, and the CPU baseline: the oracle's restatement of the reference build
(get_ham_element for every pair, OpenMP) timed on a bounded sample of rows and
extrapolated.

    python -m benchmarks.dets_bench --L 32 --n 8
"""
from __future__ import annotations

import argparse
import ctypes
import itertools
import json
import os
import sys
import time

import numpy as np

from ciflow_gb300 import _abi as A
from ciflow_gb300.ciflow import CI_Big, FCI_File, Hamiltonian
from ciflow_gb300.synthetic import make_integrals


def cisd_list(L: int, nup: int, ndown: int):
    """The reference determinant first, then singles and doubles (alpha, beta, alpha-beta)."""
    occ_a, occ_b = list(range(nup)), list(range(ndown))
    vir_a, vir_b = list(range(nup, L)), list(range(ndown, L))
    ra = sum(1 << o for o in occ_a)
    rb = sum(1 << o for o in occ_b)

    def excite(ref, occ, vir, k):
        for hs in itertools.combinations(occ, k):
            for ps in itertools.combinations(vir, k):
                s = ref
                for h in hs:
                    s ^= 1 << h
                for p in ps:
                    s |= 1 << p
                yield s
    ups, downs = [ra], [rb]
    for s in excite(ra, occ_a, vir_a, 1):
        ups.append(s)
        downs.append(rb)
    for s in excite(rb, occ_b, vir_b, 1):
        ups.append(ra)
        downs.append(s)
    for s in excite(ra, occ_a, vir_a, 2):
        ups.append(s)
        downs.append(rb)
    for s in excite(rb, occ_b, vir_b, 2):
        ups.append(ra)
        downs.append(s)
    sa = list(excite(ra, occ_a, vir_a, 1))
    sb = list(excite(rb, occ_b, vir_b, 1))
    for a in sa:
        for b in sb:
            ups.append(a)
            downs.append(b)
    return np.array(ups, np.uint64), np.array(downs, np.uint64)


def _time(fn, reps=5):
    fn()
    t0 = time.perf_counter()
    for _ in range(reps):
        fn()
    return (time.perf_counter() - t0) / reps


def cpu_build_sample(ints, up, down, rows: int) -> dict:
    """The oracle's FCI_File count pass (get_ham_element for every pair i <= j, all host
    threads) on the sub-list of the first `rows` determinants, scaled to the whole list
    by the number of pairs."""
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
    import oracle as O
    lib = O.port()
    lib.orc_build_dets.restype = ctypes.c_int
    P = ctypes.c_void_p
    lib.orc_build_dets.argtypes = [ctypes.c_int] * 3 + [P, P, ctypes.c_int64, ctypes.c_int] + [P] * 5
    n = len(up)
    h = np.ascontiguousarray(ints.h)
    e = np.ascontiguousarray(ints.eri)
    sub_u = np.ascontiguousarray(up[: rows])
    sub_d = np.ascontiguousarray(down[: rows])
    row = np.zeros(rows + 1, np.int64)
    t0 = time.perf_counter()
    lib.orc_build_dets(ints.L, ints.nup, ints.ndown, h.ctypes.data, e.ctypes.data, rows, 1, sub_u.ctypes.data,
                       sub_d.ctypes.data, row.ctypes.data, None, None)
    dt = time.perf_counter() - t0
    pairs = rows * (rows + 1) / 2
    full_pairs = n * (n + 1) / 2
    return {"sample_rows": rows, "sample_s": dt, "pairs_per_s": pairs / dt,
            "extrapolated_count_pass_s": dt * full_pairs / pairs,
            "note": "count pass of the oracle build on the first rows' sub-list (pairs i <= j), scaled by pairs"}


def run(L=32, n=8, solve=True, cpu_rows=20000, precision_mixed=True):
    ints = make_integrals(L, n, n, nchol=16, seed=7)
    up, down = cisd_list(L, n, n)
    ham = Hamiltonian.from_integrals(ints)
    ndet = len(up)
    out = {"workload": f"CISD list, L={L}, {n}a{n}b, {ndet} determinants (seeded synthetic integrals)",
           "determinants": ndet, "pairs_per_scan": ndet * ndet}
    FCI_File(ham, up=up, down=down)  # warm-up
    t0 = time.perf_counter()
    cim = FCI_File(ham, up=up, down=down)
    out["build_s"] = time.perf_counter() - t0
    out["nnz_full"] = cim.get_mat().nnz_full
    out["pairs_per_s_build"] = 2 * ndet * ndet / out["build_s"]  # count + fill pass
    lib = A.lib()
    x = np.random.default_rng(0).standard_normal(ndet)
    import torch  # device buffers for the device matvec timing
    dx = torch.tensor(x, device="cuda")
    dy = torch.empty_like(dx)
    h = cim.get_mat().handle

    def mv64():
        A.check(lib.cigpu_mvprod_device(h, dx.data_ptr(), dy.data_ptr(), 0, None))
        torch.cuda.synchronize()
    out["matvec_crs_fp64_ms"] = 1e3 * _time(mv64)
    fly = CI_Big(ham, up=up, down=down)
    hf = fly.get_mat().handle

    def mvf():
        A.check(lib.cigpu_mvprod_device(hf, dx.data_ptr(), dy.data_ptr(), 0, None))
        torch.cuda.synchronize()
    out["matvec_onthefly_ms"] = 1e3 * _time(mvf, reps=3)
    out["pairs_per_s_onthefly"] = ndet * ndet / (out["matvec_onthefly_ms"] * 1e-3)
    if solve:
        cim.solve(tol=1e-8)
        out["solve_crs_fp64"] = {"e0": cim.get_ci_energy(), "seconds": cim.info["seconds"],
                                 "matvecs": cim.info["matvecs_fp64"]}
        if precision_mixed:
            mx = FCI_File(ham, up=up, down=down, precision=A.MIXED)
            mx.solve(tol=1e-6)
            out["solve_crs_mixed"] = {"e0": mx.get_ci_energy(), "seconds": mx.info["seconds"],
                                      "matvecs_fp32": mx.info["matvecs_fp32"], "matvecs_fp64": mx.info["matvecs_fp64"],
                                      "dE0_vs_fp64": abs(mx.get_ci_energy() - cim.get_ci_energy())}
        fly.solve(tol=1e-8)
        out["solve_onthefly"] = {"e0": fly.get_ci_energy(), "seconds": fly.info["seconds"],
                                 "matvecs": fly.info["matvecs_fp64"]}
    if cpu_rows:
        out["cpu_oracle_build"] = cpu_build_sample(ints, up, down, min(cpu_rows, ndet))
        out["cpu_oracle_build"]["cores"] = len(os.sched_getaffinity(0))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--L", type=int, default=32)
    ap.add_argument("--n", type=int, default=8)
    ap.add_argument("--no-solve", action="store_true")
    ap.add_argument("--cpu-rows", type=int, default=20000)
    a = ap.parse_args()
    print(json.dumps(run(a.L, a.n, not a.no_solve, a.cpu_rows)))


if __name__ == "__main__":
    main()
