"""Orbital-optimisation throughput: simulated annealing and the DOCI local minimiser.

Workload: DOCI on seeded synthetic integrals (the reference's orbital optimisers
run on DOCI; FCI energies do not depend on the orbitals). A step of simulated
annealing is one proposal decided (rotation + build + eigensolve of the rotated
Hamiltonian, SimulatedAnnealing.cpp:306-391); a step of the local minimiser is
one iteration (DOCI pair matrices + pair scan of all L(L-1)/2 pairs + rotation +
build + eigensolve, LocalMinimizer.cpp:130-235). Arms:

* ``cold``: every solve from a random start, one proposal at a time (the
  reference's loop, where ARPACK restarts from scratch);
* ``warm``: every solve from the current eigenvector;
* ``speculate=K``: warm, K proposals solved concurrently on K streams (same chain).

    python -m benchmarks.orbopt_bench --L 16 --pairs 8 --steps 200
"""
from __future__ import annotations

import argparse
import ctypes
import json
import time

from ciflow_gb300 import _abi as A
from ciflow_gb300.ciflow import Hamiltonian
from ciflow_gb300.synthetic import make_integrals


def _create(ints, precision, warm, tol, seed):
    H = Hamiltonian.from_integrals(ints)
    cfg = A.OrboptConfig(A.DOCI, precision, tol, 1 if warm else 0, 0, seed)
    out = ctypes.c_void_p()
    A.check(A.lib().cigpu_orbopt_create(H.device(), ctypes.byref(cfg), ctypes.byref(out)), "cigpu_orbopt_create")
    return out.value


def _stats(opt):
    st = A.OrboptStats()
    A.check(A.lib().cigpu_orbopt_get(opt, None, None, None, ctypes.byref(st)), "cigpu_orbopt_get")
    return st.as_dict()


def anneal_arm(ints, steps, precision, warm, speculate, tol=1e-8, seed=11):
    """(steps/s, stats, e_last, e_opt) of one annealing run with the reference's
    parameters (0.4, 0.99, 1.4, 0.999; Main.cpp orb_opt)."""
    opt = _create(ints, precision, warm, tol, seed)
    try:
        before = _stats(opt)
        p = A.AnnealParams(0.4, 0.99, 1.4, 0.999, steps, 2000, 1e-7, speculate, 0)
        e = ctypes.c_double()
        t0 = time.perf_counter()
        A.check(A.lib().cigpu_orbopt_anneal(opt, ctypes.byref(p), ctypes.byref(e)), "cigpu_orbopt_anneal")
        dt = time.perf_counter() - t0
        st = _stats(opt)
    finally:
        A.lib().cigpu_orbopt_destroy(opt)
    decided = st["steps"] - before["steps"]
    st = {k: (st[k] - before[k] if k not in ("e_current", "e_opt") else st[k]) for k in st}
    ns = max(1, st["solves"])
    return {"steps_per_s": decided / dt, "seconds": dt, "steps": decided, "accepted": st["accepted"],
            "solves": st["solves"], "speculative_waste": st["speculative_waste"],
            "matvecs_per_solve": (st["matvecs_fp64"] + st["matvecs_fp32"]) / ns,
            "ms_per_solve": {"rotate": 1e3 * st["seconds_rotate"] / ns, "build": 1e3 * st["seconds_build"] / ns,
                             "eigensolve": 1e3 * st["seconds_solve"] / ns},
            "e_last": e.value, "e_opt": st["e_opt"]}


def local_arm(ints, iters, precision, warm, tol=1e-8, seed=21):
    opt = _create(ints, precision, warm, tol, seed)
    try:
        before = _stats(opt)
        p = A.LocalParams(1e-6, iters, iters, 0, 0)  # runs exactly `iters` iterations unless converged sooner
        e = ctypes.c_double()
        t0 = time.perf_counter()
        A.check(A.lib().cigpu_orbopt_local(opt, ctypes.byref(p), ctypes.byref(e)), "cigpu_orbopt_local")
        dt = time.perf_counter() - t0
        st = _stats(opt)
    finally:
        A.lib().cigpu_orbopt_destroy(opt)
    n = st["steps"] - before["steps"]
    return {"iterations_per_s": n / dt, "seconds": dt, "iterations": n,
            "scan_ms_per_iteration": 1e3 * (st["seconds_scan"] - before["seconds_scan"]) / max(1, n),
            "solve_ms_per_iteration": 1e3 * sum(st[k] - before[k] for k in ("seconds_rotate", "seconds_build",
                                                                             "seconds_solve")) / max(1, n),
            "e_final": e.value, "e_start": before["e_current"]}


def run(L=16, pairs=8, steps=200, iters=30, speculate=(8, 16), precision=A.FP64, seed=4):
    ints = make_integrals(L, pairs, pairs, nchol=16, seed=seed)
    anneal_arm(ints, 20, precision, True, 1)  # warm-up: kernels and allocator cache
    out = {"workload": f"DOCI L={L} {pairs} pairs", "precision": "fp64" if precision == A.FP64 else "mixed",
           "anneal": {}, "local": {}}
    out["anneal"]["cold"] = anneal_arm(ints, steps, precision, False, 1)
    out["anneal"]["warm"] = anneal_arm(ints, steps, precision, True, 1)
    for K in speculate:
        out["anneal"][f"speculate{K}"] = anneal_arm(ints, steps, precision, True, K)
    out["local"]["cold"] = local_arm(ints, iters, precision, False)
    out["local"]["warm"] = local_arm(ints, iters, precision, True)
    a = out["anneal"]
    out["anneal_speedup_over_cold"] = {k: v["steps_per_s"] / a["cold"]["steps_per_s"] for k, v in a.items()}
    return out


def cpu_anneal(ints, steps: int) -> dict:
    """The reference loop on the host cores: the oracle's restatement of the Jacobi
    rotation, of the reference CRS build and ARPACK with the reference's settings
    for each solve, over the first `steps` steps of the same chain parameters."""
    import os
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
    import orbopt as OO
    o = OO.Optimizer(ints, OO.O.DOCI, seed=11)
    t0 = time.perf_counter()
    _, acc, rej = o.anneal(OO.AnnealParams(steps=steps))
    dt = time.perf_counter() - t0
    return {"steps_per_s": (acc + rej) / dt, "steps": acc + rej, "seconds": dt}


def bench_section(steps=600, L=16, pairs=8, local_iters=30, cpu_steps=0, seed=4):
    """The bench.py sub-object: reference-like loop, warm starts, speculation and the
    mixed form on the same chain, plus the local minimiser."""
    ints = make_integrals(L, pairs, pairs, nchol=16, seed=seed)
    anneal_arm(ints, 20, A.FP64, True, 1)
    anneal_arm(ints, 20, A.MIXED, True, 8)
    a = {"cold_fp64": anneal_arm(ints, steps, A.FP64, False, 1),
         "warm_fp64": anneal_arm(ints, steps, A.FP64, True, 1),
         "warm_fp64_speculate16": anneal_arm(ints, steps, A.FP64, True, 16),
         "warm_mixed_speculate16": anneal_arm(ints, steps, A.MIXED, True, 16)}
    loc = {"warm_fp64": local_arm(ints, local_iters, A.FP64, True),
           "warm_mixed": local_arm(ints, local_iters, A.MIXED, True)}
    out = {"workload": f"DOCI L={L} {pairs} pairs ({ints.L} orbitals, seeded synthetic integrals)",
           "anneal_params": "SimulatedAnnealing(cim, 0.4, 0.99, 1.4, 0.999) as in Main.cpp orb_opt",
           "anneal_steps": steps, "anneal": a, "local": loc,
           "speedup_over_cold_fp64": {k: v["steps_per_s"] / a["cold_fp64"]["steps_per_s"] for k, v in a.items()},
           "same_chain": len({(v["accepted"], v["steps"]) for v in a.values()}) == 1}
    if cpu_steps > 0:
        out["cpu_reference_loop"] = cpu_anneal(ints, cpu_steps)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--L", type=int, default=16)
    ap.add_argument("--pairs", type=int, default=8)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--iters", type=int, default=30)
    ap.add_argument("--speculate", type=int, nargs="*", default=[8, 16])
    ap.add_argument("--mixed", action="store_true")
    a = ap.parse_args()
    print(json.dumps(run(a.L, a.pairs, a.steps, a.iters, tuple(a.speculate), A.MIXED if a.mixed else A.FP64)))


if __name__ == "__main__":
    main()
