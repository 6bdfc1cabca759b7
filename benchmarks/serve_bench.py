"""Served solve stream: open-loop Poisson arrivals into the continuous-batching server.

The stream is the L=10 5a5b FCI problem (63,504 determinants) under random
orbital rotations U = exp(kappa) of one seeded base integral set, as in an
orbital-optimisation sweep (CIFlow SimulatedAnnealing.cpp:72-86, 130-134); each
such request carries the base integrals and its U, and the server rotates the
integrals on the device (cigpu_ham_rotate) inside the measured path. Mixed
with uneven problems of the batched-solve shape (L uniform in 6..12, FCI with
1..L/2 electrons per spin or DOCI with 2..L/2 pairs) and a few L=12 6a6b
requests. The same request list runs through the mixed FP32/FP64 form and the
plain FP64 form; every result carries |dE0| against the plain FP64 result of the
same request solved to a tighter tolerance, and a seeded sample of the rotated
requests is checked against the oracle.

    python -m benchmarks.serve_bench --rate 1000 --requests 300
"""
from __future__ import annotations

import argparse
import json
import threading
import time

import numpy as np

from ciflow_gb300 import _abi as A
from ciflow_gb300.server import Server
from ciflow_gb300.ciflow import unitary_exp
from ciflow_gb300.synthetic import make_integrals


def rotation(L: int, sigma: float, seed: int) -> np.ndarray:
    """U = exp(-kappa) with kappa antisymmetric, N(0, sigma) entries drawn as
    synthetic.rotate_integrals draws them; rotating by U on the device gives the
    integrals rotate_integrals computes on the host."""
    rng = np.random.default_rng(seed)
    k = np.zeros((L, L))
    iu = np.triu_indices(L, 1)
    k[iu] = rng.normal(0.0, sigma, size=len(iu[0]))
    return unitary_exp(-(k - k.T))


def make_stream(n: int, seed: int = 4, frac_other: float = 0.15, every_big: int = 100):
    """Request list [(kind, ints, method, rotation or None)], deterministic in `seed`.
    The L=10 requests carry the base integrals and their rotation, applied on the
    device by the server (cigpu_ham_rotate)."""
    rng = np.random.default_rng(seed + 17)
    base = make_integrals(10, 5, 5, nchol=16, seed=seed)
    big = None
    out = []
    for i in range(n):
        if every_big and i % every_big == every_big // 2:
            if big is None:
                big = make_integrals(12, 6, 6, nchol=16, seed=1)
            out.append(("c1", big, A.FCI, None))
        elif rng.random() < frac_other:
            L = int(rng.integers(6, 13))
            if rng.random() < 0.5:
                ne = int(rng.integers(1, L // 2 + 1))
                out.append(("c3", make_integrals(L, ne, ne, nchol=16, seed=1000 + i), A.FCI, None))
            else:
                p = int(rng.integers(2, L // 2 + 1))
                out.append(("c3", make_integrals(L, p, p, nchol=16, seed=1000 + i), A.DOCI, None))
        else:
            out.append(("c4", base, A.FCI, rotation(10, 0.05, 10**6 + i)))
    return out


def pct(v, q):
    return float(np.percentile(np.asarray(v), q)) if len(v) else None


def run_stream(stream, precision: int, rate: float, tol: float, max_inflight: int, seed: int = 0):
    """Submits `stream` at Poisson arrival times; returns per-request results and the wall time."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=len(stream)) if rate > 0 else np.zeros(len(stream))
    with Server(max_inflight=max_inflight, max_queue=1 << 16) as srv:
        # warm-up: one request of each kind builds the allocator cache and kernel state
        seen = set()
        for kind, ints, m, rot in stream:
            if kind not in seen:
                seen.add(kind)
                srv.wait(srv.submit(ints, method=m, precision=precision, tol=tol, rot=rot))
        ids = [None] * len(stream)
        results = [None] * len(stream)
        t0 = time.perf_counter()

        def submitter():
            t = t0
            for i, (kind, ints, m, rot) in enumerate(stream):
                t += gaps[i]
                d = t - time.perf_counter()
                if d > 0:
                    time.sleep(d)
                ids[i] = srv.submit(ints, method=m, precision=precision, tol=tol, rot=rot)

        th = threading.Thread(target=submitter)
        th.start()
        th.join()
        for i, rid in enumerate(ids):
            results[i] = srv.wait(rid)
        wall = time.perf_counter() - t0
    return results, wall


def summarise(stream, results, wall):
    lat = {"all": [r["latency_s"] for r in results]}
    for k in ("c4", "c3", "c1"):
        lat[k] = [r["latency_s"] for (kind, _, _, _), r in zip(stream, results) if kind == k]
    ok = sum(r["status"] == A.OK for r in results)
    return {
        "solves_per_s": len(results) / wall,
        "wall_s": wall,
        "ok": ok,
        "p50_ms": {k: (pct(v, 50) * 1e3 if v else None) for k, v in lat.items()},
        "p99_ms": {k: (pct(v, 99) * 1e3 if v else None) for k, v in lat.items()},
        "counts": {k: len(v) for k, v in lat.items()},
        "matvecs_fp32": int(sum(r["matvecs_fp32"] for r in results)),
        "matvecs_fp64": int(sum(r["matvecs_fp64"] for r in results)),
    }


def oracle_check(stream, res_m, res_p, oracle, sample: int, seed: int) -> dict:
    """A seeded sample of the rotated L=10 requests against the oracle: the integrals
    rotated on the host (synthetic.rotate_integrals, the transform the reference's
    OrbitalTransform::fillHamCI performs, pinned by tests/golden/rotate.*), the
    oracle's CRS and ARPACK (eigsh, tol 1e-12) on it."""
    from ciflow_gb300.synthetic import rotate_integrals
    O = oracle
    idx = [i for i, s in enumerate(stream) if s[0] == "c4"]
    pick = sorted(np.random.default_rng(seed + 99).choice(idx, size=min(sample, len(idx)), replace=False).tolist())
    errs_m, errs_p = [], []
    t0 = time.perf_counter()
    for i in pick:
        ints = rotate_integrals(stream[i][1], 0.05, seed=10**6 + i)
        e_ref, _ = O.lowest_eigenpair(O.build_upper(O.FCI, ints), tol=1e-12)
        e_ref += ints.econst
        errs_m.append(abs(res_m[i]["e0"] - e_ref))
        errs_p.append(abs(res_p[i]["e0"] - e_ref))
    return {"requests": pick, "max_abs_dE0_vs_oracle": {"mixed": float(max(errs_m)), "plain_fp64": float(max(errs_p))},
            "oracle_s": time.perf_counter() - t0}


def served(n: int = 300, rate: float = 1000.0, max_inflight: int = 8, tol_mixed: float = 1e-5,
           tol_fp64: float = 1e-5, tol_ref: float = 1e-8, every_big: int = 100, seed: int = 4,
           ref_results=None, extra_rates=(), oracle=None, oracle_sample: int = 3):
    """Both forms over the same stream; the tighter FP64 pass gives each request's E0.
    `extra_rates`: further arrival rates at which both forms run the same stream
    again, for latencies at and below saturation (summaries under "by_rate").
    `oracle`: the oracle module (given by the caller) for a sample check of the
    rotated requests, run after all timed streams."""
    stream = make_stream(n, seed=seed, every_big=every_big)
    res_m, wall_m = run_stream(stream, A.MIXED, rate, tol_mixed, max_inflight, seed=seed)
    res_p, wall_p = run_stream(stream, A.FP64, rate, tol_fp64, max_inflight, seed=seed)
    if ref_results is None:
        ref_results, _ = run_stream(stream, A.FP64, 0.0, tol_ref, max_inflight, seed=seed)
    e_ref = np.array([r["e0"] for r in ref_results])
    dm = np.abs(np.array([r["e0"] for r in res_m]) - e_ref)
    dp = np.abs(np.array([r["e0"] for r in res_p]) - e_ref)
    def failures(res, de, tol_e=1e-6):
        return [{"i": i, "kind": stream[i][0], "dim": r["dim"], "status": r["status"], "dE0": float(de[i]),
                 "residual": r["residual"], "mv32": r["matvecs_fp32"], "mv64": r["matvecs_fp64"]}
                for i, r in enumerate(res) if r["status"] != A.OK or de[i] > tol_e][:10]

    out = {
        "requests": n, "arrival_rate_per_s": rate, "max_inflight": max_inflight,
        "failures": {"mixed": failures(res_m, dm), "plain_fp64": failures(res_p, dp)},
        "mix": {k: sum(1 for s in stream if s[0] == k) for k in ("c4", "c3", "c1")},
        "dims": {"min": min(r["dim"] for r in res_m), "max": max(r["dim"] for r in res_m)},
        "mixed": summarise(stream, res_m, wall_m) | {"max_abs_dE0": float(dm.max()), "tol": tol_mixed},
        "plain_fp64": summarise(stream, res_p, wall_p) | {"max_abs_dE0": float(dp.max()), "tol": tol_fp64},
    }
    out["mixed_over_plain_solves_per_s"] = out["mixed"]["solves_per_s"] / out["plain_fp64"]["solves_per_s"]
    by_rate = {}
    for r in extra_rates:
        row = {}
        for prec, tol, name in ((A.MIXED, tol_mixed, "mixed"), (A.FP64, tol_fp64, "plain_fp64")):
            res, wall = run_stream(stream, prec, r, tol, max_inflight, seed=seed)
            de = np.abs(np.array([x["e0"] for x in res]) - e_ref)
            sm = summarise(stream, res, wall)
            row[name] = {"solves_per_s": sm["solves_per_s"], "p50_ms": sm["p50_ms"], "p99_ms": sm["p99_ms"],
                         "max_abs_dE0": float(de.max()), "failures": len(failures(res, de))}
        by_rate[str(r)] = row
    if by_rate:
        out["by_rate"] = by_rate
    if oracle is not None and oracle_sample > 0:
        out["oracle_sample"] = oracle_check(stream, res_m, res_p, oracle, oracle_sample, seed)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--requests", type=int, default=300)
    ap.add_argument("--rate", type=float, default=1000.0)
    ap.add_argument("--inflight", type=int, default=8)
    ap.add_argument("--tol", type=float, default=1e-5)
    ap.add_argument("--every-big", type=int, default=100)
    a = ap.parse_args()
    print(json.dumps(served(a.requests, a.rate, a.inflight, a.tol, a.tol, every_big=a.every_big)))


if __name__ == "__main__":
    main()
