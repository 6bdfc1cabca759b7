#!/usr/bin/env python
"""Benchmark of the lowest-eigenpair CI path: solves/s and p50/p99 latency at
|dE0| <= 1e-6 Eh, mixed precision vs plain FP64, on one GB300 per rank.

Workload (default): FCI, 12 orbitals, 6 alpha + 6 beta electrons, 853,776
determinants, seeded synthetic integrals (no dataset), ~1.55e9 stored
nonzeros. One step = one full solve: CRS build from device-resident integrals
+ GPU-resident Lanczos to the residual target (+ FP64 corrections for mixed).

    python bench.py [--gpus N --steps K --warmup W] [--impl reference]

Multi-GPU runs are replicas (each rank solves its own instance; no data-path
collective), scaling "weak". Rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "solves/s and p50/p99 latency at |dE0|<=1e-6 Eh, mixed vs plain FP64 on 1 GB300"
CLOCK_FIELDS = ("index,uuid,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["cigpu", "reference"], default="cigpu")
    ap.add_argument("--config", default="c1")
    ap.add_argument("--tol", type=float, default=1e-5, help="FP64 residual target (|dE0| ~ tol^2/gap)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="target length of the CPU baseline sample")
    ap.add_argument("--cpu-full-solve", type=int, default=1,
                    help="1: also time one whole CPU solve of L=10 5a5b end to end (about 20 s)")
    ap.add_argument("--served-requests", type=int, default=2000,
                    help="served-stream requests per form and rate (0 skips the served stream)")
    ap.add_argument("--served-rate", type=float, default=2000.0, help="Poisson arrival rate of the served stream (1/s)")
    ap.add_argument("--served-inflight", type=int, default=8, help="server worker slots")
    ap.add_argument("--served-low-rates", type=float, nargs="*", default=[1000.0, 200.0, 50.0],
                    help="further arrival rates (1/s), down to below saturation")
    ap.add_argument("--dets-orbitals", type=int, default=32,
                    help="orbitals of the CISD determinant-list section (0: skip); electrons per spin = L/4")
    ap.add_argument("--doci", type=int, default=1, help="1: the DOCI L=24 12-pair section (0 skips it)")
    ap.add_argument("--rdm", type=int, default=1,
                    help="1: RDMs of the mixed ground state, timed, with their errors against the oracle (0 skips)")
    ap.add_argument("--orbopt-steps", type=int, default=600,
                    help="simulated-annealing steps of the orbital-optimisation section (0: skip)")
    ap.add_argument("--batched-problems", type=int, default=512,
                    help="uneven problems of the batched-solve comparison (0 skips it)")
    return ap.parse_args()


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi samples every 200 ms while the timed region runs."""

    def __init__(self, uuid: str | None):
        self.uuid = uuid
        self.rows = []
        self.proc = None
        self.thread = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={CLOCK_FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 10:
                self.rows.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        rows = [r for r in self.rows if self.uuid is None or self.uuid in r[1]] or self.rows
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[2]) for r in rows if num(r[2]) is not None]
        mx = [num(r[3]) for r in rows if num(r[3]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[6:10]) if v.strip().lower() == "active"})
        under = sorted(sm)[len(sm) // 4:] if sm else []  # drop idle samples at the edges
        return {"sm_mhz": statistics.median(under) if under else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows),
                "power_w_max": max((num(r[4]) or 0) for r in rows)}


def measured_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": d["hbm_gbs"], "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def ncu_traffic(kernel: str) -> float | None:
    """DRAM bytes per launch of `kernel` from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", f"{kernel}.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("traffic_bytes_per_launch_full_workload:"):
            try:
                return float(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


# ---------------------------------------------------------------------------
# Cross-rank reductions of the replica runs (one process per GPU; the timed
# region's length is the slowest rank's, throughputs add up).
def reduce_over_ranks(values, dist, op: str = "max", device: str = "cuda") -> list:
    if dist is None:
        return [float(v) for v in values]
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return [float(v) for v in t.tolist()]


def job_throughput(units_per_rank: float, seconds: float, world: int, dist, device: str = "cuda"):
    """(whole-job units/s, slowest rank's seconds): every rank processed
    units_per_rank; the job took as long as its slowest rank."""
    slowest = reduce_over_ranks([seconds], dist, "max", device)[0]
    return world * units_per_rank / slowest, slowest


def calibration(cfg_name: str) -> dict | None:
    """The committed calibration of the oracle port against the reference itself
    (tests/golden/calibration.json, made by tests/golden/make_golden.py on a host
    with the reference tree): reference/port time ratios of the build and of the
    serial Sym::mvprod at the same thread count, and ARPACK's matvec count at the
    reference's settings (which='SA', ncv=42, tol=0) driving the reference mvprod."""
    p = os.path.join(ROOT, "tests", "golden", "calibration.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    if cfg_name not in d:
        return None
    rec = dict(d[cfg_name])
    rec.update({"host": d.get("host"), "threads": d.get("threads")})
    return rec


def cpu_baseline(cfg_name: str, ints, threads: int, target_s: float) -> dict:
    """The reference CPU solve of the workload, estimated from the oracle port (the
    restatement of the reference build and serial Sym::mvprod) timed on a bounded
    sample of rows on these host cores and calibrated by the committed
    reference/port ratios: t = k_build t_build + n_arpack k_mv t_mvprod, with
    n_arpack the reference ARPACK run's matvec count."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import oracle as O
    from ciflow_gb300.synthetic import CONFIGS
    method = O.DOCI if CONFIGS[cfg_name]["method"] == "DOCI" else O.FCI
    n = O.dim(method, ints.L, ints.nup, ints.ndown)
    os.environ["OMP_NUM_THREADS"] = str(threads)
    t_start = time.perf_counter()
    # size the sample from a short probe
    probe = max(200, min(n, 2000))
    t0 = time.perf_counter()
    O.build_rows(method, ints, 0, probe)
    tp = time.perf_counter() - t0
    rows = int(min(n, max(probe, probe * (0.6 * target_s) / max(tp, 1e-6))))
    stride_start = (n - rows) // 2
    t0 = time.perf_counter()
    off, col, val = O.build_rows(method, ints, stride_start, stride_start + rows)
    t_build = time.perf_counter() - t0
    x = np.random.default_rng(0).standard_normal(n)
    y = np.zeros(n)
    t0 = time.perf_counter()
    O.sym_mvprod_rows(stride_start, off, col, val, x, y)
    t_mv = time.perf_counter() - t0
    frac = rows / n
    full_build = t_build / frac
    full_mv = t_mv / frac
    cal = calibration(cfg_name)
    if cal:
        n_mv, k_b, k_mv = cal["arpack_matvecs"], cal["build_ratio_ref_over_port"], cal["mvprod_ratio_ref_over_port"]
    else:  # no calibration: the port as measured and ARPACK's count unknown
        n_mv, k_b, k_mv = 105, 1.0, 1.0
    t_solve = k_b * full_build + n_mv * k_mv * full_mv
    return {"value": 1.0 / t_solve, "unit": "solves/s", "cores": threads, "kind": "port",
            "sample": (f"rows {stride_start}..{stride_start + rows} of {n} ({100 * frac:.2f}%): port build "
                       f"{t_build:.2f}s with {threads} threads (the reference build_parallel algorithm with sorted "
                       f"row insertion), serial Sym::mvprod {t_mv:.3f}s; full solve = {k_b:.2f} x {full_build:.1f}s "
                       f"build + {n_mv} ARPACK matvecs x {k_mv:.3f} x {full_mv:.2f}s"),
            "extrapolated_build_s": full_build, "extrapolated_mvprod_s": full_mv,
            "solve_s_estimate": t_solve, "port_uncalibrated_solve_s": full_build + n_mv * full_mv,
            "arpack_matvecs": n_mv,
            "calibration": ({"build_ratio_ref_over_port": k_b, "mvprod_ratio_ref_over_port": k_mv,
                             "measured_on": f"{cal['host']}, {cal['threads']} threads",
                             "source": "tests/golden/calibration.json"} if cal else None),
            "sample_wall_s": time.perf_counter() - t_start}


def cpu_full_solve(cfg_name: str, threads: int) -> dict:
    """One whole CPU solve, measured end to end, not extrapolated: the oracle port's
    build (all threads) and ARPACK (scipy eigsh, which='SA', ncv=42, tol=0, as
    SparseMatrix_CRS::arpackDiagonalize) driving the port's serial Sym::mvprod."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import scipy.sparse.linalg as sla
    import oracle as O
    from ciflow_gb300.synthetic import CONFIGS, config_integrals
    cfg = CONFIGS[cfg_name]
    method = O.DOCI if cfg["method"] == "DOCI" else O.FCI
    ints = config_integrals(cfg_name)
    os.environ["OMP_NUM_THREADS"] = str(threads)
    t0 = time.perf_counter()
    m = O.build_upper(method, ints)
    t_build = time.perf_counter() - t0
    count = [0]

    def mv(v):
        count[0] += 1
        return O.sym_mvprod(m, v)

    n = m.n
    op = sla.LinearOperator((n, n), matvec=mv, dtype=np.float64)
    t1 = time.perf_counter()
    w, _ = sla.eigsh(op, k=1, which="SA", ncv=min(42, n - 1), tol=0, maxiter=3 * n,
                     v0=np.random.default_rng(12345).standard_normal(n))
    t_eig = time.perf_counter() - t1
    out = {"workload": f"{cfg['method']} L={cfg['L']} {cfg['nup']}a{cfg['ndown']}b ({n} determinants)",
           "solve_s": t_build + t_eig, "build_s": t_build, "eigensolve_s": t_eig, "matvecs": count[0],
           "cores": threads, "kind": "port", "e0": float(w[0]) + ints.econst}
    gpath = os.path.join(ROOT, "tests", "golden", f"{cfg_name}.json")
    if os.path.exists(gpath):
        with open(gpath) as f:
            out["abs_dE0_vs_reference"] = abs(out["e0"] - json.load(f)["e0"])
    cal = calibration(cfg_name)
    if cal:
        out["reference_solve_s_measured_at_calibration"] = cal["ref_solve_s"]
        out["port_solve_s_at_calibration"] = cal["port_build_s"] + cal["arpack_matvecs"] * cal["port_mvprod_s"]
    return out


def small_solves(lib, cfg_name: str, tol: float, reps: int = 5) -> dict:
    """Whole solves of a small configuration on the GPU through the C ABI with host
    buffers (create + build + solve + eigenvector to the host), both forms, median of
    `reps` after one warm-up: the GPU side of the measured whole CPU solve."""
    import numpy as np

    from ciflow_gb300 import _abi as A
    from ciflow_gb300.synthetic import CONFIGS, config_integrals
    cfg = CONFIGS[cfg_name]
    ints = config_integrals(cfg_name)
    method = A.DOCI if cfg["method"] == "DOCI" else A.FCI
    h, eri = np.ascontiguousarray(ints.h), np.ascontiguousarray(ints.eri)
    golden = load_golden(cfg_name)
    out = {}
    for prec, name in ((A.MIXED, "mixed"), (A.FP64, "plain_fp64")):
        ts, e = [], None
        for i in range(reps + 1):
            t0 = time.perf_counter()
            ham, crs = ctypes.c_void_p(), ctypes.c_void_p()
            A.check(lib.cigpu_ham_create(ints.L, ints.nup, ints.ndown, ints.econst, A.ptr(h), A.ptr(eri),
                                         ctypes.byref(ham)))
            A.check(lib.cigpu_build(ham, method, prec, None, ctypes.byref(crs)))
            dim = ctypes.c_int64()
            lib.cigpu_crs_dims(crs, ctypes.byref(dim), None, None)
            c = np.empty(dim.value)
            info = A.SolveInfo()
            st = lib.cigpu_solve(crs, tol, 0, None, A.ptr(c), ctypes.byref(info))
            lib.cigpu_crs_destroy(crs)
            lib.cigpu_ham_destroy(ham)
            if st not in (A.OK, A.ENOCONV):
                A.check(st, "cigpu_solve")
            if i:
                ts.append(time.perf_counter() - t0)
            e = info.e0
        out[name] = {"solve_s": statistics.median(ts), "e0": e,
                     "abs_dE0_vs_reference": abs(e - golden["e0"]) if golden else None}
    return out


def config_dict(args, cfg: dict, golden: dict | None, world: int) -> dict:
    """The workload description both arms print (identical for the same config)."""
    return {"workload": f"{cfg['method']} L={cfg['L']} {cfg['nup']}a{cfg['ndown']}b "
                        f"({golden['dim'] if golden else '?'} determinants)",
            "name": args.config, **cfg, "tol_residual": args.tol,
            "l2": "inputs larger than L2 (CRS of ~1.55e9 nonzeros, 12-19 GB)" if args.config == "c1" else "n/a",
            "parallelism": f"replicas x{world}"}


def load_golden(name: str) -> dict | None:
    gpath = os.path.join(ROOT, "tests", "golden", f"{name}.json")
    if os.path.exists(gpath):
        with open(gpath) as f:
            return json.load(f)
    return None


def rdm_section(lib, ham, method: int, ints, cfg_name: str, tol: float, stream, reps: int = 3,
                check: bool = True) -> dict:
    """1-RDM and 2-RDM of the mixed ground state through cigpu_rdm (host c in, host
    RDMs out), timed with CUDA events on the CRS stream, and their errors against the
    oracle: the oracle's restatement of DensFCI/DensDOCI on the same vector (kernel
    parity) and, where the fixture holds them, the RDMs of the reference's own FP64
    ARPACK ground state (error of the mixed state), with |E_dens - E_CI|."""
    import numpy as np
    import torch

    from ciflow_gb300 import _abi as A
    sh = ctypes.c_void_p(stream.cuda_stream)
    crs = ctypes.c_void_p()
    A.check(lib.cigpu_build(ham, method, A.MIXED, sh, ctypes.byref(crs)))
    dim = ctypes.c_int64()
    lib.cigpu_crs_dims(crs, ctypes.byref(dim), None, None)
    c = np.empty(dim.value)
    info = A.SolveInfo()
    st = lib.cigpu_solve(crs, tol, 0, None, A.ptr(c), ctypes.byref(info))
    if st not in (A.OK, A.ENOCONV):
        A.check(st, "cigpu_solve")
    L = ints.L
    np_ = L * (L - 1) // 2
    two = method == A.FCI or L <= 32
    r1 = np.empty((2, L, L))
    aa, ab, bb = np.empty((np_, np_)), np.empty((L * L, L * L)), np.empty((np_, np_))
    outs = (A.ptr(r1), A.ptr(aa), A.ptr(ab), A.ptr(bb)) if two else (A.ptr(r1), None, None, None)
    ms = []
    for i in range(reps + 1):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        A.check(lib.cigpu_rdm(crs, A.ptr(c), *outs), "cigpu_rdm")
        e1.record(stream)
        torch.cuda.synchronize()
        if i:  # the first call warms the allocator cache
            ms.append(e0.elapsed_time(e1))
    lib.cigpu_crs_destroy(crs)
    out = {"state": "mixed ground state", "e0": info.e0, "residual": info.residual,
           "rdms": "1-RDM + 2-RDM (aa, ab, bb)" if two else "1-RDM",
           "ms_per_call": statistics.median(ms), "ms_all": [round(x, 3) for x in ms],
           "path": "cigpu_rdm with host c and host outputs (H2D of c and D2H of the RDMs included)"}
    if not check:
        return out
    # the oracle as the checker (after the timed calls)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    t0 = time.perf_counter()
    ref = O.rdm(O.FCI if method == A.FCI else O.DOCI, L, ints.nup, ints.ndown, c)
    out["oracle_s"] = time.perf_counter() - t0
    got = (r1, aa, ab, bb)
    names = ("rdm1", "rdm2_aa", "rdm2_ab", "rdm2_bb") if two else ("rdm1",)
    out["max_abs_err_vs_oracle_same_vector"] = {n: float(np.abs(g - r).max()) for n, g, r in zip(names, got, ref)}
    if two:
        out["abs_E_dens_minus_E_ci"] = abs(O.dens_energy(ints, r1, aa, ab, bb) - info.e0)
    npz = os.path.join(ROOT, "tests", "golden", f"{cfg_name}.npz")
    if os.path.exists(npz):
        g = np.load(npz)
        keys = {"rdm1": "rdm1", "rdm2_aa": "aa", "rdm2_ab": "ab", "rdm2_bb": "bb"}
        errs = {n: float(np.abs(x - g[keys[n]]).max()) for n, x in zip(names, got) if keys[n] in g}
        if errs:
            out["max_abs_err_vs_reference_fp64_state"] = errs
    return out


def host_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# ---------------------------------------------------------------------------
def run_reference(args, rank: int, world: int):
    """--impl reference: the reference CPU implementation of the path on the host
    cores, rank 0 only. Each step is a bounded sample of the workload (the oracle
    port's build of a slice of rows with all threads, and the serial matvec over
    it); the value is the full solve those samples give, calibrated against the
    reference itself (ARPACK's matvec count and the reference/port time ratios,
    tests/golden/calibration.json). One whole L=10 5a5b solve is also measured end
    to end without extrapolation."""
    if rank != 0:
        return
    from ciflow_gb300.synthetic import CONFIGS, config_integrals
    ints = config_integrals(args.config)
    threads = host_threads()
    vals, walls = [], []
    for _ in range(args.warmup):
        cpu_baseline(args.config, ints, threads, min(args.cpu_seconds, 4.0) / 2)
    for _ in range(args.steps):
        t0 = time.perf_counter()
        vals.append(cpu_baseline(args.config, ints, threads, args.cpu_seconds / 2))
        walls.append(time.perf_counter() - t0)
    v = statistics.median([b["value"] for b in vals])
    full = cpu_full_solve("c4", threads) if args.cpu_full_solve else None
    cfg = CONFIGS[args.config]
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": "solves/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * statistics.mean(walls),
           "ms_per_solve_estimate": 1000.0 / v, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded integrals)",
           "config": config_dict(args, cfg, load_golden(args.config), world),
           "step": "one bounded sample of the solve (build of a slice of rows + serial matvec over it); "
                   "value = the full solve the sample gives, calibrated against the reference",
           "cpu_baseline": {**vals[-1], "value": v},
           "cpu_full_solve_c4": full,
           "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def run_cigpu(args, rank: int, world: int, dist):
    import numpy as np
    import torch

    from ciflow_gb300 import _abi as A
    from ciflow_gb300.synthetic import CONFIGS, config_integrals

    torch.cuda.set_device(0)
    lib = A.lib()
    cfg = CONFIGS[args.config]
    method = A.DOCI if cfg["method"] == "DOCI" else A.FCI
    ints = config_integrals(args.config)
    golden = None
    gpath = os.path.join(ROOT, "tests", "golden", f"{args.config}.json")
    if os.path.exists(gpath):
        with open(gpath) as f:
            golden = json.load(f)
    stream = torch.cuda.Stream()
    sh = ctypes.c_void_p(stream.cuda_stream)
    h = np.ascontiguousarray(ints.h)
    eri = np.ascontiguousarray(ints.eri)
    ham = ctypes.c_void_p()
    A.check(lib.cigpu_ham_create(ints.L, ints.nup, ints.ndown, ints.econst, A.ptr(h), A.ptr(eri), ctypes.byref(ham)))

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    def solve_once(precision):
        crs = ctypes.c_void_p()
        A.check(lib.cigpu_build(ham, method, precision, sh, ctypes.byref(crs)), "build")
        info = A.SolveInfo()
        st = lib.cigpu_solve(crs, args.tol, 0, None, None, ctypes.byref(info))
        lib.cigpu_crs_destroy(crs)
        if st not in (A.OK, A.ENOCONV):
            A.check(st, "solve")
        return info

    def timed(precision):
        for _ in range(args.warmup):
            solve_once(precision)
        barrier()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        infos = []
        l0 = lib.cigpu_kernel_launches()
        for e0, e1 in evs:
            e0.record(stream)
            infos.append(solve_once(precision))
            e1.record(stream)
        barrier()
        launches = lib.cigpu_kernel_launches() - l0
        ms = [a.elapsed_time(b) for a, b in evs]
        tot = reduce_over_ranks([sum(ms) / 1000.0], dist, "max")[0]
        return ms, tot, infos, launches

    uuid = None
    try:
        uuid = str(torch.cuda.get_device_properties(0).uuid)
    except Exception:
        pass

    with ClockSampler(uuid) as clk:
        ms_mixed, tot_mixed, inf_mixed, launches_mixed = timed(A.MIXED)
        ms_plain, tot_plain, inf_plain, launches_plain = timed(A.FP64)

    def summary(ms, tot, infos):
        srt = sorted(ms)
        de = [abs(i.e0 - golden["e0"]) for i in infos] if golden else []
        return {"solves_per_s": world * len(ms) / tot, "ms_per_solve": statistics.mean(ms), "step_ms": [round(x, 3) for x in ms],
                "p50_ms": srt[len(srt) // 2], "p99_ms": srt[min(len(srt) - 1, int(round(0.99 * (len(srt) - 1))))],
                "max_abs_dE0": max(de) if de else None, "residual": max(i.residual for i in infos),
                "matvecs_fp64": infos[-1].matvecs_fp64, "matvecs_fp32": infos[-1].matvecs_fp32,
                "restarts": infos[-1].restarts, "corrections": infos[-1].corrections}

    mixed = summary(ms_mixed, tot_mixed, inf_mixed)
    plain = summary(ms_plain, tot_plain, inf_plain)

    # dominant kernels, timed alone with CUDA events on their stream: the mixed
    # method's FP32 product (the factorised sigma vector where it applies), the same
    # product from the stored FP32 slot values, and the plain FP64 matvec
    roof = {}
    peaks = measured_peaks()
    for prec, tag in ((A.MIXED, "fp32"), (A.MIXED, "fp32_slots"), (A.FP64, "fp64")):
        if tag == "fp32_slots":
            os.environ["CIGPU_FP32_PRODUCT"] = "slots"  # read by the build
        crs = ctypes.c_void_p()
        try:
            A.check(lib.cigpu_build(ham, method, prec, sh, ctypes.byref(crs)))
        finally:
            os.environ.pop("CIGPU_FP32_PRODUCT", None)
        kind = A.fp32_product(crs) if prec == A.MIXED else (A.FP32_STORED, 0, 0)
        if tag == "fp32_slots" and roof.get("fp32", {}).get("bound") == "hbm":
            lib.cigpu_crs_destroy(crs)  # the default product is the stored one already
            continue
        dim, nu, nf = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        lib.cigpu_crs_dims(crs, ctypes.byref(dim), ctypes.byref(nu), ctypes.byref(nf))
        f32 = tag.startswith("fp32")
        dt = torch.float32 if f32 else torch.float64
        x = torch.randn(dim.value, device="cuda", dtype=dt)
        y = torch.empty_like(x)
        dtype_code = 1 if f32 else 0
        for _ in range(3):
            lib.cigpu_mvprod_device(crs, A.ptr(x), A.ptr(y), dtype_code, sh)
        reps = 20
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            lib.cigpu_mvprod_device(crs, A.ptr(x), A.ptr(y), dtype_code, sh)
        e1.record(stream)
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / 1000.0 / reps
        shape = f"{cfg['method'].lower()}_L{cfg['L']}_{cfg['nup']}a{cfg['ndown']}b"
        if kind[0] == A.FP32_SIGMA:
            # the factorised sigma vector reads the matrix from no DRAM stream: its work
            # is FP32 FMAs over every determinant's single excitations times the rank,
            # on vectors that stay in L2; its roofline is the FP32 FMA rate
            w = A.sigma_work(cfg["L"], cfg["nup"], cfg["ndown"], kind[1], kind[2])
            sms = torch.cuda.get_device_properties(0).multi_processor_count
            peak_tf = sms * 128 * 2 * 2070e6 / 1e12
            ach = w["flops"] / t / 1e12
            roof[tag] = {"bound": "fp32", "achieved": ach, "peak": peak_tf, "unit": "TFLOP/s", "frac": ach / peak_tf,
                         "traffic": ncu_traffic(f"sigma_fp32_{shape}"), "algorithmic_flops": w["flops"],
                         "l2_bytes_per_launch": w["l2_bytes"], "l2_gbs": w["l2_bytes"] / t / 1e9,
                         "l2_note": "the factor vectors the kernels read per excitation live in L2 (about half of "
                                    "those reads hit L1); ncu: L2 27% busy, issue 46-50% at L=11",
                         "layout": f"sigma-fp32 (rank {kind[1]}, padded {kind[2]})",
                         "kernels": "k_transpose32 + k_sigma_a + k_sigma_b", "ms_per_launch": t * 1000,
                         "nnz_full": nf.value,
                         "peak_source": "nominal FP32 FMA rate: SMs x 128 lanes x 2 flops x 2070 MHz "
                                        "(no measured FP32 figure)"}
        else:
            bytes_alg, layout = A.matvec_bytes(crs, f32)
            ach = bytes_alg / t / 1e9
            roof[tag] = {"bound": "hbm", "achieved": ach, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                         "frac": ach / peaks["hbm_gbs"],
                         "traffic": ncu_traffic(f"spmv_{'fp32' if f32 else 'fp64'}_{shape}"),
                         "algorithmic_bytes": bytes_alg, "layout": layout, "ms_per_launch": t * 1000,
                         "nnz_full": nf.value, "peak_source": peaks["source"]}
        if tag == "fp64":
            # the plain FP64 matvec issues one DFMA per stored slot (padding included);
            # GB300 retires 2 FP64 FMAs per clock per SM, so this is its bound
            lay, stored = ctypes.c_int(), ctypes.c_int64()
            lib.cigpu_crs_layout(crs, ctypes.byref(lay), ctypes.byref(stored))
            fmas = stored.value if stored.value > 0 else nf.value
            sms = torch.cuda.get_device_properties(0).multi_processor_count
            peak_fma = 2.0 * sms * 2070e6  # at the maximum SM clock (2070 MHz on GB300)
            roof[tag]["fp64_pipe"] = {"dfma_per_launch": fmas, "achieved_dfma_per_s": fmas / t,
                                      "peak_dfma_per_s": peak_fma, "frac": fmas / t / peak_fma,
                                      "note": "2 FP64 FMA per clock per SM x SMs x 2070 MHz"}
        lib.cigpu_crs_destroy(crs)

    # e2e through the C ABI with host buffers, H2D of the integrals and D2H of c inside the region
    def e2e_once():
        hh = ctypes.c_void_p()
        A.check(lib.cigpu_ham_create(ints.L, ints.nup, ints.ndown, ints.econst, A.ptr(h), A.ptr(eri),
                                     ctypes.byref(hh)))
        crs = ctypes.c_void_p()
        A.check(lib.cigpu_build(hh, method, A.MIXED, None, ctypes.byref(crs)))
        info = A.SolveInfo()
        lib.cigpu_solve(crs, args.tol, 0, None, A.ptr(c_host), ctypes.byref(info))
        lib.cigpu_crs_destroy(crs)
        lib.cigpu_ham_destroy(hh)
        return info

    dimv = golden["dim"] if golden else None
    c_host = np.empty(dimv if dimv else 1)
    if not dimv:
        crs = ctypes.c_void_p()
        A.check(lib.cigpu_build(ham, method, A.MIXED, sh, ctypes.byref(crs)))
        d = ctypes.c_int64()
        lib.cigpu_crs_dims(crs, ctypes.byref(d), None, None)
        lib.cigpu_crs_destroy(crs)
        c_host = np.empty(d.value)
    e2e_once()
    barrier()
    t0 = time.perf_counter()
    n_e2e = max(1, min(args.steps, 3))
    for _ in range(n_e2e):
        e2e_once()
    barrier()
    e2e_value, t_e2e = job_throughput(n_e2e, time.perf_counter() - t0, world, dist)
    e2e = {"value": e2e_value, "unit": "solves/s",
           "h2d_bytes_per_step": int(h.nbytes + eri.nbytes), "d2h_bytes_per_step": int(c_host.nbytes),
           "path": "cigpu_ham_create + cigpu_build(MIXED) + cigpu_solve(c_out host), pageable host buffers"}

    # RDMs of the mixed ground state: time through the C ABI, errors against the oracle
    rdm = None
    if args.rdm:
        barrier()
        rdm = rdm_section(lib, ham, method, ints, args.config, args.tol, stream, check=(rank == 0))

    # served stream: L=10 5a5b FCI under random orbital rotations mixed with uneven
    # problems, Poisson arrivals into the continuous-batching server, both forms
    served = None
    if args.served_requests > 0:
        from benchmarks.serve_bench import served as run_served
        barrier()
        oracle_srv = None
        if rank == 0:  # a sample of the rotated requests against the oracle, after the timed streams
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import oracle as oracle_srv
        served = run_served(args.served_requests, args.served_rate, args.served_inflight, tol_mixed=args.tol,
                            tol_fp64=args.tol, seed=4 + rank, extra_rates=tuple(args.served_low_rates),
                            oracle=oracle_srv)
        if dist is not None:
            tm, tp = reduce_over_ranks([served["mixed"]["solves_per_s"], served["plain_fp64"]["solves_per_s"]],
                                       dist, "sum")
            served["mixed"]["solves_per_s_all_ranks"] = tm
            served["plain_fp64"]["solves_per_s_all_ranks"] = tp

    # batched uneven solves: one cigpu_solve_batch call against the same problems one at a time
    batched = None
    if args.batched_problems > 0:
        from benchmarks.batch_bench import run as run_batched
        barrier()
        oracle_mod = None
        if rank == 0:  # the sample check against the oracle runs after the timed calls
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import oracle as oracle_mod
        batched = run_batched(args.batched_problems, seed=rank, oracle=oracle_mod)

    # orbital optimisation: the optimisers' set_ham -> solve loop on the device
    orbopt = None
    if args.orbopt_steps > 0:
        from benchmarks.orbopt_bench import bench_section
        barrier()
        orbopt = bench_section(args.orbopt_steps, cpu_steps=20 if (rank == 0 and world == 1) else 0)

    # determinant lists (FCI_File / CI_Big): a CISD list, stored CRS and on-the-fly matvecs
    dets = None
    if args.dets_orbitals > 0:
        from benchmarks.dets_bench import run as run_dets
        barrier()
        dets = run_dets(args.dets_orbitals, args.dets_orbitals // 4,
                        cpu_rows=20000 if (rank == 0 and world == 1) else 0)

    # DOCI pair space, L=24 12 pairs: both forms' build + solve, matvec roofline and 1-RDM
    doci = None
    if args.doci:
        from benchmarks.doci_bench import run as run_doci
        barrier()
        checker = None
        if rank == 0:  # RDM errors against the oracle, after the timed calls
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import oracle as O
            checker = O.rdm
        doci = run_doci(args.tol, peak_gbs=peaks["hbm_gbs"], rdm_checker=checker)

    # the same L=10 5a5b problem the CPU solves whole below, on the GPU (C ABI, host buffers)
    small = small_solves(lib, "c4", args.tol) if args.cpu_full_solve else None

    cpu = None
    if rank == 0 and world == 1:
        cpu = cpu_baseline(args.config, ints, host_threads(), args.cpu_seconds)
        if args.cpu_full_solve:
            cpu["full_solve_c4"] = cpu_full_solve("c4", host_threads())
            cpu["full_solve_c4"]["gpu_same_problem"] = small

    lib.cigpu_ham_destroy(ham)
    if rank != 0:
        return
    out = {
        "metric": METRIC, "value": mixed["solves_per_s"], "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": mixed["ms_per_solve"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32/f64 (mixed)",
        "data": "synthetic (seeded integrals, no dataset)",
        "config": config_dict(args, cfg, golden, world),
        "p50_ms": mixed["p50_ms"], "p99_ms": mixed["p99_ms"],
        "mixed": mixed, "plain_fp64": plain,
        "mixed_over_plain": mixed["solves_per_s"] / plain["solves_per_s"],
        "roofline": roof["fp32"], "roofline_fp32_slots": roof.get("fp32_slots"), "roofline_fp64": roof["fp64"],
        "e2e": e2e, "gpu_launches": launches_mixed,
        "gpu_launches_plain": launches_plain,
        "clocks": clk.summary(),
        "rdm": rdm,
        "served": served,
        "doci": doci,
        "batched": batched,
        "orbopt": orbopt,
        "dets": dets,
        "cpu_baseline": cpu,
    }
    print(json.dumps(out), flush=True)


def main():
    args = parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        # one GPU per process: the library and torch both see it as device 0
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    dist = None
    if world > 1:
        import torch
        import torch.distributed as tdist
        torch.cuda.set_device(0)
        tdist.init_process_group("nccl")
        dist = tdist
    try:
        run_cigpu(args, rank, world, dist)
    finally:
        if dist is not None:
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
