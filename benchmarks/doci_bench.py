"""DOCI pair-space solve: L=24, 12 pairs (2,704,156 pair determinants).

Workload: the DOCI configuration of the reference's benchmark set, seeded synthetic
integrals (24 Cholesky vectors). For the plain FP64 and the mixed form: the build
and lowest-eigenpair solve (wall time through the C ABI, second of two runs), the
matvec timed alone with CUDA events against its algorithmic bytes, the 1-RDM, and
|dE0| against the reference's E0 (tests/golden/c2.json, from the reference CRS).

    python -m benchmarks.doci_bench
"""
from __future__ import annotations

import ctypes
import json
import os
import time

import numpy as np

from ciflow_gb300 import _abi as A
from ciflow_gb300.synthetic import config_integrals

GOLDEN = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "tests", "golden", "c2.json")


def run(tol: float = 1e-5, reps: int = 20, peak_gbs: float | None = None, rdm_checker=None) -> dict:
    """rdm_checker(method, L, nup, ndown, c) -> (rdm1, aa, ab, bb): the oracle's RDMs,
    given by the caller; the 1-RDM of each form is then compared with it on the
    same vector and with the reference's own 1-RDM of its FP64 ground state."""
    import torch  # device buffers and CUDA events for the matvec timing

    lib = A.lib()
    ints = config_integrals("c2")
    golden = None
    if os.path.exists(GOLDEN):
        with open(GOLDEN) as f:
            golden = json.load(f)
    h = np.ascontiguousarray(ints.h)
    eri = np.ascontiguousarray(ints.eri)
    ham = ctypes.c_void_p()
    A.check(lib.cigpu_ham_create(ints.L, ints.nup, ints.ndown, ints.econst, A.ptr(h), A.ptr(eri), ctypes.byref(ham)))
    stream = torch.cuda.Stream()
    sh = ctypes.c_void_p(stream.cuda_stream)
    out = {"workload": f"DOCI L={ints.L} {ints.nup} pairs, seeded synthetic integrals (24 Cholesky vectors)",
           "tol_residual": tol}
    try:
        for prec, name in ((A.MIXED, "mixed"), (A.FP64, "plain_fp64")):
            row = {}
            c = None
            walls = []
            nrun = 6  # the first run warms the allocator cache; the line reports the median of the other five
            for _ in range(nrun):
                t0 = time.perf_counter()
                crs = ctypes.c_void_p()
                A.check(lib.cigpu_build(ham, A.DOCI, prec, sh, ctypes.byref(crs)), "cigpu_build")
                t1 = time.perf_counter()
                dim, nu, nf = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
                lib.cigpu_crs_dims(crs, ctypes.byref(dim), ctypes.byref(nu), ctypes.byref(nf))
                c = np.empty(dim.value)
                info = A.SolveInfo()
                st = lib.cigpu_solve(crs, tol, 0, None, A.ptr(c), ctypes.byref(info))
                t2 = time.perf_counter()
                if st not in (A.OK, A.ENOCONV):
                    A.check(st, "cigpu_solve")
                if _ > 0:
                    walls.append((t2 - t0, t1 - t0, t2 - t1))
                med = sorted(walls)[len(walls) // 2] if walls else (t2 - t0, t1 - t0, t2 - t1)
                row = {"dim": dim.value, "nnz_full": nf.value, "build_s": med[1], "solve_s": med[2],
                       "solves_per_s": 1.0 / med[0], "runs": len(walls), "e0": info.e0, "residual": info.residual,
                       "matvecs_fp32": info.matvecs_fp32, "matvecs_fp64": info.matvecs_fp64}
                if golden:
                    row["abs_dE0_vs_reference"] = abs(info.e0 - golden["e0"])
                if _ < nrun - 1:
                    lib.cigpu_crs_destroy(crs)
            # matvec of the form's working precision, timed alone
            fp32 = prec == A.MIXED
            dt = torch.float32 if fp32 else torch.float64
            x = torch.randn(dim.value, device="cuda", dtype=dt)
            y = torch.empty_like(x)
            code = 1 if fp32 else 0
            for _ in range(3):
                lib.cigpu_mvprod_device(crs, A.ptr(x), A.ptr(y), code, sh)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            for _ in range(reps):
                lib.cigpu_mvprod_device(crs, A.ptr(x), A.ptr(y), code, sh)
            e1.record(stream)
            torch.cuda.synchronize()
            t = e0.elapsed_time(e1) / 1000.0 / reps
            nbytes, layout = A.matvec_bytes(crs, fp32)
            row["matvec"] = {"layout": layout, "ms_per_launch": t * 1e3, "algorithmic_bytes": nbytes,
                             "achieved_gbs": nbytes / t / 1e9}
            if peak_gbs:
                row["matvec"]["frac_of_peak"] = nbytes / t / 1e9 / peak_gbs
            rdm1 = np.empty((2, ints.L, ints.L))
            ms = []
            for i in range(4):  # the first call warms the allocator cache
                ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                torch.cuda.synchronize()
                ev0.record(stream)
                A.check(lib.cigpu_rdm(crs, A.ptr(c), A.ptr(rdm1), None, None, None), "cigpu_rdm")
                ev1.record(stream)
                torch.cuda.synchronize()
                if i:
                    ms.append(ev0.elapsed_time(ev1))
            row["rdm1_ms"] = float(np.median(ms))
            row["rdm1_trace"] = float(rdm1[0].trace() + rdm1[1].trace())
            if rdm_checker is not None:
                ref = rdm_checker(1, ints.L, ints.nup, ints.ndown, c)
                row["rdm1_max_abs_err_vs_oracle_same_vector"] = float(np.abs(rdm1 - ref[0]).max())
            gnpz = GOLDEN[:-5] + ".npz"
            if os.path.exists(gnpz):
                row["rdm1_max_abs_err_vs_reference_fp64_state"] = float(np.abs(rdm1 - np.load(gnpz)["rdm1"]).max())
            lib.cigpu_crs_destroy(crs)
            out[name] = row
        m, p = out["mixed"], out["plain_fp64"]
        out["mixed_over_plain_solves_per_s"] = m["solves_per_s"] / p["solves_per_s"]
        out["abs_dE0_mixed_vs_plain"] = abs(m["e0"] - p["e0"])
    finally:
        lib.cigpu_ham_destroy(ham)
    return out


def main():
    print(json.dumps(run()))


if __name__ == "__main__":
    main()
