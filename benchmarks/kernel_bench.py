"""Kernel microbenchmark: launch one hot kernel of the CI path a few times on a
named configuration (used for profiler captures and roofline timing).

    python -m benchmarks.kernel_bench --config c4 --kernel spmv_f32 --reps 3

Kernels: spmv_f32 (the mixed form's FP32 matvec: the factorised sigma vector for
FCI where it applies, CIGPU_FP32_PRODUCT=slots for the stored FP32 values), spmv_f64 (the plain form's FP64
matvec), build_f64, build_f32 (the matrix build of either form), matvec_hilo (the
mixed form's FP64 product), solve_mixed / solve_fp64 (one eigensolve on a prebuilt
matrix), rdm (cigpu_rdm of a random normalised vector: 1- and 2-RDM, DOCI spaces
beyond 32 orbitals the 1-RDM).
Prints one JSON line with the CUDA-event time per launch and the algorithmic
bytes of the matvec.
"""
from __future__ import annotations

import argparse
import ctypes
import json

import numpy as np


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="c4")
    ap.add_argument("--kernel", default="spmv_f32",
                    choices=["spmv_f32", "spmv_f64", "build_f64", "build_f32", "matvec_hilo", "solve_mixed",
                             "solve_fp64", "rdm"])
    ap.add_argument("--tol", type=float, default=1e-5)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=1)
    args = ap.parse_args()

    import torch

    from ciflow_gb300 import _abi as A
    from ciflow_gb300.synthetic import CONFIGS, config_integrals

    lib = A.lib()
    cfg = CONFIGS[args.config]
    method = A.DOCI if cfg["method"] == "DOCI" else A.FCI
    ints = config_integrals(args.config)
    h = np.ascontiguousarray(ints.h)
    eri = np.ascontiguousarray(ints.eri)
    ham = ctypes.c_void_p()
    A.check(lib.cigpu_ham_create(ints.L, ints.nup, ints.ndown, ints.econst, A.ptr(h), A.ptr(eri), ctypes.byref(ham)))
    stream = torch.cuda.Stream()
    sh = ctypes.c_void_p(stream.cuda_stream)
    prec = A.MIXED if args.kernel in ("spmv_f32", "build_f32", "matvec_hilo", "solve_mixed", "rdm") else A.FP64

    def build():
        crs = ctypes.c_void_p()
        A.check(lib.cigpu_build(ham, method, prec, sh, ctypes.byref(crs)))
        return crs

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = {"config": args.config, "kernel": args.kernel, "reps": args.reps}
    if args.kernel.startswith("solve"):
        crs = build()
        info = A.SolveInfo()
        for _ in range(args.warmup):
            lib.cigpu_solve(crs, args.tol, 0, None, None, ctypes.byref(info))
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.reps):
            lib.cigpu_solve(crs, args.tol, 0, None, None, ctypes.byref(info))
        e1.record(stream)
        torch.cuda.synchronize()
        out["ms_per_solve"] = e0.elapsed_time(e1) / args.reps
        out["info"] = info.as_dict()
        lib.cigpu_crs_destroy(crs)
    elif args.kernel == "rdm":
        crs = build()
        dim = ctypes.c_int64()
        lib.cigpu_crs_dims(crs, ctypes.byref(dim), None, None)
        c = np.random.default_rng(0).standard_normal(dim.value)
        c /= np.linalg.norm(c)
        L = ints.L
        np_ = L * (L - 1) // 2
        r1, aa = np.empty((2, L, L)), np.empty((np_, np_))
        ab, bb = np.empty((L * L, L * L)), np.empty((np_, np_))
        outs = (A.ptr(r1), A.ptr(aa), A.ptr(ab), A.ptr(bb)) if L <= 32 else (A.ptr(r1), None, None, None)
        for _ in range(args.warmup):
            A.check(lib.cigpu_rdm(crs, A.ptr(c), *outs))
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.reps):
            A.check(lib.cigpu_rdm(crs, A.ptr(c), *outs))
        e1.record(stream)
        torch.cuda.synchronize()
        out["ms_per_rdm"] = e0.elapsed_time(e1) / args.reps
        out["trace"] = float(r1[0].trace() + r1[1].trace())
        lib.cigpu_crs_destroy(crs)
    elif args.kernel.startswith("build"):
        for _ in range(args.warmup):
            lib.cigpu_crs_destroy(build())
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.reps):
            lib.cigpu_crs_destroy(build())
        e1.record(stream)
        torch.cuda.synchronize()
        out["ms_per_build"] = e0.elapsed_time(e1) / args.reps
    else:
        crs = build()
        dim, nu, nf = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        lib.cigpu_crs_dims(crs, ctypes.byref(dim), ctypes.byref(nu), ctypes.byref(nf))
        f32 = args.kernel == "spmv_f32"
        dt = torch.float32 if f32 else torch.float64
        x = torch.randn(dim.value, device="cuda", dtype=dt)
        y = torch.empty_like(x)
        code = 1 if f32 else 0
        for _ in range(args.warmup):
            A.check(lib.cigpu_mvprod_device(crs, A.ptr(x), A.ptr(y), code, sh))
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.reps):
            lib.cigpu_mvprod_device(crs, A.ptr(x), A.ptr(y), code, sh)
        e1.record(stream)
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / args.reps
        n = dim.value
        kind, rank, padded = A.fp32_product(crs) if prec == A.MIXED else (A.FP32_STORED, 0, 0)
        if f32 and kind == A.FP32_SIGMA:  # the factorised sigma vector: FMAs, not a matrix stream
            w = A.sigma_work(ints.L, ints.nup, ints.ndown, rank, padded)
            out.update({"dim": n, "nnz_full": nf.value, "layout": f"sigma-fp32 (rank {rank}, padded {padded})",
                        "ms_per_launch": t, "algorithmic_flops": w["flops"],
                        "achieved_tflops": w["flops"] / (t / 1000) / 1e12, "l2_bytes": w["l2_bytes"]})
        else:
            alg, layout = A.matvec_bytes(crs, f32)
            out.update({"dim": n, "nnz_full": nf.value, "layout": layout, "ms_per_launch": t, "algorithmic_bytes": alg,
                        "achieved_gbs": alg / (t / 1000) / 1e9})
        lib.cigpu_crs_destroy(crs)
    lib.cigpu_ham_destroy(ham)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
