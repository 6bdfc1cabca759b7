"""ctypes binding of libcigpu.so (the C ABI declared in include/cigpu.h).

The library is the only compute path: importing this module loads the in-tree
``ciflow_gb300/_lib/libcigpu.so`` and raises if it is missing -- there is no
CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libcigpu.so")
CHECKED_LIB_PATH = os.path.join(HERE, "_lib", "libcigpu_checked.so")

OK, EINVAL, ENOMEM, EAGAIN, ECANCELED, ETIMEDOUT, ENOTSUP, ENOCONV, ECUDA, ENOTFOUND = (
    0, 22, 12, 11, 125, 110, 95, 200, 201, 202)
FCI, DOCI, DETS = 0, 1, 2
DETS_CRS, DETS_ONTHEFLY = 0, 1
FP64, MIXED = 0, 1
LAYOUT_CRS, LAYOUT_SLOTS, LAYOUT_ONTHEFLY, LAYOUT_PAIRS = 0, 1, 2, 3
FP32_STORED, FP32_SIGMA = 0, 1

_P = ctypes.c_void_p
_I = ctypes.c_int
_I64 = ctypes.c_int64
_D = ctypes.c_double


class SolveInfo(ctypes.Structure):
    _fields_ = [("e0", _D), ("residual", _D), ("error_bound", _D), ("gap", _D),
                ("matvecs_fp64", _I64), ("matvecs_fp32", _I64), ("restarts", ctypes.c_int32),
                ("corrections", ctypes.c_int32), ("converged", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("seconds", _D)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class Request(ctypes.Structure):
    _fields_ = [("L", ctypes.c_int32), ("nup", ctypes.c_int32), ("ndown", ctypes.c_int32),
                ("method", ctypes.c_int32), ("precision", ctypes.c_int32), ("want_rdm", ctypes.c_int32),
                ("econst", _D), ("tol", _D), ("h", _P), ("eri", _P), ("c0", _P), ("rot", _P)]


class BatchStats(ctypes.Structure):
    _fields_ = [("batched", ctypes.c_int32), ("individual", ctypes.c_int32), ("lanes", ctypes.c_int32),
                ("grid", ctypes.c_int32), ("steps", ctypes.c_int32), ("graph_launches", ctypes.c_int32),
                ("tuned", ctypes.c_int32), ("reserved", ctypes.c_int32), ("seconds_build", _D), ("seconds", _D)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class Result(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("done", ctypes.c_int32), ("dim", _I64), ("info", SolveInfo),
                ("queued_s", _D), ("latency_s", _D)]


class OrboptConfig(ctypes.Structure):
    _fields_ = [("method", ctypes.c_int32), ("precision", ctypes.c_int32), ("tol", _D),
                ("warm_start", ctypes.c_int32), ("reserved", ctypes.c_int32), ("seed", ctypes.c_uint64)]


class AnnealParams(ctypes.Structure):
    _fields_ = [("temp", _D), ("change_temp", _D), ("max_angle", _D), ("change_angle", _D),
                ("steps", _I64), ("max_unaccept", _I64), ("min_angle", _D), ("speculate", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class LocalParams(ctypes.Structure):
    _fields_ = [("conv_crit", _D), ("conv_steps", ctypes.c_int32), ("max_iters", ctypes.c_int32),
                ("dist_choice", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class OrboptStats(ctypes.Structure):
    _fields_ = [("e_current", _D), ("e_opt", _D), ("solves", _I64), ("steps", _I64), ("accepted", _I64),
                ("rejected", _I64), ("speculative_waste", _I64), ("matvecs_fp64", _I64), ("matvecs_fp32", _I64),
                ("seconds_rotate", _D), ("seconds_build", _D), ("seconds_solve", _D), ("seconds_scan", _D),
                ("seconds", _D)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


# name -> (restype, argtypes); every symbol include/cigpu.h declares
SIGNATURES = {
    "cigpu_get_version": (_I, []),
    "cigpu_strerror": (ctypes.c_char_p, [_I]),
    "cigpu_device_count": (_I, [_P]),
    "cigpu_kernel_launches": (_I64, []),
    "cigpu_checked_build": (_I, []),
    "cigpu_check_word": (_I, [_P, _I]),
    "cigpu_ham_create": (_I, [_I, _I, _I, _D, _P, _P, _P]),
    "cigpu_ham_destroy": (_I, [_P]),
    "cigpu_ham_rotate": (_I, [_P, _P, _P, _P]),
    "cigpu_unitary_exp": (_I, [_I, _P, _P]),
    "cigpu_ham_export": (_I, [_P, _P, _P]),
    "cigpu_build": (_I, [_P, _I, _I, _P, _P]),
    "cigpu_crs_destroy": (_I, [_P]),
    "cigpu_crs_dims": (_I, [_P, _P, _P, _P]),
    "cigpu_crs_layout": (_I, [_P, _P, _P]),
    "cigpu_crs_fp32_product": (_I, [_P, _P, _P, _P]),
    "cigpu_crs_export_upper": (_I, [_P, _P, _P, _P]),
    "cigpu_crs_export_full": (_I, [_P, _P, _P, _P]),
    "cigpu_mvprod": (_I, [_P, _P, _P, _P]),
    "cigpu_mvprod_device": (_I, [_P, _P, _P, _I, _P]),
    "cigpu_solve": (_I, [_P, _D, _I64, _P, _P, _P]),
    "cigpu_rdm": (_I, [_P, _P, _P, _P, _P, _P]),
    "cigpu_rdm_doci_noalloc": (_I, [_P, _P, _P, _P, _P, _P, _P]),
    "cigpu_server_create": (_I, [_I, ctypes.c_size_t, _I, _I, _P]),
    "cigpu_server_submit": (_I, [_P, _P, _P]),
    "cigpu_server_poll": (_I, [_P, ctypes.c_uint64, _I, _P, _P, _P]),
    "cigpu_server_cancel": (_I, [_P, ctypes.c_uint64]),
    "cigpu_server_stats": (_I, [_P, _P, _P, _P, _P]),
    "cigpu_server_destroy": (_I, [_P]),
    "cigpu_solve_batch": (_I, [_I, _P, _I64, _P, _P, _P, _P]),
    "cigpu_estimate_bytes": (_I, [_I, _I, _I, _I, _I, _P]),
    "cigpu_build_dets": (_I, [_P, _I64, _I, _P, _P, _I, _I, _P, _P]),
    "cigpu_build_dets_partial": (_I, [_P, _I64, _I, _P, _P, _I64, _P, _P]),
    "cigpu_dets_read": (_I, [ctypes.c_char_p, _I, _I64, _P, _P, _P, _P]),
    "cigpu_ham_read_psi4": (_I, [ctypes.c_char_p, _P, _P, _P, _P, _P, _P, _P, _P]),
    "cigpu_ham_write_psi4": (_I, [ctypes.c_char_p, _I, _I, _I, _D, _P, _P, _D]),
    "cigpu_write_civec": (_I, [ctypes.c_char_p, _I, _I, _I, _I, _I64, _P, _D, _D, _D, _P, _P, _I, ctypes.c_char_p]),
    "cigpu_write_rdm": (_I, [ctypes.c_char_p, _I, _P, _P, _P, _P]),
    "cigpu_ham_jacobi": (_I, [_P, _I, _I, _D, _P, _P]),
    "cigpu_doci_pair_scan": (_I, [_P, _P, _P, _P, _P]),
    "cigpu_orbopt_create": (_I, [_P, _P, _P]),
    "cigpu_orbopt_destroy": (_I, [_P]),
    "cigpu_orbopt_anneal": (_I, [_P, _P, _P]),
    "cigpu_orbopt_local": (_I, [_P, _P, _P]),
    "cigpu_orbopt_jacobi": (_I, [_P, _I, _I, _D, _P]),
    "cigpu_orbopt_natural": (_I, [_P, _I, _P]),
    "cigpu_orbopt_set_optimal": (_I, [_P]),
    "cigpu_orbopt_get": (_I, [_P, _P, _P, _P, _P]),
    "cigpu_orbopt_ham": (_I, [_P, _P]),
}

_lib = None
_lib_checked = None


class CigpuError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = lib().cigpu_strerror(status).decode() if _lib is not None else str(status)
        super().__init__(f"{what}: {msg} (status {status})" if what else f"{msg} (status {status})")


def _load(path: str):
    if not os.path.exists(path):
        raise ImportError(f"{os.path.basename(path)} is missing ({path}); build it with "
                          "`python -m ciflow_gb300.build` (nvcc, sm_103a)")
    l = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(l, name)
        f.restype = res
        f.argtypes = args
    return l


def lib():
    """The loaded library; raises if the CUDA extension has not been built."""
    global _lib
    if _lib is None:
        _lib = _load(LIB_PATH)
    return _lib


def checked_lib():
    """The checked build (bounds checks recorded in a device error word), loaded
    beside the regular library."""
    global _lib_checked
    if _lib_checked is None:
        _lib_checked = _load(CHECKED_LIB_PATH)
    return _lib_checked


def check(status: int, what: str = "") -> None:
    if status != OK:
        raise CigpuError(status, what)


def ptr(a) -> int | None:
    """Address of a numpy array (host) or torch tensor (device); None passes NULL."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data


def device_count() -> int:
    n = ctypes.c_int(0)
    lib().cigpu_device_count(ctypes.byref(n))
    return n.value


def estimate_bytes(L: int, nup: int, ndown: int, method: int, precision: int) -> int:
    """Device bytes a solve of this shape needs (the server's admission estimate)."""
    b = ctypes.c_size_t()
    check(lib().cigpu_estimate_bytes(L, nup, ndown, method, precision, ctypes.byref(b)), "cigpu_estimate_bytes")
    return b.value


def fp32_product(handle) -> tuple[int, int, int]:
    """(kind, rank, padded rank) of a MIXED matrix's FP32 product (FP32_STORED or
    FP32_SIGMA, the factorised direct-CI sigma vector)."""
    kind, rank, padded = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    check(lib().cigpu_crs_fp32_product(handle, ctypes.byref(kind), ctypes.byref(rank), ctypes.byref(padded)))
    return kind.value, rank.value, padded.value


def sigma_work(L: int, nup: int, ndown: int, rank: int, padded: int) -> dict:
    """Algorithmic work of one FP32 sigma product on the FCI space (nup, ndown) of L
    orbitals with `rank` factors: FP32 FMAs per determinant (pass 1: (R + 1) per
    single excitation and on the diagonal, the one-body matrix included; pass 2: R
    per excitation and on the diagonal) and the bytes the passes move through L2
    (x read per excitation, the padded factor vectors written twice and read per
    excitation, y written)."""
    from math import comb
    ns = nup * (L - nup) + ndown * (L - ndown)
    dim = comb(L, nup) * comb(L, ndown)
    fma = dim * (ns * (rank + 1) + rank + 1 + rank + ns * rank)
    l2 = dim * 4 * ((1 + ns) + 2 * padded + (1 + ns) * padded + 2)
    return {"fma": fma, "flops": 2 * fma, "l2_bytes": l2, "dim": dim, "excitations_per_det": ns}


def matvec_bytes(handle, fp32: bool) -> tuple[int, str]:
    """Algorithmic bytes of one matvec for the stored layout: one read of the stored
    matrix and of x, one write of y. FP32: FP32 values/x/y; FP64: FP64 x/y with FP64
    values (plain CRS) or the split hi + lo values (MIXED)."""
    dim, nu, nf = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    check(lib().cigpu_crs_dims(handle, ctypes.byref(dim), ctypes.byref(nu), ctypes.byref(nf)))
    lay, stored = ctypes.c_int(), ctypes.c_int64()
    check(lib().cigpu_crs_layout(handle, ctypes.byref(lay), ctypes.byref(stored)))
    n, m = dim.value, stored.value
    sx = 4 if fp32 else 8
    if lay.value == LAYOUT_PAIRS:  # matrix-free DOCI: strings, diagonal, x, y (hop gathers hit x in L2)
        return n * (8 + 3 * sx), "doci-pairs-fp32" if fp32 else "doci-pairs-fp64"
    if lay.value == LAYOUT_SLOTS:
        sv = 4 if fp32 else 8  # FP32 values, or FP64 values / FP32 hi + lo
        return m * sv + 2 * n * sx, "slots-fp32" if fp32 else "slots-fp64"
    sv = 4 if fp32 else 8
    return m * (sv + 4) + 8 * (n + 1) + 2 * n * sx, "crs-fp32" if fp32 else "crs-fp64"
