"""Python client of the continuous-batching solve server (cigpu_server_* in the C ABI).

    srv = Server(max_inflight=4)
    rid = srv.submit(ints, method=FCI, precision=MIXED, tol=1e-6)
    res = srv.wait(rid)          # dict: status, e0, residual, latency_s, c, rdm1, ...

The server is the served form of the orbital optimisers' set_ham -> solve loop
(CIFlow SimulatedAnnealing.cpp:72-86, 130-134): many Hamiltonians of uneven size
solved concurrently on one GPU, each admitted when its device-memory estimate
fits the HBM budget.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _abi as A


@dataclass
class _Pending:
    L: int
    dim: int
    want_rdm: bool


def request_dim(L: int, nup: int, ndown: int, method: int) -> int:
    from math import comb
    return comb(L, nup) if method == A.DOCI else comb(L, nup) * comb(L, ndown)


class Server:
    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0, max_inflight: int = 4, max_queue: int = 4096):
        h = ctypes.c_void_p()
        A.check(A.lib().cigpu_server_create(device, hbm_budget_bytes, max_inflight, max_queue, ctypes.byref(h)),
                "cigpu_server_create")
        self.h = h
        self._pending: dict[int, _Pending] = {}

    def submit(self, ints, method: int = A.FCI, precision: int = A.MIXED, tol: float = 1e-6,
               want_rdm: bool = False, c0: np.ndarray | None = None, rot: np.ndarray | None = None) -> int:
        """Queues one lowest-eigenpair solve; raises CigpuError (EAGAIN: queue full,
        ENOMEM: can never fit the budget, EINVAL: bad integrals or rotation). `rot`: an
        orthogonal L x L matrix U; the integrals are rotated by it on the device first."""
        hh = np.ascontiguousarray(ints.h, dtype=np.float64)
        ee = np.ascontiguousarray(ints.eri, dtype=np.float64)
        cc = None if c0 is None else np.ascontiguousarray(c0, dtype=np.float64)
        uu = None if rot is None else np.ascontiguousarray(rot, dtype=np.float64)
        req = A.Request(ints.L, ints.nup, ints.ndown, method, precision, int(want_rdm), ints.econst, tol,
                        A.ptr(hh), A.ptr(ee), A.ptr(cc), A.ptr(uu))
        rid = ctypes.c_uint64()
        A.check(A.lib().cigpu_server_submit(self.h, ctypes.byref(req), ctypes.byref(rid)), "cigpu_server_submit")
        self._pending[rid.value] = _Pending(ints.L, request_dim(ints.L, ints.nup, ints.ndown, method), want_rdm)
        return rid.value

    def wait(self, rid: int, wait_ms: int = -1):
        """Result dict once request `rid` is done (the request is then released),
        None if it is still running after wait_ms (0 = poll, <0 = until done)."""
        p = self._pending[rid]
        res = A.Result()
        c = np.empty(p.dim)
        rdm1 = np.empty((2, p.L, p.L)) if p.want_rdm else None
        st = A.lib().cigpu_server_poll(self.h, rid, wait_ms, ctypes.byref(res), A.ptr(c), A.ptr(rdm1))
        if st == A.ETIMEDOUT or (st == A.OK and not res.done):
            return None
        A.check(st, "cigpu_server_poll")
        del self._pending[rid]
        ok = res.status in (A.OK, A.ENOCONV)
        return {"status": res.status, "dim": res.dim, "e0": res.info.e0, "residual": res.info.residual,
                "converged": bool(res.info.converged), "matvecs_fp64": res.info.matvecs_fp64,
                "matvecs_fp32": res.info.matvecs_fp32, "queued_s": res.queued_s, "latency_s": res.latency_s,
                "c": c if ok else None, "rdm1": rdm1 if ok else None}

    def cancel(self, rid: int) -> None:
        A.check(A.lib().cigpu_server_cancel(self.h, rid), "cigpu_server_cancel")

    def stats(self) -> dict:
        a, c, i = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        b = ctypes.c_size_t()
        A.check(A.lib().cigpu_server_stats(self.h, ctypes.byref(a), ctypes.byref(c), ctypes.byref(i),
                                           ctypes.byref(b)), "cigpu_server_stats")
        return {"admitted": a.value, "completed": c.value, "inflight": i.value, "hbm_in_use": b.value}

    def close(self) -> None:
        if self.h:
            A.lib().cigpu_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
