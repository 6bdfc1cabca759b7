"""Continuous-batching solve server (cigpu_server_*), through the C ABI.

The served stream is the orbital optimisers' set_ham -> solve loop (CIFlow
SimulatedAnnealing.cpp:72-86, 130-134) with many Hamiltonians in flight: the
L=10 5a5b FCI space under random orbital rotations, mixed with smaller FCI and
DOCI problems. The central check is that every result is the same alone and in
the mix: each request is solved once by itself (cigpu_build + cigpu_solve on the
calling thread) and once among concurrent requests on the server's worker
streams. The kernels are deterministic (no atomics, fixed grids), so the two
energies agree to 1e-10 Eh and the vectors to |<c_alone|c_mix>| >= 1 - 1e-10.
"""
import time

import numpy as np
import pytest

from ciflow_gb300 import _abi as A
from ciflow_gb300.ciflow import DOCI, FCI, Hamiltonian
from ciflow_gb300.server import Server
from ciflow_gb300.synthetic import make_integrals, rotate_integrals

pytestmark = pytest.mark.gpu

E_TOL = 1e-10


def mix_requests():
    base = make_integrals(10, 5, 5, nchol=16, seed=4)
    reqs = []
    for i in range(6):  # rotated L=10 FCI, as in an orbital-optimisation sweep
        reqs.append((rotate_integrals(base, 0.05, seed=10**6 + i), A.FCI, A.MIXED if i % 2 else A.FP64))
    for i, (L, n) in enumerate([(6, 3), (8, 2), (7, 3), (9, 4)]):  # small FCI problems
        reqs.append((make_integrals(L, n, n, nchol=16, seed=1000 + i), A.FCI, A.MIXED))
    for i, (L, p) in enumerate([(12, 6), (14, 5)]):  # DOCI problems
        reqs.append((make_integrals(L, p, p, nchol=16, seed=2000 + i), A.DOCI, A.MIXED if i else A.FP64))
    return reqs


def solve_alone(ints, method, precision, tol):
    ham = Hamiltonian.from_integrals(ints)
    cim = (DOCI if method == A.DOCI else FCI)(ham, precision=precision)
    cim.solve(tol=tol)
    return cim.get_ci_energy(), cim.get_eigvec(), cim.info


def test_same_result_alone_and_in_the_mix():
    tol = 1e-7
    reqs = mix_requests()
    alone = [solve_alone(ints, m, p, tol) for ints, m, p in reqs]
    with Server(max_inflight=4) as srv:
        ids = [srv.submit(ints, method=m, precision=p, tol=tol) for ints, m, p in reqs]
        peak_inflight = 0
        results = {}
        while len(results) < len(ids):
            peak_inflight = max(peak_inflight, srv.stats()["inflight"])
            for rid in ids:
                if rid not in results:
                    r = srv.wait(rid, wait_ms=0)
                    if r is not None:
                        results[rid] = r
            time.sleep(0.001)
        st = srv.stats()
    assert st["admitted"] == len(reqs) and st["completed"] == len(reqs) and st["inflight"] == 0
    assert st["hbm_in_use"] == 0
    assert peak_inflight >= 2, "requests never overlapped on the device"
    for (e_alone, c_alone, info), rid in zip(alone, ids):
        r = results[rid]
        assert r["status"] == A.OK and r["converged"]
        assert abs(r["e0"] - e_alone) <= E_TOL, (r["e0"], e_alone)
        assert abs(abs(float(np.dot(r["c"], c_alone))) - 1.0) <= 1e-10
        assert r["latency_s"] >= r["queued_s"] >= 0


def test_mixed_matches_fp64_within_the_served_tolerance():
    """|dE0| <= 1e-6 Eh between the mixed and plain forms of the same served request."""
    base = make_integrals(10, 5, 5, nchol=16, seed=4)
    ints = rotate_integrals(base, 0.05, seed=10**6 + 99)
    with Server(max_inflight=2) as srv:
        a = srv.submit(ints, method=A.FCI, precision=A.FP64, tol=1e-9)
        b = srv.submit(ints, method=A.FCI, precision=A.MIXED, tol=1e-6)
        ra, rb = srv.wait(a), srv.wait(b)
    assert ra["status"] == A.OK and rb["status"] == A.OK
    assert abs(ra["e0"] - rb["e0"]) <= 1e-6
    assert rb["matvecs_fp32"] > 0


def test_budget_admission_never_exceeds_the_budget():
    big = make_integrals(10, 5, 5, nchol=16, seed=4)
    small = [make_integrals(8, 4, 4, nchol=16, seed=3000 + i) for i in range(6)]
    est_big = A.estimate_bytes(10, 5, 5, A.FCI, A.FP64)
    est_small = A.estimate_bytes(8, 4, 4, A.FCI, A.FP64)
    budget = est_big + est_small  # the big one plus one small one at a time
    with Server(hbm_budget_bytes=budget, max_inflight=8) as srv:
        ids = [srv.submit(big, method=A.FCI, precision=A.FP64, tol=1e-8)]
        ids += [srv.submit(s, method=A.FCI, precision=A.FP64, tol=1e-8) for s in small]
        ids.append(srv.submit(big, method=A.FCI, precision=A.FP64, tol=1e-8))
        seen = 0
        pending = set(ids)
        res = {}
        while pending:
            s = srv.stats()
            assert s["hbm_in_use"] <= budget
            seen = max(seen, s["hbm_in_use"])
            for rid in list(pending):
                r = srv.wait(rid, wait_ms=0)
                if r is not None:
                    res[rid] = r
                    pending.discard(rid)
        assert srv.stats()["hbm_in_use"] == 0
    assert all(r["status"] == A.OK for r in res.values())
    assert res[ids[0]]["e0"] == pytest.approx(res[ids[-1]]["e0"], abs=E_TOL)
    assert seen > 0


def test_refusals_and_cancellation():
    big = make_integrals(11, 5, 5, nchol=16, seed=5)  # 213,444 determinants: long enough to queue behind
    small = make_integrals(6, 3, 3, nchol=8, seed=6)
    with Server(max_inflight=1, max_queue=1) as srv:
        first = srv.submit(big, method=A.FCI, precision=A.FP64, tol=1e-8)
        queued = srv.submit(small, method=A.FCI, precision=A.FP64, tol=1e-8)
        with pytest.raises(A.CigpuError) as e:  # queue of one is full
            srv.submit(small, method=A.FCI, precision=A.FP64, tol=1e-8)
        assert e.value.status == A.EAGAIN
        srv.cancel(queued)
        r = srv.wait(queued)
        assert r["status"] == A.ECANCELED and r["c"] is None
        srv.cancel(first)  # running: stops before the solve or finishes normally
        r = srv.wait(first)
        assert r["status"] in (A.OK, A.ECANCELED)
        with pytest.raises(A.CigpuError) as e:  # released after the completed poll
            srv.cancel(first)
        assert e.value.status == A.ENOTFOUND
        bad = make_integrals(6, 3, 3, nchol=8, seed=6)
        bad.eri[0, 1, 2, 3] += 1e-3  # breaks 8-fold symmetry
        with pytest.raises(A.CigpuError) as e:
            srv.submit(bad, method=A.FCI)
        assert e.value.status == A.EINVAL
        with pytest.raises(A.CigpuError) as e:
            srv.submit(small, method=A.DOCI, tol=0.0)
        assert e.value.status == A.EINVAL
        ok = srv.submit(small, method=A.FCI, precision=A.MIXED, tol=1e-7, want_rdm=True)
        r = srv.wait(ok)
        assert r["status"] == A.OK
        assert np.trace(r["rdm1"][0]) == pytest.approx(3.0, abs=1e-9)
        assert np.trace(r["rdm1"][1]) == pytest.approx(3.0, abs=1e-9)
    with Server(hbm_budget_bytes=1 << 20, max_inflight=1) as srv:
        with pytest.raises(A.CigpuError) as e:  # can never fit a 1 MiB budget
            srv.submit(big, method=A.FCI, precision=A.FP64)
        assert e.value.status == A.ENOMEM


def test_destroy_with_requests_in_flight():
    base = make_integrals(10, 5, 5, nchol=16, seed=4)
    srv = Server(max_inflight=2)
    for i in range(6):
        srv.submit(rotate_integrals(base, 0.05, seed=i), method=A.FCI, precision=A.MIXED, tol=1e-6)
    srv.close()  # cancels the queue, lets running requests stop, joins the workers
    assert srv.h is None
