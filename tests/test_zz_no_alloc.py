"""The allocation-free DOCI RDM entry point, cigpu_rdm_doci_noalloc.

Callers that cannot allocate device memory on their request path -- a host
framework that hands out all device memory from its own fixed pool, or a
latency-bound loop that cannot afford the device synchronisation cudaMalloc
implies -- use this variant of the DOCI RDM: its block partial sums live in a
fixed array inside the library. These tests call it through the C ABI with
device buffers, twice in a row, and compare each result with the allocating
entry point cigpu_rdm on the same vector (the two differ only in how the block
partial sums are grouped, so they agree to FP64 round-off: tolerance 1e-13).
This file is collected last so that a failure here stops a -x run only after
every other test has run; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from ciflow_gb300 import _abi as A
from ciflow_gb300.ciflow import DOCI, FCI, Hamiltonian
from ciflow_gb300.synthetic import make_integrals

pytestmark = pytest.mark.gpu

TOL = 1e-13


def host_rdm(handle, L, c):
    np_ = L * (L - 1) // 2
    out = (np.empty((2, L, L)), np.empty((np_, np_)), np.empty((L * L, L * L)), np.empty((np_, np_)))
    A.check(A.lib().cigpu_rdm(handle, A.ptr(np.ascontiguousarray(c)), *(A.ptr(o) for o in out)))
    return out


def test_noalloc_matches_allocating_entry_point_twice():
    torch = pytest.importorskip("torch")
    L, n = 10, 5
    ints = make_integrals(L, n, n, nchol=8, seed=31)
    cim = DOCI(Hamiltonian.from_integrals(ints))
    cim.solve(tol=1e-9)
    handle = cim.get_mat().handle
    np_ = L * (L - 1) // 2
    c0 = cim.get_eigvec()
    rng = np.random.default_rng(7)
    c1 = c0 + 0.05 * rng.standard_normal(c0.size)
    c1 /= np.linalg.norm(c1)
    stream = torch.cuda.current_stream().cuda_stream
    outs = [torch.full(shape, float("nan"), dtype=torch.float64, device="cuda")
            for shape in ((2, L, L), (np_, np_), (L * L, L * L), (np_, np_))]
    for c in (c0, c1):  # two calls in a row; the second must not see the first's contents
        ref = host_rdm(handle, L, c)
        cd = torch.tensor(c, dtype=torch.float64, device="cuda")
        for o in outs:
            o.fill_(float("nan"))
        st = A.lib().cigpu_rdm_doci_noalloc(handle, cd.data_ptr(), outs[0].data_ptr(), outs[1].data_ptr(),
                                           outs[2].data_ptr(), outs[3].data_ptr(), ctypes.c_void_p(stream))
        assert st == A.OK, A.lib().cigpu_strerror(st)
        torch.cuda.synchronize()
        for got, want, name in zip(outs, ref, ("rdm1", "aa", "ab", "bb")):
            g = got.cpu().numpy()
            assert np.all(np.isfinite(g)), name
            assert np.abs(g - want).max() <= TOL, (name, np.abs(g - want).max())


def test_noalloc_rejects_what_it_cannot_do():
    torch = pytest.importorskip("torch")
    fci = FCI(Hamiltonian.from_integrals(make_integrals(6, 3, 3, nchol=4, seed=1)))
    buf = torch.zeros(1 << 16, dtype=torch.float64, device="cuda")
    p = buf.data_ptr()
    assert A.lib().cigpu_rdm_doci_noalloc(fci.get_mat().handle, p, p, p, p, p, None) == A.EINVAL
    assert A.lib().cigpu_rdm_doci_noalloc(None, p, p, p, p, p, None) == A.EINVAL
    # L = 34 needs more partial sums per block than the fixed array is laid out for
    big = DOCI(Hamiltonian.from_integrals(make_integrals(34, 2, 2, nchol=2, seed=2)))
    assert A.lib().cigpu_rdm_doci_noalloc(big.get_mat().handle, p, p, p, p, p, None) == A.ENOTSUP
