"""Seeded synthetic one- and two-electron integrals for the CI benchmarks.

The generator follows the workload specification of the lowest-eigenpair CI
benchmarks (no public dataset is involved):

1. h: the strict upper triangle is drawn row-major from N(0, sigma=0.05) and
   mirrored; the diagonal is h_pp = -2.0 + 0.25 p.
2. For k < K, an L x L symmetric factor L^k: upper triangle (diagonal included)
   drawn row-major from N(0, sigma=0.1) and mirrored, plus 0.3 on the diagonal.
3. (pq|rs) = sum_k L^k_pq L^k_rs (chemist notation), which is 8-fold symmetric
   and positive semidefinite as a pair matrix.

The ERI sum is accumulated with elementwise numpy operations in a fixed k
order (no BLAS), so the tensor is bit-identical on every platform and exactly
8-fold symmetric: a_i * a_j == a_j * a_i in IEEE arithmetic and each L^k is
mirrored exactly.
"""
from __future__ import annotations

import dataclasses

import numpy as np


@dataclasses.dataclass
class Integrals:
    L: int
    nup: int
    ndown: int
    econst: float
    h: np.ndarray      # (L, L) float64, symmetric
    eri: np.ndarray    # (L, L, L, L) float64, chemist (pq|rs), 8-fold symmetric

    def checksum(self) -> str:
        import hashlib
        m = hashlib.sha256()
        m.update(np.ascontiguousarray(self.h).tobytes())
        m.update(np.ascontiguousarray(self.eri).tobytes())
        return m.hexdigest()[:16]


def _sym_from_upper(rng: np.random.Generator, L: int, sigma: float, include_diag: bool) -> np.ndarray:
    iu = np.triu_indices(L, 0 if include_diag else 1)
    vals = rng.normal(0.0, sigma, size=len(iu[0]))
    m = np.zeros((L, L))
    m[iu] = vals
    m = m + np.triu(m, 1).T
    return m


def make_integrals(L: int, nup: int, ndown: int, nchol: int = 16, seed: int = 0) -> Integrals:
    """Integrals for one problem; ``nchol`` is K, the number of symmetric factors."""
    rng = np.random.default_rng(seed)
    h = _sym_from_upper(rng, L, 0.05, include_diag=False)
    h[np.diag_indices(L)] = -2.0 + 0.25 * np.arange(L)
    eri = np.zeros((L * L, L * L))
    for _ in range(nchol):
        lk = _sym_from_upper(rng, L, 0.1, include_diag=True)
        lk[np.diag_indices(L)] += 0.3
        v = lk.reshape(-1)
        eri += np.multiply.outer(v, v)
    return Integrals(L, nup, ndown, 0.0, h, eri.reshape(L, L, L, L))


def symmetrize_eri(eri: np.ndarray) -> np.ndarray:
    """Exact 8-fold symmetrization: every index permutation takes the value stored
    at its canonical representative (p>=q, r>=s, pq>=rs)."""
    L = eri.shape[0]
    p, q, r, s = np.indices((L, L, L, L))
    a = np.maximum(p, q); b = np.minimum(p, q)
    c = np.maximum(r, s); d = np.minimum(r, s)
    swap = (a * L + b) < (c * L + d)
    a2 = np.where(swap, c, a); b2 = np.where(swap, d, b)
    c2 = np.where(swap, a, c); d2 = np.where(swap, b, d)
    return eri[a2, b2, c2, d2]


def rotate_integrals(ints: Integrals, kappa_sigma: float = 0.05, seed: int = 0) -> Integrals:
    """Orbital rotation U = exp(kappa), kappa antisymmetric with N(0, kappa_sigma)
    entries; returns integrals in the rotated basis, re-symmetrized exactly."""
    import scipy.linalg

    L = ints.L
    rng = np.random.default_rng(seed)
    k = np.zeros((L, L))
    iu = np.triu_indices(L, 1)
    k[iu] = rng.normal(0.0, kappa_sigma, size=len(iu[0]))
    k = k - k.T
    u = scipy.linalg.expm(k)
    h = u.T @ ints.h @ u
    h = 0.5 * (h + h.T)
    eri = np.einsum("pqrs,pi,qj,rk,sl->ijkl", ints.eri, u, u, u, u, optimize=True)
    return Integrals(L, ints.nup, ints.ndown, ints.econst, h, symmetrize_eri(eri))


# Benchmark configurations (orbitals, electrons per spin, Cholesky-like factors, seed).
CONFIGS = {
    "c0": dict(method="FCI", L=8, nup=4, ndown=4, nchol=16, seed=0),
    "c1": dict(method="FCI", L=12, nup=6, ndown=6, nchol=16, seed=1),
    "c2": dict(method="DOCI", L=24, nup=12, ndown=12, nchol=24, seed=2),
    "c4": dict(method="FCI", L=10, nup=5, ndown=5, nchol=16, seed=4),
    # profiling size: same construction, CRS of a few GB (x larger than L1, CRS larger than L2)
    "p11": dict(method="FCI", L=11, nup=5, ndown=5, nchol=16, seed=11),
    # DOCI profiling size: 184,756 pair determinants, an FP64 CRS of ~224 MB (larger than L2)
    "p20": dict(method="DOCI", L=20, nup=10, ndown=10, nchol=24, seed=20),
}


def config_integrals(name: str) -> Integrals:
    c = CONFIGS[name]
    return make_integrals(c["L"], c["nup"], c["ndown"], c["nchol"], c["seed"])
