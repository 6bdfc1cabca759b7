"""Orbital optimisers restated for the oracle (test infrastructure, not product code).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
import this module. It restates, in numpy on the host:

* OrbitalTransform::do_jacobi_rotation (OrbitalTransform.cpp:278-414): the one-body
  formulas and one pass per index of the two-electron tensor, each pass mixing the
  k and l slices; UnitaryMatrix::jacobi_rotation (UnitaryMatrix.cpp:186-207) for
  the accumulated unitary;
* DensDOCI::find_min_angle and calc_rotate (CIDens.cpp:1279-1464), and the pair
  selection of LocalMinimizer::scan_orbitals (LocalMinimizer.cpp:73-128);
* SimulatedAnnealing::optimize with accept_function (SimulatedAnnealing.cpp:274-391),
  LocalMinimizer::optimize with choose_orbitalpair (LocalMinimizer.cpp:130-280),
  OrbitalOptimization::transform_to_no / set_cim_optimal
  (SimulatedAnnealing.cpp:69-74, 120-156), drawing from the same splitmix64
  streams as the library so that a chain can be compared step by step.

Every solve is the oracle's CRS (the C restatement of the reference build) with a
dense eigensolve: the cases here have a few thousand determinants at most.
"""
from __future__ import annotations

import math
import os
import sys
from dataclasses import dataclass

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import oracle as O  # noqa: E402

M64 = (1 << 64) - 1


class SplitMix64:
    """splitmix64 (Steele, Lea and Flood, OOPSLA 2014); uniform() has 53 random bits."""

    def __init__(self, seed: int):
        self.s = seed & M64

    def next(self) -> int:
        self.s = (self.s + 0x9E3779B97F4A7C15) & M64
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
        return z ^ (z >> 31)

    def uniform(self) -> float:
        return (self.next() >> 11) * 2.0 ** -53

    def below(self, n: int) -> int:
        return int(self.uniform() * n)


def stream_seed(seed: int, tag: int) -> int:
    return SplitMix64(seed ^ ((0xD1B54A32D192ED03 * (tag + 1)) & M64)).next()


# ---------------------------------------------------------------- rotations

def jacobi(h: np.ndarray, eri: np.ndarray, k: int, l: int, theta: float):
    """do_jacobi_rotation: k' = cos k - sin l, l' = sin k + cos l (new arrays)."""
    c, s = math.cos(theta), math.sin(theta)
    h = h.copy()
    tkk, tll, tkl = h[k, k], h[l, l], h[k, l]
    for a in range(h.shape[0]):
        if a in (k, l):
            continue
        tk, tl = h[k, a], h[l, a]
        h[a, k] = h[k, a] = c * tk - s * tl
        h[a, l] = h[l, a] = c * tl + s * tk
    h[k, k] = c * c * tkk + s * s * tll - 2 * c * s * tkl
    h[l, l] = c * c * tll + s * s * tkk + 2 * c * s * tkl
    h[k, l] = h[l, k] = tkl * (c * c - s * s) + c * s * (tkk - tll)
    v = eri.copy()
    for ax in range(4):
        vk = np.take(v, k, axis=ax).copy()
        vl = np.take(v, l, axis=ax).copy()
        sl = [slice(None)] * 4
        sl[ax] = k
        v[tuple(sl)] = c * vk - s * vl
        sl[ax] = l
        v[tuple(sl)] = c * vl + s * vk
    return h, v


def jacobi_unitary(U: np.ndarray, k: int, l: int, theta: float) -> np.ndarray:
    c, s = math.cos(theta), math.sin(theta)
    U = U.copy()
    uk, ul = U[k].copy(), U[l].copy()
    U[k] = c * uk - s * ul
    U[l] = c * ul + s * uk
    return U


def rotate(h: np.ndarray, eri: np.ndarray, U: np.ndarray):
    """h' = U h U^T, (ab|cd)' = sum U_ap U_bq U_cr U_ds (pq|rs) (fillHamCI)."""
    h2 = U @ h @ U.T
    e2 = np.einsum("ap,bq,cr,ds,pqrs->abcd", U, U, U, U, eri, optimize=True)
    return h2, e2


# ---------------------------------------------------------------- DOCI pair scan

def doci_pair_matrices(L: int, n: int, c: np.ndarray):
    """P[a,b] = get_two_rdm(1,a,a,b,b), D[a,b] = get_two_rdm(0,a,b,a,b) of a DOCI state."""
    r1, aa, ab, bb = O.rdm(O.DOCI, L, n, n, c)
    P = np.zeros((L, L))
    D = np.zeros((L, L))
    for a in range(L):
        for b in range(L):
            P[a, b] = O.two_rdm_get(L, aa, ab, bb, 1, a, a, b, b)
            D[a, b] = O.two_rdm_get(L, aa, ab, bb, 0, a, b, a, b)
    return P, D


@dataclass
class PairTerms:
    rest: float
    cos4: float
    sin4: float
    cos2: float
    sin2: float
    sincos: float
    cos2sin2: float
    sin3cos: float
    cos3sin: float


def pair_terms(h, eri, P, D, N: int, k: int, l: int) -> PairTerms:
    """The coefficients of calc_rotate (CIDens.cpp:1389-1464) for the pair k, l."""
    L = h.shape[0]
    T = lambda a, b: h[a, b]  # noqa: E731
    V = lambda a, b, c, d: eri[a, c, b, d]  # noqa: E731  <ab|cd> = (ac|bd)
    f = 2.0 / (N - 1.0)
    energy = 2 * f * (T(k, k) + T(l, l)) * D[k, l]
    cos2 = f * (T(k, k) * P[k, k] + T(l, l) * P[l, l])
    sin2 = f * (T(l, l) * P[k, k] + T(k, k) * P[l, l])
    sincos = f * T(k, l) * (P[l, l] - P[k, k])
    for a in range(L):
        if a in (k, l):
            continue
        energy += f * T(a, a) * (P[a, a] + 2 * D[a, k] + 2 * D[a, l])
        for b in range(L):
            if b in (k, l):
                continue
            energy += f * (T(a, a) + T(b, b)) * D[a, b]
            energy += V(a, a, b, b) * P[a, b]
            energy += (2 * V(a, b, a, b) - V(a, b, b, a)) * D[a, b]
        xk = 2 * V(k, a, k, a) - V(k, a, a, k) + f * T(k, k)
        xl = 2 * V(l, a, l, a) - V(l, a, a, l) + f * T(l, l)
        cos2 += 2 * V(k, k, a, a) * P[k, a] + 2 * V(l, l, a, a) * P[l, a] + 2 * xk * D[k, a] + 2 * xl * D[l, a]
        sin2 += 2 * V(l, l, a, a) * P[k, a] + 2 * V(k, k, a, a) * P[l, a] + 2 * xk * D[l, a] + 2 * xl * D[k, a]
        sincos += 2 * V(k, l, a, a) * (P[l, a] - P[k, a]) + \
            2 * (2 * V(k, a, l, a) - V(k, a, a, l) + f * T(k, l)) * (D[l, a] - D[k, a])
    cos4 = V(k, k, k, k) * P[k, k] + V(l, l, l, l) * P[l, l] + 2 * V(k, k, l, l) * P[k, l] + \
        2 * (2 * V(k, l, k, l) - V(k, k, l, l)) * D[k, l]
    sin4 = V(k, k, k, k) * P[l, l] + V(l, l, l, l) * P[k, k] + 2 * V(k, k, l, l) * P[k, l] + \
        2 * (2 * V(k, l, k, l) - V(k, k, l, l)) * D[k, l]
    cos2sin2 = (2 * V(k, k, l, l) + V(k, l, k, l)) * (P[k, k] + P[l, l]) + \
        (V(k, k, k, k) + V(l, l, l, l) - 2 * (V(k, l, k, l) + V(k, k, l, l))) * P[k, l] + \
        (V(k, k, k, k) + V(l, l, l, l) - 6 * V(k, k, l, l) + 2 * V(k, l, k, l)) * D[k, l]
    sin3cos = V(k, l, k, k) * P[l, l] - V(k, l, l, l) * P[k, k] - \
        (V(k, l, k, k) - V(k, l, l, l)) * (P[k, l] + D[k, l])
    cos3sin = V(k, l, l, l) * P[l, l] - V(k, l, k, k) * P[k, k] + \
        (V(k, l, k, k) - V(k, l, l, l)) * (P[k, l] + D[k, l])
    return PairTerms(energy, cos4, sin4, cos2, sin2, sincos, cos2sin2, sin3cos, cos3sin)


def calc_rotate(t: PairTerms, theta: float) -> float:
    c, s = math.cos(theta), math.sin(theta)
    return (t.rest + c ** 4 * t.cos4 + s ** 4 * t.sin4 + c * c * t.cos2 + s * s * t.sin2 + 2 * s * c * t.sincos
            + 2 * c * c * s * s * t.cos2sin2 + 4 * c * s ** 3 * t.sin3cos + 4 * c ** 3 * s * t.cos3sin)


def _gradient(t: PairTerms, th: float) -> float:
    c, s = math.cos(th), math.sin(th)
    return (16 * (t.cos3sin - t.sin3cos) * c ** 4 - 4 * (t.cos4 + t.sin4 - 2 * t.cos2sin2) * s * c ** 3
            + 4 * (t.sincos - 3 * t.cos3sin + 5 * t.sin3cos) * c * c
            + 2 * (2 * t.sin4 - t.cos2 + t.sin2 - 2 * t.cos2sin2) * s * c - 2 * t.sincos - 4 * t.sin3cos)


def _hessian(t: PairTerms, th: float) -> float:
    c, s = math.cos(th), math.sin(th)
    return (-16 * (t.cos4 + t.sin4 - 2 * t.cos2sin2) * c ** 4 + 64 * (t.sin3cos - t.cos3sin) * s * c ** 3
            + 4 * (3 * t.cos4 + 5 * t.sin4 - t.cos2 + t.sin2 - 8 * t.cos2sin2) * c * c
            - 8 * (t.sincos - 3 * t.cos3sin + 5 * t.sin3cos) * s * c + 2 * (t.cos2 - 2 * t.sin4 - t.sin2 + 2 * t.cos2sin2))


def find_min_angle(t: PairTerms, start: float):
    """Newton-Raphson of find_min_angle: (theta, is_minimum)."""
    th = start
    if _gradient(t, th) * th + _hessian(t, th) * th * th / 2.0 > 0:
        th = -th
    for _ in range(20):
        dx = _gradient(t, th) / _hessian(t, th)
        th -= dx
        if abs(dx) < 1e-12:
            break
    return th, _hessian(t, th) > 0


def scan(h, eri, P, D, N: int):
    """(theta, energy, found) for every pair k < l, as scan_orbitals decides them."""
    L = h.shape[0]
    th, en, fd = [], [], []
    for k in range(L):
        for l in range(k + 1, L):
            t = pair_terms(h, eri, P, D, N, k, l)
            a, ok = find_min_angle(t, 0.3)
            if not ok:
                a, ok = find_min_angle(t, 0.01)
            th.append(a)
            en.append(calc_rotate(t, a))
            fd.append(1 if ok and abs(a) <= math.pi / 2 else 0)
    return np.array(th), np.array(en), np.array(fd, np.int32)


# ---------------------------------------------------------------- solves

class _Ints:
    def __init__(self, L, nup, ndown, econst, h, eri):
        self.L, self.nup, self.ndown, self.econst, self.h, self.eri = L, nup, ndown, econst, h, eri


def solve(method: int, L: int, nup: int, ndown: int, econst: float, h, eri):
    """(E0 with Econst, c) from the oracle CRS: a dense eigensolve up to 2000
    determinants, above that ARPACK with the reference's settings."""
    m = O.build_upper(method, _Ints(L, nup, ndown, econst, h, eri))
    if m.n > 2000:
        e, c = O.lowest_eigenpair(m)
        return e + econst, c
    w, v = np.linalg.eigh(m.full_csr().toarray())
    return float(w[0]) + econst, v[:, 0]


@dataclass
class AnnealParams:
    temp: float = 0.4
    change_temp: float = 0.99
    max_angle: float = 1.4
    change_angle: float = 0.999
    steps: int = 20000
    max_unaccept: int = 2000
    min_angle: float = 1e-7


@dataclass
class LocalParams:
    conv_crit: float = 1e-6
    conv_steps: int = 25
    max_iters: int = 1000
    dist_choice: bool = False


class Optimizer:
    """cigpu_orbopt restated: the starting integrals, the current orbitals (U) with
    their integrals and ground state, and the lowest energy seen with its U."""

    def __init__(self, ints, method: int, seed: int):
        self.method = method
        self.L, self.nup, self.ndown, self.econst = ints.L, ints.nup, ints.ndown, ints.econst
        self.h0 = np.array(ints.h, dtype=np.float64)
        self.eri0 = np.array(ints.eri, dtype=np.float64)
        self.h, self.eri = self.h0.copy(), self.eri0.copy()
        self.U = np.eye(self.L)
        self.e, self.c = self._solve(self.h, self.eri)
        self.e_opt = self.e
        self.U_opt = self.U.copy()
        self.seed = seed
        self.calls = 0
        self.acc = SplitMix64(stream_seed(seed, 0))
        self.solves = 1

    def _solve(self, h, eri):
        return solve(self.method, self.L, self.nup, self.ndown, self.econst, h, eri)

    def jacobi(self, k: int, l: int, theta: float) -> float:
        self.h, self.eri = jacobi(self.h, self.eri, k, l, theta)
        self.U = jacobi_unitary(self.U, k, l, theta)
        self.e, self.c = self._solve(self.h, self.eri)
        self.solves += 1
        return self.e

    def anneal(self, p: AnnealParams):
        """SimulatedAnnealing::optimize; returns (e_last, accepted, rejected)."""
        prop = SplitMix64(stream_seed(self.seed, 2 * self.calls + 1))
        self.calls += 1
        temp, max_angle = p.temp, p.max_angle
        e_old = self.e
        unaccept = accepted = rejected = 0
        for _ in range(p.steps):
            i, j = prop.below(self.L), prop.below(self.L)
            if i == j:
                continue
            u1, u2 = prop.uniform(), prop.uniform()
            angle = max_angle * (u1 - u2)
            h2, e2 = jacobi(self.h, self.eri, i, j, angle)
            e_new, c_new = self._solve(h2, e2)
            self.solves += 1
            if e_new < e_old:
                accept = True
            else:
                cost = math.exp((e_old - e_new) / temp)
                accept = not (self.acc.uniform() * (1 + cost) > cost)
            if accept:
                accepted += 1
                e_old = e_new
                self.h, self.eri, self.e, self.c = h2, e2, e_new, c_new
                self.U = jacobi_unitary(self.U, i, j, angle)
                if e_new < self.e_opt:
                    self.e_opt = e_new
                    self.U_opt = self.U.copy()
                unaccept = 0
            else:
                rejected += 1
                unaccept += 1
            temp *= p.change_temp
            max_angle *= p.change_angle
            if unaccept > p.max_unaccept or max_angle < p.min_angle:
                break
        return e_old, accepted, rejected

    def local(self, p: LocalParams):
        """LocalMinimizer::optimize (DOCI); returns (e_final, iterations)."""
        L, N = self.L, self.nup + self.ndown
        converged, iters, opt_energy, prev = 0, 1, 0.0, (0, 0)

        def choose(rots):
            u = self.acc.uniform()
            norm = sum(opt_energy - r[3] for r in rots)
            cum = 0.0
            for i, r in enumerate(rots):
                cum += (opt_energy - r[3]) / norm
                if u < cum:
                    return i
            return len(rots) - 1

        while converged < p.conv_steps:
            P, D = doci_pair_matrices(L, self.nup, self.c)
            th, en, fd = scan(self.h, self.eri, P, D, N)
            rots, pi = [], 0
            for k in range(L):
                for l in range(k + 1, L):
                    if fd[pi]:
                        rots.append((k, l, th[pi], en[pi]))
                    pi += 1
            if not rots:
                raise RuntimeError("no pair to rotate")
            rots.sort(key=lambda r: r[3])  # stable
            idx = 0
            if p.dist_choice:
                idx = choose(rots)
                if rots[idx][:2] == prev:
                    idx = choose(rots)
                if rots[idx][:2] == prev:
                    idx = 0
            if rots[idx][:2] == prev and idx + 1 < len(rots):
                idx += 1
            k, l, a, _ = rots[idx]
            prev = (k, l)
            E = self.jacobi(k, l, a)
            if abs(opt_energy - E) < p.conv_crit:
                converged += 1
            opt_energy = E
            iters += 1
            if iters > p.max_iters:
                break
        self.e_opt = opt_energy
        self.U_opt = self.U.copy()
        return self.e, iters - 1

    def natural(self, density_method: int) -> float:
        """transform_to_no with the density of `density_method` in the current orbitals."""
        L = self.L
        if density_method == self.method:
            c = self.c
        else:
            _, c = solve(density_method, L, self.nup, self.ndown, self.econst, self.h, self.eri)
        r1, _, _, _ = O.rdm(density_method, L, self.nup, self.ndown, c)
        w, z = np.linalg.eigh(r1[0] + r1[1])
        NO = z[:, ::-1]  # descending occupations
        self.U = NO.T @ self.U
        self.h, self.eri = rotate(self.h0, self.eri0, self.U)
        self.e, self.c = self._solve(self.h, self.eri)
        return self.e

    def set_optimal(self) -> None:
        self.U = self.U_opt.copy()
        self.h, self.eri = rotate(self.h0, self.eri0, self.U)
        self.e, self.c = self._solve(self.h, self.eri)
