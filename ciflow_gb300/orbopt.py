"""Orbital optimisers over the cigpu C ABI, with CIFlow's class names.

* ``OrbitalOptimization(cim)`` (SimulatedAnnealing.cpp:42-191): ``get_opt_ci_energy``,
  ``get_opt_unitary``, ``set_cim_optimal``, ``get_cim_no``, ``get_fci_no``,
  ``transform_orbitals``, ``update_cim``.
* ``SimulatedAnnealing(cim, temp, change_temp, angle, change_angle)``
  (SimulatedAnnealing.cpp:195-391): ``optimize``, ``set_good_start``, ``run_multiple``.
* ``LocalMinimizer(cim)`` (LocalMinimizer.cpp:23-280), DOCI only: ``optimize``,
  ``scan_orbitals``, ``set_conv_crit``, ``set_conv_steps``, ``get_conv_crit``.

The loops run inside the library (``cigpu_orbopt_*``): every rotation, build,
eigensolve and DOCI pair scan stays on the device, and each solve starts from the
current eigenvector. ``update_cim`` hands the optimiser's current Hamiltonian to
the CIMethod and solves it there; ``optimize``/``set_cim_optimal`` call it when
they end, so the CIMethod is left solved in the current orbitals as in the
reference. Random draws come from seeded splitmix64 streams (the reference seeds
std::mt19937 from std::random_device); ``speculate`` > 1 solves that many
annealing proposals concurrently without changing the chain.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _abi as A
from .ciflow import CIMethod, Hamiltonian, _Handle


class OrbitalOptimization:
    """Owns a cigpu_orbopt: a device copy of the CIMethod's Hamiltonian, the current
    orbitals (unitary U, rows = orbitals in the starting basis) with their ground
    state, and the lowest energy seen with its unitary."""

    def __init__(self, cim: CIMethod, tol: float = 1e-8, warm_start: bool = True, seed: int = 0):
        self._cim = cim
        ham = cim.get_ham()
        self._L = ham.getL()
        self._nup, self._ndown, self._econst = ham.getnup(), ham.getndown(), ham.getEconst()
        cfg = A.OrboptConfig(cim.method, cim.precision, tol, 1 if warm_start else 0, 0, seed)
        out = ctypes.c_void_p()
        A.check(A.lib().cigpu_orbopt_create(ham.device(), ctypes.byref(cfg), ctypes.byref(out)),
                "cigpu_orbopt_create")
        self._h = _Handle(out.value, A.lib().cigpu_orbopt_destroy)

    @property
    def handle(self) -> int:
        return self._h.value

    # --- state ---
    def stats(self) -> dict:
        st = A.OrboptStats()
        A.check(A.lib().cigpu_orbopt_get(self.handle, None, None, None, ctypes.byref(st)), "cigpu_orbopt_get")
        return st.as_dict()

    def get_opt_ci_energy(self) -> float:
        return self.stats()["e_opt"]

    def get_ci_energy(self) -> float:
        return self.stats()["e_current"]

    def get_unitary(self) -> np.ndarray:
        U = np.zeros((self._L, self._L))
        A.check(A.lib().cigpu_orbopt_get(self.handle, A.ptr(U), None, None, None), "cigpu_orbopt_get")
        return U

    def get_opt_unitary(self) -> np.ndarray:
        U = np.zeros((self._L, self._L))
        A.check(A.lib().cigpu_orbopt_get(self.handle, None, A.ptr(U), None, None), "cigpu_orbopt_get")
        return U

    def get_eigvec(self) -> np.ndarray:
        n = self._cim.get_dim()
        c = np.zeros(n)
        A.check(A.lib().cigpu_orbopt_get(self.handle, None, None, A.ptr(c), None), "cigpu_orbopt_get")
        return c

    def get_ham(self) -> Hamiltonian:
        """The current orbitals' Hamiltonian (a new device handle with host copies)."""
        out = ctypes.c_void_p()
        A.check(A.lib().cigpu_orbopt_ham(self.handle, ctypes.byref(out)), "cigpu_orbopt_ham")
        H = Hamiltonian(self._L, 0, self._nup, self._ndown, self._econst)
        H._dev = _Handle(out.value, A.lib().cigpu_ham_destroy)
        A.check(A.lib().cigpu_ham_export(H._dev.value, A.ptr(H.h), A.ptr(H.eri)), "cigpu_ham_export")
        return H

    # --- reference operations ---
    def update_cim(self) -> None:
        """CIMethod::set_ham + solve with the current orbitals (update_cim, :83-87)."""
        self._cim.set_ham(self.get_ham())
        self._cim.solve(c0=self.get_eigvec())

    def transform_orbitals(self, i: int, j: int, angle: float) -> float:
        """transform_orbitals + solve (:89-100): returns the new energy."""
        e = ctypes.c_double()
        A.check(A.lib().cigpu_orbopt_jacobi(self.handle, i, j, angle, ctypes.byref(e)), "cigpu_orbopt_jacobi")
        return e.value

    def set_cim_optimal(self) -> None:
        A.check(A.lib().cigpu_orbopt_set_optimal(self.handle), "cigpu_orbopt_set_optimal")
        self.update_cim()

    def _natural(self, method: int) -> float:
        e = ctypes.c_double()
        A.check(A.lib().cigpu_orbopt_natural(self.handle, method, ctypes.byref(e)), "cigpu_orbopt_natural")
        return e.value

    def get_cim_no(self) -> float:
        """Natural orbitals of this CIMethod's ground state (:139-144)."""
        return self._natural(self._cim.method)

    def get_fci_no(self) -> float:
        """Natural orbitals of the FCI ground state in the current orbitals (:146-156)."""
        return self._natural(A.FCI)


class SimulatedAnnealing(OrbitalOptimization):
    def __init__(self, cim: CIMethod, temp: float, change_temp: float, angle: float, change_angle: float,
                 steps: int = 20000, speculate: int = 1, **kw):
        super().__init__(cim, **kw)
        self._temp, self._change_temp = temp, change_temp
        self._max_angle, self._change_angle = angle, change_angle
        self._c_steps = steps
        self.speculate = speculate
        self.max_unaccept = 2000
        self.min_angle = 1e-7

    def optimize(self, update: bool = True) -> float:
        """SimulatedAnnealing::optimize: the energy of the final current orbitals."""
        p = A.AnnealParams(self._temp, self._change_temp, self._max_angle, self._change_angle, self._c_steps,
                           self.max_unaccept, self.min_angle, self.speculate, 0)
        e = ctypes.c_double()
        A.check(A.lib().cigpu_orbopt_anneal(self.handle, ctypes.byref(p), ctypes.byref(e)), "cigpu_orbopt_anneal")
        if update:
            self.update_cim()
        return e.value

    def set_good_start(self) -> None:
        """FCI natural orbitals (this method's if FCI is not possible), a cold short
        anneal, then the best orbitals (SimulatedAnnealing.cpp:206-232)."""
        try:
            self.get_fci_no()
        except A.CigpuError:
            self.get_cim_no()
        saved = (self._temp, self._max_angle, self._change_temp, self._change_angle)
        self._temp, self._max_angle, self._change_temp, self._change_angle = 0.01, 0.1, 0.9, 0.99
        self.optimize(update=False)
        self._temp, self._max_angle, self._change_temp, self._change_angle = saved
        self.set_cim_optimal()

    def run_multiple(self, num: int) -> float:
        """set_good_start, then num annealing runs each restarted from the best
        orbitals, the last one cold (SimulatedAnnealing.cpp:234-272)."""
        self.set_good_start()
        for i in range(num):
            self.optimize(update=False)
            A.check(A.lib().cigpu_orbopt_set_optimal(self.handle), "cigpu_orbopt_set_optimal")
            if i == num - 2:
                self._temp, self._max_angle, self._change_temp, self._change_angle = 0.01, 0.1, 0.9, 0.99
        self.set_cim_optimal()
        return self.get_opt_ci_energy()


class LocalMinimizer(OrbitalOptimization):
    def __init__(self, cim: CIMethod, **kw):
        if cim.method != A.DOCI:
            raise ValueError("the local minimiser works for DOCI only, as in the reference")
        super().__init__(cim, **kw)
        self._conv_crit = 1e-6
        self._conv_steps = 25
        self.max_iters = 1000

    def get_conv_crit(self) -> float: return self._conv_crit
    def set_conv_crit(self, crit: float) -> None: self._conv_crit = crit
    def set_conv_steps(self, steps: int) -> None: self._conv_steps = steps

    def scan_orbitals(self):
        """[(k, l, theta, energy)] of the pairs scan_orbitals keeps (LocalMinimizer.cpp:73-128);
        energy without Econst, as calc_rotate returns it."""
        L = self._L
        np_ = L * (L - 1) // 2
        th, en = np.zeros(np_), np.zeros(np_)
        fd = np.zeros(np_, np.int32)
        cim = self._cim
        if cim.get_mat() is None or not cim.is_solved():
            self.update_cim()
        c = np.ascontiguousarray(cim.get_eigvec())
        A.check(A.lib().cigpu_doci_pair_scan(cim.get_mat().handle, A.ptr(c), A.ptr(th), A.ptr(en), A.ptr(fd)),
                "cigpu_doci_pair_scan")
        out, p = [], 0
        for k in range(L):
            for l in range(k + 1, L):
                if fd[p]:
                    out.append((k, l, float(th[p]), float(en[p])))
                p += 1
        return out

    def optimize(self, dist_choice: bool = False, update: bool = True) -> float:
        p = A.LocalParams(self._conv_crit, self._conv_steps, self.max_iters, 1 if dist_choice else 0, 0)
        e = ctypes.c_double()
        A.check(A.lib().cigpu_orbopt_local(self.handle, ctypes.byref(p), ctypes.byref(e)), "cigpu_orbopt_local")
        if update:
            self.update_cim()
        return e.value
