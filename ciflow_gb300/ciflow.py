"""Python mirror of CIFlow's lowest-eigenpair API over the cigpu C ABI.

Class and method names follow the reference so code written against CIFlow
reads the same:

* ``Hamiltonian``   -- Hamiltonian(L, nGroup=0, nup, ndown, Econst) with
  setTmat/setVmat/getTmat/getVmat (Hamiltonian.cpp:77-113, 255-320); V is in
  physics notation <ij|kl>, stored internally as chemist (ik|jl).
* ``FCI`` / ``DOCI`` -- the constructor builds the CRS (CIMethod.cpp:566-580),
  ``solve``, ``get_ci_energy``, ``get_eigvec``, ``set_ham``, ``construct_density``
  (CIMethod.h:37-162).
* ``SparseMatrix_CRS_Sym`` -- the upper-triangle CRS view with ``mvprod``,
  ``getn``/``getm``/``datasize`` and element access (SparseMatrix_CRS.h:33-130).
* ``FCI_File`` / ``CI_Big`` -- determinant lists (CIMethod.h:164-189): the CRS
  of a list, or no stored matrix and elements recomputed in every matvec;
  ``read_determinants`` reads a determinant file (Permutator.cpp:179-224).
* ``DensFCI`` / ``DensDOCI`` -- ``construct_density``, ``get_one_rdm``,
  ``get_two_rdm``, ``get_dens_energy`` (CIDens.h:29-174).

Differences from the reference, by design: errors raise ``CigpuError`` instead
of calling exit(1); ``solve`` keeps the CRS resident (the reference frees it
after solving, CIMethod.cpp:262) so later matvecs and re-solves reuse it.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _abi as A

NEIGVAL = 1  # Options.h:37


class Hamiltonian:
    """In-memory integral store (point group C1)."""

    def __init__(self, L: int, nGroup: int = 0, nup: int = 0, ndown: int = 0, Econst: float = 0.0,
                 h: np.ndarray | None = None, eri: np.ndarray | None = None):
        if nGroup != 0:
            raise ValueError("only point group 0 (C1) is supported, as in Hamiltonian.cpp:81-86")
        self.L = int(L)
        self.nup = int(nup)
        self.ndown = int(ndown)
        self.Econst = float(Econst)
        self.h = np.zeros((L, L)) if h is None else np.array(h, dtype=np.float64).reshape(L, L)
        self.eri = np.zeros((L,) * 4) if eri is None else np.array(eri, dtype=np.float64).reshape((L,) * 4)
        self._dev = None

    @classmethod
    def from_integrals(cls, ints) -> "Hamiltonian":
        return cls(ints.L, 0, ints.nup, ints.ndown, ints.econst, ints.h, ints.eri)

    # --- reference accessors ---
    def getL(self) -> int: return self.L
    def getnup(self) -> int: return self.nup
    def getndown(self) -> int: return self.ndown
    def getEconst(self) -> float: return self.Econst
    def setEconst(self, v: float) -> None: self.Econst = float(v); self._dev = None

    def getTmat(self, i: int, j: int) -> float:
        return float(self.h[i, j])

    def setTmat(self, i: int, j: int, val: float) -> None:
        self.h[i, j] = self.h[j, i] = val
        self._dev = None

    def getVmat(self, i: int, j: int, k: int, l: int) -> float:
        return float(self.eri[i, k, j, l])  # <ij|kl> = (ik|jl)

    def setVmat(self, i: int, j: int, k: int, l: int, val: float) -> None:
        """Sets <ij|kl> and its 8 symmetry partners."""
        p, q, r, s = i, k, j, l  # chemist (pq|rs)
        for a, b, c, d in ((p, q, r, s), (q, p, r, s), (p, q, s, r), (q, p, s, r),
                           (r, s, p, q), (s, r, p, q), (r, s, q, p), (s, r, q, p)):
            self.eri[a, b, c, d] = val
        self._dev = None

    def device(self):
        """The device copy (created on first use)."""
        if self._dev is None:
            out = ctypes.c_void_p()
            h = np.ascontiguousarray(self.h)
            e = np.ascontiguousarray(self.eri)
            A.check(A.lib().cigpu_ham_create(self.L, self.nup, self.ndown, self.Econst, A.ptr(h), A.ptr(e),
                                              ctypes.byref(out)), "cigpu_ham_create")
            self._dev = _Handle(out.value, A.lib().cigpu_ham_destroy)
        return self._dev.value


    def rotated(self, U: np.ndarray) -> "Hamiltonian":
        """The Hamiltonian in rotated orbitals, h' = U h U^T and (ab|cd)' = sum U_ap U_bq
        U_cr U_ds (pq|rs), computed on the device (cigpu_ham_rotate; the reference's
        OrbitalTransform::fillHamCI, OrbitalTransform.cpp:64-135)."""
        u = np.ascontiguousarray(U, dtype=np.float64)
        out = ctypes.c_void_p()
        A.check(A.lib().cigpu_ham_rotate(self.device(), A.ptr(u), None, ctypes.byref(out)), "cigpu_ham_rotate")
        H = Hamiltonian(self.L, 0, self.nup, self.ndown, self.Econst)
        H._dev = _Handle(out.value, A.lib().cigpu_ham_destroy)
        A.check(A.lib().cigpu_ham_export(H._dev.value, A.ptr(H.h), A.ptr(H.eri)), "cigpu_ham_export")
        return H

    @classmethod
    def read_file(cls, path: str) -> "Hamiltonian":
        """Hamiltonian(filename) for a psi4 integral text dump (Hamiltonian::read_file,
        Hamiltonian.cpp:707-885), parsed by the library; point-group labels are read
        and not used (C1)."""
        L, na, nb = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        ec, hf = ctypes.c_double(), ctypes.c_double()
        p = path.encode()
        A.check(A.lib().cigpu_ham_read_psi4(p, ctypes.byref(L), ctypes.byref(na), ctypes.byref(nb), ctypes.byref(ec),
                                            None, None, None, None), "cigpu_ham_read_psi4")
        n = L.value
        h, eri = np.zeros((n, n)), np.zeros((n,) * 4)
        A.check(A.lib().cigpu_ham_read_psi4(p, ctypes.byref(L), ctypes.byref(na), ctypes.byref(nb), ctypes.byref(ec),
                                            A.ptr(h), A.ptr(eri), None, ctypes.byref(hf)), "cigpu_ham_read_psi4")
        H = cls(n, 0, na.value, nb.value, ec.value, h, eri)
        H.hf_energy = hf.value
        return H

    def save_file(self, path: str, hf_energy: float = 0.0) -> None:
        """The psi4 integral text dump (Hamiltonian::save_file's format, C1, 17 digits)."""
        h = np.ascontiguousarray(self.h)
        e = np.ascontiguousarray(self.eri)
        A.check(A.lib().cigpu_ham_write_psi4(path.encode(), self.L, self.nup, self.ndown, self.Econst, A.ptr(h),
                                             A.ptr(e), hf_energy), "cigpu_ham_write_psi4")

    def jacobi(self, k: int, l: int, theta: float) -> "Hamiltonian":
        """The Hamiltonian with orbitals k, l rotated by theta (k' = cos k - sin l,
        l' = sin k + cos l), computed on the device (cigpu_ham_jacobi; the reference's
        OrbitalTransform::do_jacobi_rotation, OrbitalTransform.cpp:278-414)."""
        out = ctypes.c_void_p()
        A.check(A.lib().cigpu_ham_jacobi(self.device(), k, l, theta, None, ctypes.byref(out)), "cigpu_ham_jacobi")
        H = Hamiltonian(self.L, 0, self.nup, self.ndown, self.Econst)
        H._dev = _Handle(out.value, A.lib().cigpu_ham_destroy)
        A.check(A.lib().cigpu_ham_export(H._dev.value, A.ptr(H.h), A.ptr(H.eri)), "cigpu_ham_export")
        return H


def unitary_exp(X: np.ndarray) -> np.ndarray:
    """exp(X) of an antisymmetric generator (UnitaryMatrix.cpp:229-290), host code of the library."""
    x = np.ascontiguousarray(X, dtype=np.float64)
    u = np.empty_like(x)
    A.check(A.lib().cigpu_unitary_exp(x.shape[0], A.ptr(x), A.ptr(u)), "cigpu_unitary_exp")
    return u


class _Handle:
    def __init__(self, value, destroy):
        self.value = value
        self._destroy = destroy

    def __del__(self):
        try:
            if self.value:
                self._destroy(self.value)
        except Exception:
            pass
        self.value = None


class SparseMatrix_CRS_Sym:
    """The device CRS, viewed as CIFlow's upper-triangle SparseMatrix_CRS_Sym."""

    def __init__(self, handle, ham: Hamiltonian):
        self._h = handle
        self._ham = ham  # the device Hamiltonian must outlive the CRS
        dim = ctypes.c_int64()
        # the dimension only: the nonzero counts of a build whose last part runs
        # beside the first solve are read when first asked for (nnz_upper, nnz_full)
        A.check(A.lib().cigpu_crs_dims(handle.value, ctypes.byref(dim), None, None))
        self.n = dim.value
        self._counts = None
        self._upper = None

    def _nnz(self) -> tuple[int, int]:
        if self._counts is None:
            nu, nf = ctypes.c_int64(), ctypes.c_int64()
            A.check(A.lib().cigpu_crs_dims(self._h.value, None, ctypes.byref(nu), ctypes.byref(nf)))
            self._counts = (nu.value, nf.value)
        return self._counts

    @property
    def nnz_upper(self) -> int:
        return self._nnz()[0]

    @property
    def nnz_full(self) -> int:
        return self._nnz()[1]

    @property
    def handle(self):
        return self._h.value

    def getn(self) -> int: return self.n
    def getm(self) -> int: return self.n
    def datasize(self) -> int: return self.nnz_upper

    def upper(self):
        """(row uint32[n+1], col uint32[nnz], data float64[nnz]) in the reference layout."""
        if self._upper is None:
            row = np.empty(self.n + 1, np.uint32)
            col = np.empty(self.nnz_upper, np.uint32)
            val = np.empty(self.nnz_upper, np.float64)
            A.check(A.lib().cigpu_crs_export_upper(self.handle, A.ptr(row), A.ptr(col), A.ptr(val)),
                    "cigpu_crs_export_upper")
            self._upper = (row, col, val)
        return self._upper

    def full(self):
        """(row int64[n+1], col uint32[nnz], val float64[nnz]) of both triangles."""
        row = np.empty(self.n + 1, np.int64)
        col = np.empty(self.nnz_full, np.uint32)
        val = np.empty(self.nnz_full, np.float64)
        A.check(A.lib().cigpu_crs_export_full(self.handle, A.ptr(row), A.ptr(col), A.ptr(val)),
                "cigpu_crs_export_full")
        return row, col, val

    def __call__(self, i: int, j: int) -> float:
        if i > j:
            i, j = j, i
        row, col, val = self.upper()
        s, e = int(row[i]), int(row[i + 1])
        k = s + int(np.searchsorted(col[s:e], j))
        return float(val[k]) if k < e and col[k] == j else 0.0

    def mvprod(self, x: np.ndarray, y: np.ndarray | None = None) -> np.ndarray:
        """y = H x with host buffers (SparseMatrix_CRS_Sym::mvprod)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        if y is None:
            y = np.empty(self.n)
        A.check(A.lib().cigpu_mvprod(self.handle, A.ptr(x), A.ptr(y), None), "cigpu_mvprod")
        return y

    def mvprod_device(self, x, y, stream=None) -> None:
        """y = H x for device tensors (float64: FP64 product; float32: FP32 product)."""
        dtype = 1 if str(x.dtype).endswith("float32") else 0
        A.check(A.lib().cigpu_mvprod_device(self.handle, A.ptr(x), A.ptr(y), dtype, stream), "cigpu_mvprod_device")


class CIMethod:
    """Common part of FCI and DOCI (CIMethod.h:37-132)."""

    method = A.FCI
    name = "FCI"

    def __init__(self, ham: Hamiltonian, precision: int = A.FP64, build: bool = True):
        self._ham = ham
        self.precision = precision
        self._eigval = None
        self._eigvec = None
        self._solved = False
        self.info = None
        self._cid = None
        self._mat = None
        if build:
            self.build_ci()

    # --- construction ---
    def build_ci(self) -> None:
        out = ctypes.c_void_p()
        A.check(A.lib().cigpu_build(self._ham.device(), self.method, self.precision, None, ctypes.byref(out)),
                "cigpu_build")
        self._mat = SparseMatrix_CRS_Sym(_Handle(out.value, A.lib().cigpu_crs_destroy), self._ham)

    def set_ham(self, ham: Hamiltonian, build: bool = True) -> None:
        """CIMethod::set_ham (CIMethod.cpp:117-126)."""
        self._ham = ham
        self._mat = None
        self._solved = False
        self._cid = None
        if build:
            self.build_ci()

    def reset_mat(self) -> None:
        self._mat = None

    # --- accessors ---
    def get_ham(self) -> Hamiltonian: return self._ham
    def get_name(self) -> str: return self.name
    def get_l(self) -> int: return self._ham.L
    def gNup(self) -> int: return self._ham.nup
    def gNdown(self) -> int: return self._ham.ndown
    def get_econst(self) -> float: return self._ham.Econst
    def is_solved(self) -> bool: return self._solved

    def get_dim(self) -> int:
        return self._mat.n if self._mat is not None else self._dim()

    def get_mat(self, i: int | None = None, j: int | None = None):
        if i is None:
            return self._mat
        return self._mat(i, j)

    # --- eigensolver ---
    def solve(self, neigval: int = NEIGVAL, tol: float = 1e-8, max_matvec: int = 0,
              c0: np.ndarray | None = None) -> None:
        """Lowest eigenpair (CIMethod::solve, CIMethod.cpp:241-264); only neigval=1."""
        if neigval != 1:
            raise ValueError("the GPU solver computes the lowest eigenpair only (neigval=1)")
        if self._mat is None:
            self.build_ci()
        n = self._mat.n
        c = np.empty(n)
        info = A.SolveInfo()
        c0a = None if c0 is None else np.ascontiguousarray(c0, dtype=np.float64)
        st = A.lib().cigpu_solve(self._mat.handle, tol, max_matvec, A.ptr(c0a), A.ptr(c), ctypes.byref(info))
        if st not in (A.OK, A.ENOCONV):
            A.check(st, "cigpu_solve")
        self.info = info.as_dict()
        self.info["status"] = st
        self._eigval = np.array([info.e0 - self._ham.Econst])
        self._eigvec = c.reshape(n, 1)
        self._solved = True
        self._cid = None

    def get_ci_energy(self, neigval: int = 0) -> float:
        return float(self._eigval[neigval]) + self.get_econst()

    def get_eigvec(self, numstate: int | None = None, numvec: int = 0):
        if numstate is None:
            return self._eigvec[:, numvec].copy()
        return float(self._eigvec[numstate, numvec])

    # --- output ---
    def print_ci_vec(self, path: str, threshold: float = -1.0) -> None:
        """The CI-vector text of the reference's output (print_solutions + print_ci_vec,
        Output.cpp:135-144, 190-263): coefficients with |c| >= threshold."""
        c = np.ascontiguousarray(self.get_eigvec())
        up = getattr(self, "up", None)
        down = getattr(self, "down", None)
        name = getattr(self, "list_name", None)
        A.check(A.lib().cigpu_write_civec(path.encode(), self.method, self.get_l(), self.gNup(), self.gNdown(), len(c),
                                          A.ptr(c), self.get_ci_energy(), self.get_econst(), threshold, A.ptr(up),
                                          A.ptr(down), getattr(self, "words", 1),
                                          name.encode() if name else None), "cigpu_write_civec")

    def print_rdm(self, path: str, twordm: bool = True) -> None:
        """CIMethod::print_one_rdm / print_two_rdm text (CIMethod.cpp:184-195)."""
        self.construct_density(0, twordm)
        one, aa, ab, bb = self._cid.arrays()
        A.check(A.lib().cigpu_write_rdm(path.encode(), self.get_l(), A.ptr(one), A.ptr(aa) if twordm else None,
                                        A.ptr(ab) if twordm else None, A.ptr(bb) if twordm else None),
                "cigpu_write_rdm")

    # --- density ---
    def get_density(self):
        raise NotImplementedError

    def construct_density(self, state: int = 0, trdm: bool = True) -> None:
        if state != 0:
            raise ValueError("only the ground state is available")
        if self._cid is None:
            self._cid = self.get_density()
        self._cid.construct_density(trdm)

    @property
    def cid(self):
        return self._cid


class FCI(CIMethod):
    method = A.FCI
    name = "FCI"

    def _dim(self) -> int:
        return math.comb(self._ham.L, self._ham.nup) * math.comb(self._ham.L, self._ham.ndown)

    def gUpDim(self) -> int: return math.comb(self._ham.L, self._ham.nup)
    def gDownDim(self) -> int: return math.comb(self._ham.L, self._ham.ndown)

    def get_density(self):
        return DensFCI(self)


class DOCI(CIMethod):
    method = A.DOCI
    name = "DOCI"

    def _dim(self) -> int:
        return math.comb(self._ham.L, self._ham.nup)

    def gUpDim(self) -> int: return math.comb(self._ham.L, self._ham.nup)
    def gDownDim(self) -> int: return math.comb(self._ham.L, self._ham.ndown)

    def get_density(self):
        return DensDOCI(self)


def read_determinants(path: str, L: int):
    """Permutator_File::read_file (Permutator.cpp:179-224) through the library's reader:
    (up, down, words) with `words` 64-bit words per string (2 when L > 64)."""
    words = 1 if L <= 64 else 2
    n, nb = ctypes.c_int64(), ctypes.c_int()
    p = path.encode()
    A.check(A.lib().cigpu_dets_read(p, words, 0, None, None, ctypes.byref(n), ctypes.byref(nb)), "cigpu_dets_read")
    up = np.zeros(n.value * words, np.uint64)
    down = np.zeros(n.value * words, np.uint64)
    A.check(A.lib().cigpu_dets_read(p, words, n.value, A.ptr(up), A.ptr(down), ctypes.byref(n), ctypes.byref(nb)),
            "cigpu_dets_read")
    return up, down, words


class FCI_File(CIMethod):
    """CI over a determinant list (FCI_File, CIMethod.h:164-173): rows in list order.
    The list comes from a determinant file (``permfile``) or from ``up``/``down``
    arrays of ``words`` 64-bit words per string."""

    method = A.DETS
    name = "FCI_File"
    storage = A.DETS_CRS

    def __init__(self, ham: Hamiltonian, permfile: str | None = None, precision: int = A.FP64,
                 up: np.ndarray | None = None, down: np.ndarray | None = None, words: int | None = None,
                 build: bool = True):
        self.list_name = None
        if permfile is not None:
            up, down, words = read_determinants(permfile, ham.L)
            # Permutator::get_clean_detfile (Permutator.cpp:88-100): the file name without
            # directory and extension, with the characters _()-./\ removed
            import os
            base = os.path.splitext(os.path.basename(permfile))[0]
            self.list_name = "".join(ch for ch in base if ch not in "_()-./\\")
        if up is None or down is None:
            raise ValueError("a determinant file or up/down arrays are needed")
        self.words = words or (1 if ham.L <= 64 else 2)
        self.up = np.ascontiguousarray(up, dtype=np.uint64)
        self.down = np.ascontiguousarray(down, dtype=np.uint64)
        super().__init__(ham, precision, build)

    def build_ci(self) -> None:
        out = ctypes.c_void_p()
        A.check(A.lib().cigpu_build_dets(self._ham.device(), self._dim(), self.words, A.ptr(self.up), A.ptr(self.down),
                                         self.storage, self.precision, None, ctypes.byref(out)), "cigpu_build_dets")
        self._mat = SparseMatrix_CRS_Sym(_Handle(out.value, A.lib().cigpu_crs_destroy), self._ham)

    def _dim(self) -> int:
        return len(self.up) // self.words

    def get_density(self):
        return DensFILE(self)


def ci_big_lines(cisize_gb: float) -> int:
    """The determinants whose block of the matrix CI_Big keeps for a CISIZE memory
    budget in GB: numelements = CISIZE 2^30 3 / (64 5) 10 / 2, numlines =
    round((-1 + sqrt(1 + 8 numelements)) / 2) (CI_Big::CI_Big, CIMethod.cpp:596-598)."""
    import math
    numelements = int(cisize_gb * 1024.0 * 1024.0 * 1024.0 * 3 / (64.0 * 5) * 10.0 / 2.0)
    return int(round((-1 + math.sqrt(1 + 8 * numelements)) / 2))


class CI_Big(FCI_File):
    """CI_Big (CIMethod.h:176-189): the determinant list with the block of the matrix
    among its first ``keep`` determinants stored and every other element recomputed
    in each matvec (FP64). ``keep`` defaults to none; ``cisize_gb`` sizes it as the
    reference does from its CISIZE budget (ci_big_lines)."""

    name = "CI_Big"
    storage = A.DETS_ONTHEFLY

    def __init__(self, ham: Hamiltonian, permfile: str | None = None, precision: int = A.FP64,
                 up: np.ndarray | None = None, down: np.ndarray | None = None, words: int | None = None,
                 build: bool = True, keep: int | None = None, cisize_gb: float | None = None):
        self.keep = keep if keep is not None else (ci_big_lines(cisize_gb) if cisize_gb is not None else 0)
        super().__init__(ham, permfile, precision, up, down, words, build)

    def build_ci(self) -> None:
        out = ctypes.c_void_p()
        keep = max(0, min(self.keep, self._dim()))
        A.check(A.lib().cigpu_build_dets_partial(self._ham.device(), self._dim(), self.words, A.ptr(self.up),
                                                 A.ptr(self.down), keep, None, ctypes.byref(out)),
                "cigpu_build_dets_partial")
        self._mat = SparseMatrix_CRS_Sym(_Handle(out.value, A.lib().cigpu_crs_destroy), self._ham)


class CIDens:
    """RDMs of the solved state (CIDens.h:29-131)."""

    def __init__(self, cim: CIMethod, state: int = 0):
        self._cim = cim
        self._state = state
        self._one = None
        self._aa = self._ab = self._bb = None
        self._solved = (False, False)

    def dim(self) -> int:
        return self._cim.get_l()

    def construct_density(self, twordm: bool = True) -> None:
        L = self.dim()
        np_ = L * (L - 1) // 2
        c = np.ascontiguousarray(self._cim.get_eigvec(), dtype=np.float64)
        one = np.empty((2, L, L))
        aa = np.empty((np_, np_)) if twordm else None
        ab = np.empty((L * L, L * L)) if twordm else None
        bb = np.empty((np_, np_)) if twordm else None
        A.check(A.lib().cigpu_rdm(self._cim._mat.handle, A.ptr(c), A.ptr(one), A.ptr(aa), A.ptr(ab), A.ptr(bb)),
                "cigpu_rdm")
        self._one, self._aa, self._ab, self._bb = one, aa, ab, bb
        self._solved = (True, bool(twordm))

    def is_constructed(self):
        return self._solved

    def get_one_rdm(self, spin: int, i: int, j: int) -> float:
        return float(self._one[spin, i, j])

    def get_two_rdm(self, spin: int, i: int, j: int, k: int, l: int) -> float:
        """CIDens::get_two_rdm (CIDens.cpp:166-190)."""
        L = self.dim()
        if spin == 1:
            return float(self._ab[i * L + j, k * L + l])
        if i == j or k == l:
            return 0.0
        sign = 1.0
        if i > j:
            i, j, sign = j, i, -sign
        if k > l:
            k, l, sign = l, k, -sign
        X = self._aa if spin == 0 else self._bb
        return sign * float(X[i * L + j - (i + 1) * (i + 2) // 2, k * L + l - (k + 1) * (k + 2) // 2])

    def arrays(self):
        return self._one, self._aa, self._ab, self._bb

    def get_one_electron_energy(self) -> float:
        h = self._cim.get_ham().h
        return float(np.sum(h * (self._one[0] + self._one[1])))

    def get_two_electron_energy(self) -> float:
        L = self.dim()
        g0 = np.zeros((L,) * 4)
        g2 = np.zeros((L,) * 4)
        iu = [(p, q) for p in range(L) for q in range(p + 1, L)]
        for a, (p, q) in enumerate(iu):
            for b, (r, s) in enumerate(iu):
                for X, G in ((self._aa, g0), (self._bb, g2)):
                    v = X[a, b]
                    G[p, q, r, s] = v
                    G[q, p, r, s] = -v
                    G[p, q, s, r] = -v
                    G[q, p, s, r] = v
        g1 = self._ab.reshape((L,) * 4)
        vphys = np.transpose(self._cim.get_ham().eri, (0, 2, 1, 3))
        return 0.5 * float(np.sum(vphys * (g0 + 2.0 * g1 + g2)))

    def get_dens_energy(self) -> float:
        """CIDens::get_dens_energy (CIDens.cpp:928-932)."""
        return self.get_one_electron_energy() + self.get_two_electron_energy() + self._cim.get_econst()

    def test_invariants(self, twordm: bool = True) -> None:
        """CIDens::test_invariants (CIDens.cpp:365-409), raising instead of exiting."""
        N = self._cim.gNup() + self._cim.gNdown()
        tr1 = float(np.trace(self._one[0]) + np.trace(self._one[1]))
        if abs(tr1 - N) > 1e-9:
            raise AssertionError(f"trace of the 1-RDM {tr1} != {N}")
        if twordm:
            tr2 = float(np.trace(self._aa) + np.trace(self._bb) + np.trace(self._ab))
            if abs(tr2 - N * (N - 1) / 2) > 1e-5:
                raise AssertionError(f"trace of the 2-RDM {tr2} != {N * (N - 1) / 2}")


class DensFILE(CIDens):
    """RDMs of a determinant list's state (DensFILE, CIDens.h:157-170)."""


class DensFCI(CIDens):
    pass


class DensDOCI(CIDens):
    pass
