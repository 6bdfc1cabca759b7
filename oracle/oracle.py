"""Python front end of the test oracle (test infrastructure, not product code).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module. It wraps two CPU libraries:

* ``port`` -- ``oracle/_build/libcigpu_oracle.so``, the project-written C
  restatement (``ciflow_oracle.c``) of the CIFlow CI path; it builds on any
  machine with gcc and is the oracle on the GPU machine;
* ``ref``  -- ``oracle/_ref/libciflow_ref.so``, the CIFlow reference sources
  compiled unmodified with link-only shims (only where the reference tree is
  present); it pins the port.

Eigenpairs come from scipy's ARPACK (``eigsh``: dsaupd/dseupd, which='SA',
ncv=min(42, n), tol=0), as in SparseMatrix_CRS::arpackDiagonalize
(SparseMatrix_CRS.cpp:360-481).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "libcigpu_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libciflow_ref.so")
# The CIFlow source tree the reference library is compiled from: CIGPU_REFERENCE_ROOT,
# else the checkout location used where the fixtures were made. Only build_ref()
# and the fixture generator read it; nothing on a GPU host needs it.
REF_ROOT = os.environ.get("CIGPU_REFERENCE_ROOT") or "/root/reference"

FCI, DOCI = 0, 1
_P = ctypes.c_void_p


def build_port() -> str:
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return PORT_LIB


def build_ref() -> str | None:
    if not os.path.isdir(os.path.join(REF_ROOT, "src")):
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_ROOT={REF_ROOT}", "-j8"], check=True)
    return REF_LIB


_port = None
_ref = None


def port():
    global _port
    if _port is None:
        if not os.path.exists(PORT_LIB):
            build_port()
        lib = ctypes.CDLL(PORT_LIB)
        lib.orc_binom.restype = ctypes.c_int64
        lib.orc_binom.argtypes = [ctypes.c_int, ctypes.c_int]
        lib.orc_dim.restype = ctypes.c_int64
        lib.orc_dim.argtypes = [ctypes.c_int] * 4
        lib.orc_build_upper.restype = ctypes.c_int
        lib.orc_build_upper.argtypes = [ctypes.c_int] * 4 + [_P] * 5
        lib.orc_sym_mvprod.argtypes = [ctypes.c_int64] + [_P] * 5
        lib.orc_sym_mvprod_omp.argtypes = [ctypes.c_int64] + [_P] * 5
        lib.orc_build_rows.restype = ctypes.c_int64
        lib.orc_build_rows.argtypes = [ctypes.c_int] * 4 + [_P, _P, ctypes.c_int64, ctypes.c_int64, _P, _P, _P]
        lib.orc_sym_mvprod_rows.argtypes = [ctypes.c_int64, ctypes.c_int64] + [_P] * 5
        for f in (lib.orc_rdm_pairs, lib.orc_rdm_excitations):
            f.restype = ctypes.c_int
            f.argtypes = [ctypes.c_int] * 4 + [_P] * 5
        _port = lib
    return _port


def ref():
    """The reference library, or None where the reference tree is absent."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_LIB) and build_ref() is None:
            return None
        lib = ctypes.CDLL(REF_LIB)
        lib.ref_ham_read_file.restype = ctypes.c_int
        lib.ref_ham_read_file.argtypes = [ctypes.c_char_p] + [_P] * 6
        lib.ref_ci_create.restype = _P
        lib.ref_ci_create.argtypes = [ctypes.c_int, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_double, _P, _P]
        lib.ref_ci_destroy.argtypes = [_P]
        lib.ref_ci_dim.restype = ctypes.c_longlong
        lib.ref_ci_dim.argtypes = [_P]
        lib.ref_ci_nnz.restype = ctypes.c_longlong
        lib.ref_ci_nnz.argtypes = [_P]
        lib.ref_ci_export.argtypes = [_P] * 4
        lib.ref_ci_mvprod.argtypes = [_P] * 3
        lib.ref_ci_density.restype = ctypes.c_double
        lib.ref_ci_density.argtypes = [_P, ctypes.c_double] + [_P] * 5
        lib.ref_file_ci_create.restype = _P
        lib.ref_file_ci_create.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                           _P, _P, ctypes.c_char_p]
        lib.ref_file_dets.argtypes = [_P, _P, _P]
        lib.ref_print_civec.restype = ctypes.c_int
        lib.ref_print_civec.argtypes = [_P, ctypes.c_double, _P, ctypes.c_double, ctypes.c_char_p]
        lib.ref_print_rdm.restype = ctypes.c_int
        lib.ref_print_rdm.argtypes = [_P, ctypes.c_double, _P, ctypes.c_char_p]
        lib.ref_jacobi.restype = ctypes.c_int
        lib.ref_jacobi.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] + [_P] * 2 + [ctypes.c_int] + [_P] * 6
        lib.ref_doci_scan.restype = ctypes.c_int
        lib.ref_doci_scan.argtypes = [_P, ctypes.c_double] + [_P] * 4 + [ctypes.c_int] + [_P] * 2
        _ref = lib
    return _ref


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_P)


class UpperCRS:
    """CIFlow's SparseMatrix_CRS_Sym content: upper triangle incl. diagonal."""

    def __init__(self, row: np.ndarray, col: np.ndarray, val: np.ndarray):
        self.row, self.col, self.val = row, col, val

    @property
    def n(self) -> int:
        return len(self.row) - 1

    @property
    def nnz(self) -> int:
        return len(self.col)

    def full_csr(self):
        import scipy.sparse as sp
        n = self.n
        u = sp.csr_matrix((self.val, self.col.astype(np.int64), self.row.astype(np.int64)), shape=(n, n))
        return (u + u.T - sp.diags(u.diagonal())).tocsr()


def dim(method: int, L: int, nup: int, ndown: int) -> int:
    return int(port().orc_dim(method, L, nup, ndown))


def build_upper(method: int, ints) -> UpperCRS:
    lib = port()
    n = dim(method, ints.L, ints.nup, ints.ndown)
    h = np.ascontiguousarray(ints.h, dtype=np.float64)
    eri = np.ascontiguousarray(ints.eri, dtype=np.float64)
    row = np.zeros(n + 1, np.int64)
    rc = lib.orc_build_upper(method, ints.L, ints.nup, ints.ndown, _ptr(h), _ptr(eri), _ptr(row), None, None)
    if rc != 0:
        raise ValueError("oracle build rejected the problem")
    col = np.empty(row[-1], np.uint32)
    val = np.empty(row[-1], np.float64)
    lib.orc_build_upper(method, ints.L, ints.nup, ints.ndown, _ptr(h), _ptr(eri), _ptr(row), _ptr(col), _ptr(val))
    return UpperCRS(row, col, val)


def build_rows(method: int, ints, r0: int, r1: int):
    """Rows [r0, r1) of the upper CRS: (local row pointers, col, val)."""
    lib = port()
    h = np.ascontiguousarray(ints.h, dtype=np.float64)
    eri = np.ascontiguousarray(ints.eri, dtype=np.float64)
    cnt = np.zeros(r1 - r0 + 1, np.int64)
    lib.orc_build_rows(method, ints.L, ints.nup, ints.ndown, _ptr(h), _ptr(eri), r0, r1, _ptr(cnt[1:]), None, None)
    off = np.concatenate([[0], np.cumsum(cnt[1:])]).astype(np.int64)
    col = np.empty(off[-1], np.uint32)
    val = np.empty(off[-1], np.float64)
    lib.orc_build_rows(method, ints.L, ints.nup, ints.ndown, _ptr(h), _ptr(eri), r0, r1, _ptr(off), _ptr(col),
                       _ptr(val))
    return off, col, val


def sym_mvprod_rows(r0: int, off, col, val, x, y) -> None:
    port().orc_sym_mvprod_rows(r0, len(off) - 1, _ptr(off), _ptr(col), _ptr(val), _ptr(x), _ptr(y))


def sym_mvprod(m: UpperCRS, x: np.ndarray, threaded: bool = False) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty(m.n)
    f = port().orc_sym_mvprod_omp if threaded else port().orc_sym_mvprod
    f(m.n, _ptr(m.row), _ptr(m.col), _ptr(m.val), _ptr(x), _ptr(y))
    return y


def lowest_eigenpair(m: UpperCRS, v0: np.ndarray | None = None, tol: float = 0.0):
    """ARPACK (scipy eigsh) with the reference's settings: which='SA', ncv=min(42,n),
    tol=0, maxiter=3n. Returns (E0 without Econst, c normalised)."""
    import scipy.sparse.linalg as sla
    n = m.n
    if n <= 2:
        w, v = np.linalg.eigh(m.full_csr().toarray())
        return float(w[0]), v[:, 0]
    a = m.full_csr()
    if v0 is None:
        v0 = np.random.default_rng(12345).standard_normal(n)
    w, v = sla.eigsh(a, k=1, which="SA", ncv=min(42, n - 1), tol=tol, maxiter=3 * n, v0=v0)
    c = v[:, 0]
    return float(w[0]), c / np.linalg.norm(c)


def rdm(method: int, L: int, nup: int, ndown: int, c: np.ndarray, literal: bool = False):
    """(rdm1[2,L,L], aa[np,np], ab[L*L,L*L], bb[np,np]) with the CIDens conventions."""
    lib = port()
    np_ = L * (L - 1) // 2
    c = np.ascontiguousarray(c, dtype=np.float64)
    r1 = np.zeros((2, L, L))
    aa = np.zeros((np_, np_))
    ab = np.zeros((L * L, L * L))
    bb = np.zeros((np_, np_))
    f = lib.orc_rdm_pairs if literal else lib.orc_rdm_excitations
    rc = f(method, L, nup, ndown, _ptr(c), _ptr(r1), _ptr(aa), _ptr(ab), _ptr(bb))
    if rc != 0:
        raise ValueError("oracle rdm rejected the problem")
    return r1, aa, ab, bb


def two_rdm_get(L: int, aa, ab, bb, spin: int, i: int, j: int, k: int, l: int) -> float:
    """CIDens::get_two_rdm semantics (CIDens.cpp:166-190)."""
    if spin == 1:
        return ab[i * L + j, k * L + l]
    if i == j or k == l:
        return 0.0
    sign = 1.0
    if i > j:
        i, j, sign = j, i, -sign
    if k > l:
        k, l, sign = l, k, -sign
    X = aa if spin == 0 else bb
    pi = i * L + j - (i + 1) * (i + 2) // 2
    pk = k * L + l - (k + 1) * (k + 2) // 2
    return sign * X[pi, pk]


def full_two_rdm_blocks(L: int, aa, ab, bb):
    """Dense Gamma0/Gamma1/Gamma2 [L,L,L,L] from the packed pair matrices."""
    g0 = np.zeros((L, L, L, L))
    g2 = np.zeros((L, L, L, L))
    iu = [(p, q) for p in range(L) for q in range(p + 1, L)]
    for a, (p, q) in enumerate(iu):
        for b, (r, s) in enumerate(iu):
            for X, G in ((aa, g0), (bb, g2)):
                v = X[a, b]
                G[p, q, r, s] = v
                G[q, p, r, s] = -v
                G[p, q, s, r] = -v
                G[q, p, s, r] = v
    g1 = ab.reshape(L, L, L, L)
    return g0, g1, g2


def dens_energy(ints, rdm1, aa, ab, bb) -> float:
    """CIDens::get_dens_energy (CIDens.cpp:898-932): one- plus two-electron energy
    (alpha-beta counted twice) plus Econst."""
    L = ints.L
    e1 = float(np.sum(ints.h * (rdm1[0] + rdm1[1])))
    g0, g1, g2 = full_two_rdm_blocks(L, aa, ab, bb)
    vphys = np.transpose(ints.eri, (0, 2, 1, 3))  # <ij|kl> = (ik|jl)
    e2 = 0.5 * float(np.sum(vphys * (g0 + 2.0 * g1 + g2)))
    return e1 + e2 + ints.econst


# ---------------- reference (only where the reference tree exists) ----------------

def ref_read_file(filename: str):
    """Integrals from a psi4 text dump through the reference reader."""
    from ciflow_gb300.synthetic import Integrals
    lib = ref()
    L, na, nb, ec = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
    fn = filename.encode()
    lib.ref_ham_read_file(fn, ctypes.byref(L), ctypes.byref(na), ctypes.byref(nb), ctypes.byref(ec), None, None)
    n = L.value
    h = np.zeros((n, n))
    eri = np.zeros((n, n, n, n))
    lib.ref_ham_read_file(fn, ctypes.byref(L), ctypes.byref(na), ctypes.byref(nb), ctypes.byref(ec), _ptr(h), _ptr(eri))
    return Integrals(n, na.value, nb.value, ec.value, h, eri)


class RefCI:
    """A reference FCI/DOCI object (CRS built by the reference constructor)."""

    def __init__(self, method: int, ints=None, filename: str | None = None, det_file: str | None = None):
        lib = ref()
        self.lib = lib
        if det_file is not None:  # FCI_File over a determinant list
            if filename is not None:
                self.h = lib.ref_file_ci_create(filename.encode(), 0, 0, 0, 0.0, None, None, det_file.encode())
            else:
                hh = np.ascontiguousarray(ints.h)
                ee = np.ascontiguousarray(ints.eri)
                self.h = lib.ref_file_ci_create(None, ints.L, ints.nup, ints.ndown, ints.econst, _ptr(hh), _ptr(ee),
                                                det_file.encode())
        elif filename is not None:
            self.h = lib.ref_ci_create(method, filename.encode(), 0, 0, 0, 0.0, None, None)
        else:
            hh = np.ascontiguousarray(ints.h)
            ee = np.ascontiguousarray(ints.eri)
            self.h = lib.ref_ci_create(method, None, ints.L, ints.nup, ints.ndown, ints.econst, _ptr(hh), _ptr(ee))
        self.method = method

    def crs(self) -> UpperCRS:
        n = self.lib.ref_ci_dim(self.h)
        nnz = self.lib.ref_ci_nnz(self.h)
        row = np.zeros(n + 1, np.uint32)
        col = np.zeros(nnz, np.uint32)
        val = np.zeros(nnz)
        self.lib.ref_ci_export(self.h, _ptr(row), _ptr(col), _ptr(val))
        return UpperCRS(row.astype(np.int64), col, val)

    def mvprod(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.lib.ref_ci_dim(self.h))
        self.lib.ref_ci_mvprod(self.h, _ptr(x), _ptr(y))
        return y

    def density(self, L: int, e: float, c: np.ndarray):
        np_ = L * (L - 1) // 2
        r1 = np.zeros((2, L, L))
        aa = np.zeros((np_, np_))
        ab = np.zeros((L * L, L * L))
        bb = np.zeros((np_, np_))
        c = np.ascontiguousarray(c, dtype=np.float64)
        ed = self.lib.ref_ci_density(self.h, e, _ptr(c), _ptr(r1), _ptr(aa), _ptr(ab), _ptr(bb))
        return (r1, aa, ab, bb), ed

    def print_civec(self, e: float, c: np.ndarray, nauw: float, path: str) -> None:
        """The reference's CI-vector text block for (e without Econst, c)."""
        c = np.ascontiguousarray(c, dtype=np.float64)
        if self.lib.ref_print_civec(self.h, e, _ptr(c), nauw, path.encode()) != 0:
            raise OSError(path)

    def print_rdm(self, e: float, c: np.ndarray, path: str) -> None:
        """The reference's RDM text (print_one_rdm + print_two_rdm) for (e, c)."""
        c = np.ascontiguousarray(c, dtype=np.float64)
        if self.lib.ref_print_rdm(self.h, e, _ptr(c), path.encode()) != 0:
            raise OSError(path)

    def dets(self):
        """(up, down) uint64 arrays of a FCI_File object's determinant list."""
        n = self.lib.ref_ci_dim(self.h)
        up = np.zeros(n, np.uint64)
        dn = np.zeros(n, np.uint64)
        self.lib.ref_file_dets(self.h, _ptr(up), _ptr(dn))
        return up, dn

    def doci_scan(self, L: int, e: float, c: np.ndarray, fixed=()):
        """DensDOCI::find_min_angle / calc_rotate for every pair k < l, with the
        selection of LocalMinimizer::scan_orbitals: (theta, energy, found, fixed_energy)."""
        np_ = L * (L - 1) // 2
        th = np.zeros(np_)
        en = np.zeros(np_)
        fd = np.zeros(np_, np.int32)
        fx = np.ascontiguousarray(np.asarray(fixed, dtype=np.float64))
        fe = np.zeros((np_, len(fx)))
        c = np.ascontiguousarray(c, dtype=np.float64)
        rc = self.lib.ref_doci_scan(self.h, e, _ptr(c), _ptr(th), _ptr(en), _ptr(fd), len(fx),
                                    _ptr(fx) if len(fx) else None, _ptr(fe) if len(fx) else None)
        if rc != 0:
            raise ValueError("reference DOCI scan needs a DOCI object")
        return th, en, fd, fe

    def close(self):
        if self.h:
            self.lib.ref_ci_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def ref_jacobi(ints, rotations):
    """OrbitalTransform::do_jacobi_rotation applied in order for (k, l, theta) in
    `rotations`: (h, eri chemist, U row-major) from the reference."""
    lib = ref()
    L = ints.L
    k = np.array([r[0] for r in rotations], np.int32)
    l = np.array([r[1] for r in rotations], np.int32)
    th = np.array([r[2] for r in rotations], np.float64)
    hh = np.ascontiguousarray(ints.h, dtype=np.float64)
    ee = np.ascontiguousarray(ints.eri, dtype=np.float64)
    h = np.zeros((L, L))
    eri = np.zeros((L,) * 4)
    U = np.zeros((L, L))
    lib.ref_jacobi(L, ints.nup, ints.ndown, ints.econst, _ptr(hh), _ptr(ee), len(k), _ptr(k), _ptr(l), _ptr(th),
                   _ptr(h), _ptr(eri), _ptr(U))
    return h, eri, U


def ref_rotate(ints, U):
    """OrbitalTransform::fillHamCI with the unitary U (row-major, U[a, p]): the
    rotated (h, eri chemist) of the reference."""
    lib = ref()
    lib.ref_rotate.restype = ctypes.c_int
    lib.ref_rotate.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] + [_P] * 5
    L = ints.L
    hh = np.ascontiguousarray(ints.h, dtype=np.float64)
    ee = np.ascontiguousarray(ints.eri, dtype=np.float64)
    U = np.ascontiguousarray(U, dtype=np.float64)
    h = np.zeros((L, L))
    eri = np.zeros((L,) * 4)
    lib.ref_rotate(L, ints.nup, ints.ndown, ints.econst, _ptr(hh), _ptr(ee), _ptr(U), _ptr(h), _ptr(eri))
    return h, eri


def build_dets(ints, up: np.ndarray, down: np.ndarray, words: int = 1) -> UpperCRS:
    """The oracle's FCI_File CRS of a determinant list (strings of `words` 64-bit words)."""
    lib = port()
    lib.orc_build_dets.restype = ctypes.c_int
    lib.orc_build_dets.argtypes = [ctypes.c_int] * 3 + [_P, _P, ctypes.c_int64, ctypes.c_int] + [_P] * 5
    n = len(up) // words
    h = np.ascontiguousarray(ints.h, dtype=np.float64)
    eri = np.ascontiguousarray(ints.eri, dtype=np.float64)
    up = np.ascontiguousarray(up, dtype=np.uint64)
    down = np.ascontiguousarray(down, dtype=np.uint64)
    row = np.zeros(n + 1, np.int64)
    if lib.orc_build_dets(ints.L, ints.nup, ints.ndown, _ptr(h), _ptr(eri), n, words, _ptr(up), _ptr(down), _ptr(row),
                          None, None) != 0:
        raise ValueError("oracle rejected the determinant list")
    col = np.empty(row[-1], np.uint32)
    val = np.empty(row[-1], np.float64)
    lib.orc_build_dets(ints.L, ints.nup, ints.ndown, _ptr(h), _ptr(eri), n, words, _ptr(up), _ptr(down), _ptr(row),
                       _ptr(col), _ptr(val))
    return UpperCRS(row, col, val)


def rdm_dets(L: int, up: np.ndarray, down: np.ndarray, c: np.ndarray):
    """DensFILE RDMs of a determinant list's state, CIDens conventions (64-bit strings)."""
    lib = port()
    lib.orc_rdm_dets.restype = ctypes.c_int
    lib.orc_rdm_dets.argtypes = [ctypes.c_int, ctypes.c_int] + [_P] * 7
    np_ = L * (L - 1) // 2
    up = np.ascontiguousarray(up, dtype=np.uint64)
    down = np.ascontiguousarray(down, dtype=np.uint64)
    c = np.ascontiguousarray(c, dtype=np.float64)
    r1 = np.zeros((2, L, L))
    aa = np.zeros((np_, np_))
    ab = np.zeros((L * L, L * L))
    bb = np.zeros((np_, np_))
    if lib.orc_rdm_dets(L, len(up), _ptr(up), _ptr(down), _ptr(c), _ptr(r1), _ptr(aa), _ptr(ab), _ptr(bb)) != 0:
        raise ValueError("oracle rejected the list")
    return r1, aa, ab, bb

