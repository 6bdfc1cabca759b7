"""GPU matvec and eigensolver parity.

mvprod must equal the reference SparseMatrix_CRS_Sym::mvprod (restated by the
oracle) to FP64 round-off; E0 must match the reference ARPACK energy to 1e-8 Eh
(plain FP64) and to 1e-6 Eh (mixed), including the DOCI known answer
-15.225362047972723 (reference tests/src/TestDOCI.cpp:31).
"""
import ctypes

import numpy as np
import pytest

import oracle as O
from ciflow_gb300 import _abi as A
from ciflow_gb300.ciflow import DOCI, FCI, Hamiltonian
from ciflow_gb300.synthetic import make_integrals
from tests.helpers import beh2_integrals, integrals, load_golden

pytestmark = pytest.mark.gpu


def build(cls, ints, precision=A.FP64):
    return cls(Hamiltonian.from_integrals(ints), precision=precision)


@pytest.mark.parametrize("name", ["c0", "c4"])
@pytest.mark.parametrize("precision", [A.FP64, A.MIXED])
def test_mvprod_matches_reference_matvec(name, precision):
    ints = integrals(name)
    ref = O.build_upper(O.FCI, ints)
    m = build(FCI, ints, precision).get_mat()
    x = np.random.default_rng(7).standard_normal(m.n)
    y_ref = O.sym_mvprod(ref, x, threaded=True)
    y = m.mvprod(x)
    scale = np.abs(y_ref).max()
    # FP64 product (from the split FP32 values hi + lo for the mixed CRS): summation order only
    assert np.abs(y - y_ref).max() <= 1e-12 * scale


@pytest.mark.parametrize("L,n", [(8, 4), (10, 3), (12, 6), (14, 1), (9, 9), (16, 8), (33, 2)])
@pytest.mark.parametrize("precision", [A.FP64, A.MIXED])
def test_doci_matvec_matches_reference_matvec(L, n, precision):
    """The DOCI matvec (MIXED: matrix-free, pair hops generated per row, here its
    FP64 product; FP64: the CRS) equals the reference's Sym::mvprod over the DOCI
    CRS (oracle restatement) to FP64 round-off, and its element counts equal the
    CRS's."""
    ints = make_integrals(L, n, n, nchol=8, seed=5 * L + n)
    ref = O.build_upper(O.DOCI, ints)
    m = build(DOCI, ints, precision).get_mat()
    lay, stored = ctypes.c_int(), ctypes.c_int64()
    A.check(A.lib().cigpu_crs_layout(m.handle, ctypes.byref(lay), ctypes.byref(stored)))
    if precision == A.MIXED:
        assert lay.value == A.LAYOUT_PAIRS and stored.value == 0
    else:
        assert lay.value == A.LAYOUT_CRS
    dim, nu, nf = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    A.check(A.lib().cigpu_crs_dims(m.handle, ctypes.byref(dim), ctypes.byref(nu), ctypes.byref(nf)))
    assert nu.value == ref.nnz and nf.value == 2 * ref.nnz - int(np.count_nonzero(ref.full_csr().diagonal()))
    x = np.random.default_rng(11).standard_normal(m.n)
    y_ref = O.sym_mvprod(ref, x)
    y = m.mvprod(x)
    assert np.abs(y - y_ref).max() <= 1e-12 * max(np.abs(y_ref).max(), 1.0)


def test_doci_pair_matvec_fp32():
    torch = pytest.importorskip("torch")
    ints = make_integrals(12, 6, 6, nchol=8, seed=9)
    ref = O.build_upper(O.DOCI, ints)
    m = build(DOCI, ints, A.MIXED).get_mat()
    x = np.random.default_rng(3).standard_normal(m.n)
    y_ref = O.sym_mvprod(ref, x)
    xd = torch.tensor(x, dtype=torch.float32, device="cuda")
    yd = torch.empty_like(xd)
    m.mvprod_device(xd, yd)
    torch.cuda.synchronize()
    y = yd.cpu().numpy().astype(np.float64)
    # FP32 K, x and accumulation over 37 terms per row
    assert np.abs(y - y_ref).max() <= 2e-5 * np.abs(y_ref).max()


@pytest.mark.parametrize("case", ["c0", "c4", "9x3x5", "11x5x4"])
def test_fp32_device_matvec(case):
    """The FP32 slot matvec against the reference mvprod: equal and unequal spin
    counts, last tiles with padding rows."""
    torch = pytest.importorskip("torch")
    if "x" in case:
        L, na, nb = (int(v) for v in case.split("x"))
        ints = make_integrals(L, na, nb, nchol=8, seed=L + 7 * na + 11 * nb)
    else:
        ints = integrals(case)
    ref = O.build_upper(O.FCI, ints)
    m = build(FCI, ints, A.MIXED).get_mat()
    x = np.random.default_rng(3).standard_normal(m.n)
    y_ref = O.sym_mvprod(ref, x)
    xd = torch.tensor(x, dtype=torch.float32, device="cuda")
    yd = torch.empty_like(xd)
    m.mvprod_device(xd, yd)
    torch.cuda.synchronize()
    y = yd.cpu().numpy().astype(np.float64)
    # FP32 values and FP32 accumulation over ~361 terms per row
    assert np.abs(y - y_ref).max() <= 2e-5 * np.abs(y_ref).max()


def _ints_case(case):
    """'LxNaxNb[xK]' with K factors (8 by default); a trailing '-indefinite' subtracts
    a rank-one pair term, so the two-electron part is no longer positive semidefinite."""
    indefinite = case.endswith("-indefinite")
    parts = [int(v) for v in case.replace("-indefinite", "").split("x")]
    L, na, nb = parts[:3]
    k = parts[3] if len(parts) > 3 else 8
    ints = make_integrals(L, na, nb, nchol=k, seed=L + 7 * na + 11 * nb + k)
    if indefinite:
        m = np.random.default_rng(L).normal(0.0, 0.2, (L, L))
        v = (m + m.T).reshape(-1)
        ints.eri = (ints.eri.reshape(L * L, L * L) - np.multiply.outer(v, v)).reshape(L, L, L, L)
    return ints


@pytest.mark.parametrize("case", ["8x4x4", "9x3x5", "10x5x3x24", "7x3x3-indefinite", "11x5x4", "6x1x5"])
def test_sigma_fp32_matvec(case, monkeypatch):
    """The mixed method's factorised FP32 product (a direct-CI sigma vector, two
    one-body passes over every determinant's single excitations), forced onto small
    spaces: equal and unequal spin counts, ragged 32 x 32 string tiles, a rank above
    one 16-factor chunk, and integrals whose pair matrix is indefinite (eigenpair
    factors with signs) against the reference mvprod."""
    torch = pytest.importorskip("torch")
    monkeypatch.setenv("CIGPU_FP32_PRODUCT", "sigma")
    ints = _ints_case(case)
    ref = O.build_upper(O.FCI, ints)
    m = build(FCI, ints, A.MIXED).get_mat()
    x = np.random.default_rng(5).standard_normal(m.n)
    y_ref = O.sym_mvprod(ref, x)
    xd = torch.tensor(x, dtype=torch.float32, device="cuda")
    yd = torch.empty_like(xd)
    torch.cuda.synchronize()
    n0 = A.lib().cigpu_kernel_launches()
    m.mvprod_device(xd, yd)
    torch.cuda.synchronize()
    assert A.lib().cigpu_kernel_launches() - n0 == 3  # transpose + the two passes: the sigma operator ran
    y = yd.cpu().numpy().astype(np.float64)
    assert np.abs(y - y_ref).max() <= 2e-5 * np.abs(y_ref).max()


@pytest.mark.parametrize("case", ["9x3x5", "7x3x3-indefinite"])
def test_sigma_mixed_solve(case, monkeypatch):
    """A mixed solve whose FP32 corrections come from the factorised operator
    reaches the FP64 ground state of the stored matrix (the anchors' residual is
    exact)."""
    monkeypatch.setenv("CIGPU_FP32_PRODUCT", "sigma")
    ints = _ints_case(case)
    e_ref = np.linalg.eigvalsh(O.build_upper(O.FCI, ints).full_csr().toarray())[0] + ints.econst
    f = build(FCI, ints, A.MIXED)
    f.solve(tol=1e-8)
    assert abs(f.get_ci_energy() - e_ref) < 1e-9


def test_doci_known_answer():
    ints, meta, _ = beh2_integrals()
    cim = build(DOCI, ints)
    cim.solve(tol=1e-10)
    # reference tests/src/TestDOCI.cpp:31 (BOOST_CHECK_CLOSE 1e-10 percent)
    assert abs(cim.get_ci_energy() - (-15.225362047972723)) <= 1e-12 * 15.3 + 1e-11
    assert cim.info["residual"] <= 1e-10


@pytest.mark.parametrize("tag,cls", [("doci", DOCI), ("fci", FCI)])
@pytest.mark.parametrize("precision", [A.FP64, A.MIXED])
def test_beh2_energy(tag, cls, precision):
    ints, meta, _ = beh2_integrals()
    cim = build(cls, ints, precision)
    cim.solve(tol=1e-8)
    tol = 1e-8 if precision == A.FP64 else 1e-6
    assert abs(cim.get_ci_energy() - meta[tag]["e0"]) <= tol


@pytest.mark.parametrize("name", ["c0", "c4", "c1", "c2"])
@pytest.mark.parametrize("precision", [A.FP64, A.MIXED])
def test_config_energy(name, precision):
    meta, _ = load_golden(name)
    ints = integrals(name)
    cls = DOCI if meta["config"]["method"] == "DOCI" else FCI
    cim = build(cls, ints, precision)
    cim.solve(tol=1e-6 if name in ("c1", "c2") else 1e-8)
    err = abs(cim.get_ci_energy() - meta["e0"])
    assert err <= (1e-8 if precision == A.FP64 else 1e-6), (err, cim.info)
    c = cim.get_eigvec()
    assert abs(np.linalg.norm(c) - 1) < 1e-10


@pytest.mark.parametrize("precision", [A.FP64, A.MIXED])
def test_residual_is_true_fp64_residual(precision):
    """The reported residual is ||H c - E c|| of the returned vector with the exact
    FP64 matrix, and the solver reaches tol = 1e-8 in both modes."""
    ints = integrals("c0")
    ref = O.build_upper(O.FCI, ints)
    cim = build(FCI, ints, precision)
    cim.solve(tol=1e-8)
    c = cim.get_eigvec()
    e = cim.get_ci_energy() - ints.econst
    r = np.linalg.norm(O.sym_mvprod(ref, c) - e * c)
    assert cim.info["status"] == A.OK and cim.info["converged"]
    assert r <= 1e-8
    assert abs(r - cim.info["residual"]) <= 1e-10
    if precision == A.MIXED:
        assert cim.info["matvecs_fp32"] > cim.info["matvecs_fp64"]


def test_warm_start_converges_faster():
    ints = integrals("c4")
    cim = build(FCI, ints)
    cim.solve(tol=1e-8)
    n_cold = cim.info["matvecs_fp64"]
    c = cim.get_eigvec()
    cim.solve(tol=1e-8, c0=c)
    assert cim.info["matvecs_fp64"] < n_cold


def test_matvec_limit_reports_no_convergence():
    ints = integrals("c4")
    cim = build(FCI, ints)
    cim.solve(tol=1e-12, max_matvec=5)
    assert cim.info["status"] == A.ENOCONV
    assert not cim.info["converged"]


# uneven shapes of the batched/served mix, down to spaces smaller than the Krylov basis
SMALL_SHAPES = [(O.FCI, 4, 0, 0), (O.FCI, 3, 1, 1), (O.DOCI, 6, 2, 2), (O.FCI, 6, 1, 1), (O.FCI, 5, 2, 1),
                (O.DOCI, 8, 3, 3), (O.FCI, 6, 3, 2), (O.FCI, 7, 2, 2)]


@pytest.mark.parametrize("shape", SMALL_SHAPES, ids=lambda s: "%s-L%d-%d-%d" % (("FCI", "DOCI")[s[0]], *s[1:]))
@pytest.mark.parametrize("precision", [A.FP64, A.MIXED])
def test_small_spaces_match_dense_eigensolve(shape, precision):
    method, L, na, nb = shape
    ints = make_integrals(L, na, nb, nchol=16, seed=100 + L * 10 + na)
    ref = O.build_upper(method, ints)
    e_ref = np.linalg.eigvalsh(ref.full_csr().toarray())[0]
    cim = build(DOCI if method == O.DOCI else FCI, ints, precision)
    cim.solve(tol=1e-9)
    tol = 1e-8 if precision == A.FP64 else 1e-6
    assert abs(cim.get_ci_energy() - ints.econst - e_ref) <= tol
    assert cim.info["converged"]


# (L, electrons per spin, seed): spaces where the lowest-diagonal determinant overlaps
# the ground state weakly, so a Davidson started from it alone settles on an excited state
HARD_STARTS = [(7, 1, 1123), (11, 1, 1109), (7, 1, 1234), (10, 4, 1237)]


@pytest.mark.parametrize("case", HARD_STARTS, ids=lambda c: "L%d-%d-s%d" % c)
@pytest.mark.parametrize("precision", [A.FP64, A.MIXED])
def test_solver_finds_the_ground_state(case, precision):
    import scipy.sparse.linalg as sla
    L, ne, seed = case
    ints = make_integrals(L, ne, ne, nchol=16, seed=seed)
    H = O.build_upper(O.FCI, ints).full_csr()
    e_ref = sla.eigsh(H, k=1, which="SA", tol=1e-12)[0][0] if H.shape[0] > 2000 else np.linalg.eigvalsh(H.toarray())[0]
    cim = build(FCI, ints, precision)
    cim.solve(tol=1e-6)
    assert abs(cim.get_ci_energy() - ints.econst - e_ref) <= 1e-6


def test_mixed_restart_keeps_the_previous_ritz_direction():
    """L=11 4a4b (seeded integrals 1114, a request of the served mix): its Davidson
    cycles of 30 vectors only halve the residual. Folds of the full basis keep the
    previous Ritz direction (restarts > 0), and the mixed solve reaches the FP64
    energy in fewer FP32 matvecs than the 165 it took restarting from the anchor
    alone (plain Lanczos takes ~107 FP64 matvecs)."""
    H = Hamiltonian.from_integrals(make_integrals(11, 4, 4, nchol=16, seed=1114))
    ref = FCI(H, precision=A.FP64)
    ref.solve(tol=1e-8)
    m = FCI(H, precision=A.MIXED)
    m.solve(tol=1e-5)  # the served stream's tolerance
    assert m.info["status"] == A.OK and m.info["converged"] == 1
    assert abs(m.get_ci_energy() - ref.get_ci_energy()) < 1e-6
    assert m.info["restarts"] >= 1
    assert m.info["matvecs_fp32"] < 150, m.info
