"""Generate the golden fixtures in tests/golden/ from the CIFlow reference.

Run where the reference tree is available (its location comes from
oracle.REF_ROOT, i.e. CIGPU_REFERENCE_ROOT):

    python tests/golden/make_golden.py [names...]

For each case the reference itself (oracle/_ref, compiled unmodified from the
reference sources) builds the upper-triangle CRS in its FCI/DOCI constructor;
the lowest eigenpair comes from scipy ARPACK driving that CRS with the
reference's arpackDiagonalize settings, and the RDMs from the reference
CIDens (DensFCI/DensDOCI) where its O(dim^2) pair loop is affordable.

Fixtures hold: integral checksum (or the integrals themselves for the BeH2
file fixture), dimension and nnz, SHA-256 of the reference CRS arrays in the
reference layout (uint32 row, uint32 col, float64 val), E0 (+Econst), and the
RDMs in the CIDens packed conventions.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from ciflow_gb300.synthetic import CONFIGS, config_integrals  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def crs_sha256(m: O.UpperCRS) -> str:
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(m.row, dtype=np.uint32).tobytes())
    h.update(np.ascontiguousarray(m.col, dtype=np.uint32).tobytes())
    h.update(np.ascontiguousarray(m.val, dtype=np.float64).tobytes())
    return h.hexdigest()


def solve_ref(r: O.RefCI, n: int, big: bool):
    """Lowest eigenpair of the reference CRS with ARPACK (reference settings)."""
    import scipy.sparse.linalg as sla
    v0 = np.random.default_rng(12345).standard_normal(n)
    if not big:
        return O.lowest_eigenpair(r.crs(), v0=v0)
    m = r.crs()
    op = sla.LinearOperator((n, n), matvec=lambda x: O.sym_mvprod(m, x, threaded=True), dtype=np.float64)
    w, v = sla.eigsh(op, k=1, which="SA", ncv=42, tol=0, maxiter=3 * n, v0=v0)
    c = v[:, 0]
    return float(w[0]), c / np.linalg.norm(c), m


def case_file(name: str, fname: str):
    path = os.path.join(O.REF_ROOT, "tests", "data", fname)
    ints = O.ref_read_file(path)
    out = {"h": ints.h, "eri": ints.eri}
    meta = {"L": ints.L, "nup": ints.nup, "ndown": ints.ndown, "econst": ints.econst, "source": f"tests/data/{fname}"}
    for method, tag in ((O.DOCI, "doci"), (O.FCI, "fci")):
        r = O.RefCI(method, filename=path)
        m = r.crs()
        e, c = O.lowest_eigenpair(m, v0=np.random.default_rng(12345).standard_normal(m.n))
        (r1, aa, ab, bb), ed = r.density(ints.L, e, c)
        meta[tag] = {"dim": m.n, "nnz": m.nnz, "crs_sha256": crs_sha256(m), "e0": e + ints.econst, "dens_energy": ed}
        out.update({f"{tag}_rdm1": r1, f"{tag}_aa": aa, f"{tag}_ab": ab, f"{tag}_bb": bb, f"{tag}_c": c})
        r.close()
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **out)
    with open(os.path.join(OUT, f"{name}.json"), "w") as f:
        json.dump(meta, f, indent=1)


def case_config(name: str, rdm: bool):
    cfg = CONFIGS[name]
    method = O.FCI if cfg["method"] == "FCI" else O.DOCI
    ints = config_integrals(name)
    t0 = time.time()
    r = O.RefCI(method, ints=ints)
    t_build = time.time() - t0
    n = int(r.lib.ref_ci_dim(r.h))
    big = n > 200000
    if big:
        e, c, m = solve_ref(r, n, True)
    else:
        m = r.crs()
        e, c = O.lowest_eigenpair(m, v0=np.random.default_rng(12345).standard_normal(n))
    meta = {"config": cfg, "integrals_sha": ints.checksum(), "dim": n, "nnz": m.nnz,
            "crs_sha256": crs_sha256(m), "e0": e + ints.econst, "ref_build_s": t_build}
    out = {}
    if rdm:
        (r1, aa, ab, bb), ed = r.density(ints.L, e, c)
        meta["dens_energy"] = ed
        out.update({"rdm1": r1, "aa": aa, "ab": ab, "bb": bb})
    r.close()
    if out:
        np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **out)
    with open(os.path.join(OUT, f"{name}.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print(name, json.dumps(meta))


# Orbital-optimiser pieces of the reference: a sequence of Jacobi rotations
# (OrbitalTransform::do_jacobi_rotation with the accumulated unitary) and the DOCI
# pair scan (DensDOCI::find_min_angle / calc_rotate, selection of scan_orbitals)
# of a DOCI ground state, on seeded L=8 integrals (4 pairs, 70 pair determinants).
ORBOPT_ROTATIONS = [(0, 3, 0.37), (2, 5, -0.81), (1, 7, 1.3), (0, 3, 0.2), (6, 4, 0.05)]
ORBOPT_FIXED = [0.1, -0.7, 2.0]


def case_orbopt(name: str):
    from ciflow_gb300.synthetic import make_integrals
    ints = make_integrals(8, 4, 4, nchol=16, seed=77)
    h, eri, U = O.ref_jacobi(ints, ORBOPT_ROTATIONS)
    out = {"h0": ints.h, "eri0": ints.eri, "jac_h": h, "jac_eri": eri, "jac_U": U}
    meta = {"L": 8, "nup": 4, "ndown": 4, "econst": ints.econst, "seed": 77, "nchol": 16,
            "rotations": ORBOPT_ROTATIONS, "fixed_angles": ORBOPT_FIXED}
    # scans in the starting orbitals and after the rotations
    from ciflow_gb300.synthetic import Integrals
    for tag, (hh, ee) in (("scan0", (ints.h, ints.eri)), ("scan1", (h, eri))):
        I = Integrals(8, 4, 4, ints.econst, hh, ee)
        r = O.RefCI(O.DOCI, ints=I)
        m = r.crs()
        e, c = O.lowest_eigenpair(m, v0=np.random.default_rng(12345).standard_normal(m.n))
        th, en, fd, fe = r.doci_scan(8, e, c, ORBOPT_FIXED)
        r.close()
        out.update({f"{tag}_c": c, f"{tag}_theta": th, f"{tag}_energy": en, f"{tag}_found": fd, f"{tag}_fixed": fe})
        meta[f"{tag}_e0"] = e + ints.econst
        meta[f"{tag}_found"] = int(fd.sum())
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **out)
    with open(os.path.join(OUT, f"{name}.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print(name, json.dumps(meta))


def case_warm_chain(name: str):
    """A warm start far above the ground state: the oracle's annealing chain (the
    reference's SimulatedAnnealing loop restated, DOCI L=16 8 pairs, seeded
    integrals 4, chain seed 11, parameters 0.4/0.99/1.4/0.999) run to its 78th
    decided step, whose proposal (a 73-degree rotation of orbitals 9 and 11) leaves
    the current ground state 14 Eh above the new one. Saves the accepted rotations
    before it, the proposal and the oracle's energies."""
    import math
    import orbopt as OO
    from ciflow_gb300.synthetic import make_integrals
    ints = make_integrals(16, 8, 8, nchol=16, seed=4)
    opt = OO.Optimizer(ints, OO.O.DOCI, seed=11)
    p = OO.AnnealParams()
    prop = OO.SplitMix64(OO.stream_seed(opt.seed, 2 * opt.calls + 1))
    temp, max_angle, e_old, decided, accepted = p.temp, p.max_angle, opt.e, 0, []
    while True:
        i, j = prop.below(opt.L), prop.below(opt.L)
        if i == j:
            continue
        u1, u2 = prop.uniform(), prop.uniform()
        angle = max_angle * (u1 - u2)
        h2, e2 = OO.jacobi(opt.h, opt.eri, i, j, angle)
        e_new, c_new = opt._solve(h2, e2)
        if decided == 77:
            meta = {"L": 16, "pairs": 8, "seed": 4, "nchol": 16, "accepted": accepted,
                    "proposal": [i, j, angle], "e_current": e_old, "e_proposal": e_new}
            break
        accept = e_new < e_old
        if not accept:
            cost = math.exp((e_old - e_new) / temp)
            accept = not (opt.acc.uniform() * (1 + cost) > cost)
        if accept:
            e_old = e_new
            opt.h, opt.eri, opt.e, opt.c = h2, e2, e_new, c_new
            accepted.append([i, j, angle])
        decided += 1
        temp *= p.change_temp
        max_angle *= p.change_angle
    with open(os.path.join(OUT, f"{name}.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print(name, json.dumps(meta)[:300])


# Determinant-list CI (FCI_File): the reference's own test cases. BeH2 STO-3G with
# the full 1225-determinant list of tests/data/fci_beh2_sto-3gdeterminants.dat
# (TestDensity.cpp), Be cc-pVDZ with the 100-determinant GKCI list (TestDetFile.cpp:
# E0 = -14.5951673370889), and the 70-orbital Be case of Testmp.cpp (E0 =
# -14.346369472944886), which needs 128-bit strings: the reference build here has
# 64-bit strings, so for it the pin is the known answer (and the oracle's 128-bit
# restatement), not the reference CRS. Integrals are stored as their canonical
# nonzero elements (p>=q, r>=s, pq>=rs) and the one-body upper triangle.
DETS_CASES = {
    "beh2": ("beh2_sto3g_1_5.dat", "fci_beh2_sto-3gdeterminants.dat", None),
    "be_gkci": ("Be_ccpVDZ.dat", "GKCI_Be_cntSp_cc-pVDZ_0100.txt", -14.5951673370889),
    "be70": ("mpbe5zmatrixelements.dat", "mpbe5zcut70determinants.dat", -14.346369472944886),
}


def sparse_integrals(ints):
    L = ints.L
    idx = np.argwhere(ints.eri != 0)
    p, q, r, s = idx.T
    keep = (p >= q) & (r >= s) & ((p * L + q) >= (r * L + s))
    hi = np.argwhere(np.triu(ints.h) != 0)
    return {"eri_idx": idx[keep].astype(np.uint8), "eri_val": ints.eri[tuple(idx[keep].T)],
            "h_idx": hi.astype(np.uint8), "h_val": ints.h[tuple(hi.T)]}


def read_det_file(path, words):
    up, down = [], []
    for line in open(path):
        if "#" in line or "|" not in line:
            continue
        a, b = line.strip().split("|")
        for s, out in ((a, up), (b, down)):
            v = int(s, 2)
            out.extend([(v >> (64 * w)) & ((1 << 64) - 1) for w in range(words)])
    return np.array(up, np.uint64), np.array(down, np.uint64)


def case_dets(name: str):
    out, meta = {}, {}
    for tag, (hf, df, known) in DETS_CASES.items():
        ints = O.ref_read_file(os.path.join(O.REF_ROOT, "tests", "data", hf))
        words = 1 if ints.L <= 64 else 2
        up, dn = read_det_file(os.path.join(O.REF_ROOT, "tests", "data", df), words)
        m_or = O.build_dets(ints, up, dn, words)
        e_or, _ = O.lowest_eigenpair(m_or)
        rec = {"L": ints.L, "nup": ints.nup, "ndown": ints.ndown, "econst": ints.econst, "words": words,
               "dim": m_or.n, "nnz": m_or.nnz, "crs_sha256": crs_sha256(m_or), "e0_oracle": e_or + ints.econst,
               "source": f"tests/data/{hf} + tests/data/{df}"}
        if known is not None:
            rec["e0_known_answer"] = known
        if words == 1:
            r = O.RefCI(O.FCI, filename=os.path.join(O.REF_ROOT, "tests", "data", hf),
                        det_file=os.path.join(O.REF_ROOT, "tests", "data", df))
            m = r.crs()
            ru, rd = r.dets()
            assert np.array_equal(ru, up) and np.array_equal(rd, dn), "reference list differs from the parse"
            e, c = O.lowest_eigenpair(m, v0=np.random.default_rng(12345).standard_normal(m.n))
            rec.update({"crs_sha256_reference": crs_sha256(m), "e0_reference": e + ints.econst})
            if tag == "beh2":  # DensFILE RDMs of the reference (TestDensity.cpp compares them with DensFCI)
                (r1, aa, ab, bb), ed = r.density(ints.L, e, c)
                out.update({f"{tag}_c": c, f"{tag}_rdm1": r1, f"{tag}_aa": aa, f"{tag}_ab": ab, f"{tag}_bb": bb})
                rec["dens_energy_reference"] = ed
            r.close()
        meta[tag] = rec
        out.update({f"{tag}_up": up, f"{tag}_down": dn})
        out.update({f"{tag}_{k}": v for k, v in sparse_integrals(ints).items()})
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **out)
    with open(os.path.join(OUT, f"{name}.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print(name, json.dumps(meta, indent=1))


# Text formats: the reference's own CI-vector blocks (OutputSFFCI / OutputSFDOCI /
# OutputSFFCI_File::print_ci_vec) and RDM dumps (print_one_rdm / print_two_rdm) for
# the BeH2 STO-3G eigenvectors stored in beh2_sto3g.npz, written by the reference.
def case_formats(name: str):
    import tempfile
    meta = json.load(open(os.path.join(OUT, "beh2_sto3g.json")))
    arr = np.load(os.path.join(OUT, "beh2_sto3g.npz"))
    path = os.path.join(O.REF_ROOT, "tests", "data", "beh2_sto3g_1_5.dat")
    det = os.path.join(O.REF_ROOT, "tests", "data", "fci_beh2_sto-3gdeterminants.dat")
    out = {}
    with tempfile.TemporaryDirectory() as td:
        for tag, method, nauw in (("fci", O.FCI, 1e-4), ("doci", O.DOCI, -1.0)):
            r = O.RefCI(method, filename=path)
            e = meta[tag]["e0"] - meta["econst"]
            c = arr[f"{tag}_c"]
            r.print_civec(e, c, nauw, os.path.join(td, "v.txt"))
            out[f"civec_{tag}"] = open(os.path.join(td, "v.txt")).read()
            r.print_rdm(e, c, os.path.join(td, "r.txt"))
            out[f"rdm_{tag}"] = open(os.path.join(td, "r.txt")).read()
            out[f"nauw_{tag}"] = nauw
            r.close()
        # FCI_File over the reference's BeH2 list: its own eigenvector
        r = O.RefCI(O.FCI, filename=path, det_file=det)
        m = r.crs()
        e, c = O.lowest_eigenpair(m, v0=np.random.default_rng(12345).standard_normal(m.n))
        r.print_civec(e, c, 1e-4, os.path.join(td, "v.txt"))
        out["civec_dets"] = open(os.path.join(td, "v.txt")).read()
        out["nauw_dets"] = 1e-4
        np.save(os.path.join(OUT, "formats_dets_c.npy"), c)
        out["e0_dets"] = e + meta["econst"]
        r.close()
    with open(os.path.join(OUT, f"{name}.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(name, {k: (len(v) if isinstance(v, str) else v) for k, v in out.items()})


# RDMs of the FP64 ground state where the reference's DensFCI (O(dim^2) pair loop)
# is out of reach (c1: 853,776 determinants): the lowest eigenpair of the CRS
# (the oracle's, bit-identical to the reference CRS by the SHA-256 of case_config)
# from ARPACK at the reference's settings, and its RDMs from the oracle's
# restatement of DensFCI (pinned to the reference's DensFCI on BeH2, c0 and c4).
def case_state_rdm(name: str):
    import scipy.sparse.linalg as sla
    cfg = CONFIGS[name]
    method = O.FCI if cfg["method"] == "FCI" else O.DOCI
    ints = config_integrals(name)
    meta = json.load(open(os.path.join(OUT, f"{name}.json")))
    m = O.build_upper(method, ints)
    assert crs_sha256(m) == meta["crs_sha256"], "oracle CRS differs from the reference CRS"
    n = m.n
    op = sla.LinearOperator((n, n), matvec=lambda x: O.sym_mvprod(m, x, threaded=True), dtype=np.float64)
    w, v = sla.eigsh(op, k=1, which="SA", ncv=42, tol=0, maxiter=3 * n,
                     v0=np.random.default_rng(12345).standard_normal(n))
    del m
    c = v[:, 0] / np.linalg.norm(v[:, 0])
    r1, aa, ab, bb = O.rdm(method, ints.L, ints.nup, ints.ndown, c)
    meta["state_rdm"] = {"e0": float(w[0]) + ints.econst,
                         "source": "ARPACK (which='SA', ncv=42, tol=0) on the reference CRS; oracle DensFCI"}
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), rdm1=r1, aa=aa, ab=ab, bb=bb)
    with open(os.path.join(OUT, f"{name}.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print(name, json.dumps(meta["state_rdm"]))


# Orbital rotation: the reference's OrbitalTransform::fillHamCI (with the real
# dgemm of oracle/ref_shims) applied to seeded integrals with U = exp(kappa),
# kappa antisymmetric with N(0, sigma) entries (the served stream's rotation is
# sigma = 0.05; sigma = 0.6 mixes the orbitals strongly). Cases: L=8 (the 4a4b
# FCI integrals) and L=10 (the 5a5b served-stream base integrals).
ROTATE_CASES = {"L8": ("c0", 0.6, 21), "L10": ("c4", 0.05, 22), "L10_strong": ("c4", 0.6, 23)}


def case_rotate(name: str):
    import scipy.linalg as sl
    out, meta = {}, {}
    for tag, (cfg_name, sigma, seed) in ROTATE_CASES.items():
        ints = config_integrals(cfg_name)
        L = ints.L
        rng = np.random.default_rng(seed)
        k = np.triu(rng.normal(0.0, sigma, (L, L)), 1)
        U = sl.expm(k - k.T)
        h, eri = O.ref_rotate(ints, U)
        out.update({f"{tag}_U": U, f"{tag}_h": h, f"{tag}_eri": eri})
        meta[tag] = {"config": cfg_name, "sigma": sigma, "seed": seed, "L": L,
                     "integrals_sha": ints.checksum()}
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **out)
    with open(os.path.join(OUT, f"{name}.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print(name, json.dumps(meta))


# CPU baseline calibration: the reference (oracle/_ref) against the oracle's
# restatement (the port that runs on hosts without the reference tree), on the same
# host with the same thread count, and ARPACK's matvec count at the reference's
# settings (SparseMatrix_CRS::arpackDiagonalize, SparseMatrix_CRS.cpp:360-481:
# which='SA', ncv=42, tol=0, maxiter=3n) driving the reference's own serial
# Sym::mvprod. For c0/c4/c2 the whole reference solve (constructor + ARPACK loop) is
# also timed end to end.
def _median_time(f, reps: int) -> float:
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        f()
        ts.append(time.perf_counter() - t0)
    return float(np.median(ts))


def case_calibration(name: str, cfgs=("c0", "c4", "c2", "c1")):
    import platform

    import scipy.sparse.linalg as sla
    threads = len(os.sched_getaffinity(0))
    os.environ["OMP_NUM_THREADS"] = str(threads)
    path = os.path.join(OUT, f"{name}.json")
    meta = json.load(open(path)) if os.path.exists(path) else {}
    meta.update({"host": platform.machine(), "cpu": platform.processor() or platform.machine(), "threads": threads})
    for cfg_name in cfgs:
        cfg = CONFIGS[cfg_name]
        method = O.FCI if cfg["method"] == "FCI" else O.DOCI
        ints = config_integrals(cfg_name)
        t0 = time.perf_counter()
        r = O.RefCI(method, ints=ints)
        t_ref_build = time.perf_counter() - t0
        n = int(r.lib.ref_ci_dim(r.h))
        t0 = time.perf_counter()
        off, col, val = O.build_rows(method, ints, 0, n)
        t_port_build = time.perf_counter() - t0
        x = np.random.default_rng(0).standard_normal(n)
        y = np.zeros(n)
        reps = 3 if n > 200000 else 10
        t_port_mv = _median_time(lambda: O.sym_mvprod_rows(0, off, col, val, x, y), reps)
        del off, col, val
        t_ref_mv = _median_time(lambda: r.mvprod(x), reps)
        count = [0]

        def mv(v):
            count[0] += 1
            return r.mvprod(v)

        v0 = np.random.default_rng(12345).standard_normal(n)
        op = sla.LinearOperator((n, n), matvec=mv, dtype=np.float64)
        t0 = time.perf_counter()
        w, _ = sla.eigsh(op, k=1, which="SA", ncv=min(42, n - 1), tol=0, maxiter=3 * n, v0=v0)
        t_eig = time.perf_counter() - t0
        r.close()
        rec = {"dim": n, "ref_build_s": t_ref_build, "port_build_s": t_port_build,
               "ref_mvprod_s": t_ref_mv, "port_mvprod_s": t_port_mv,
               "build_ratio_ref_over_port": t_ref_build / t_port_build,
               "mvprod_ratio_ref_over_port": t_ref_mv / t_port_mv,
               "arpack_matvecs": count[0], "arpack_s": t_eig, "e0": float(w[0]) + ints.econst,
               "ref_solve_s": t_ref_build + t_eig}
        meta[cfg_name] = rec
        with open(path, "w") as f:
            json.dump(meta, f, indent=1)
        print(cfg_name, json.dumps(rec), flush=True)


if __name__ == "__main__":
    names = sys.argv[1:] or ["beh2_sto3g", "c0", "c4", "orbopt", "dets", "formats", "warm_chain"]
    for nm in names:
        if nm == "c1_state":
            case_state_rdm("c1")
        elif nm == "rotate":
            case_rotate(nm)
        elif nm == "calibration":
            case_calibration(nm)
        elif nm.startswith("calibration:"):
            case_calibration("calibration", tuple(nm.split(":", 1)[1].split(",")))
        elif nm == "formats":
            case_formats(nm)
        elif nm == "orbopt":
            case_orbopt(nm)
        elif nm == "warm_chain":
            case_warm_chain(nm)
        elif nm == "dets":
            case_dets(nm)
        elif nm == "beh2_sto3g":
            case_file(nm, "beh2_sto3g_1_5.dat")
        elif nm == "be_ccpvdz":
            case_file(nm, "Be_ccpVDZ.dat")
        else:
            case_config(nm, rdm=nm in ("c0", "c4", "c2"))
