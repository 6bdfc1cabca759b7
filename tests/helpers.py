"""Shared helpers of the test suite (fixtures, hashing, builders)."""
import hashlib
import json
import os

import numpy as np

from ciflow_gb300.synthetic import Integrals, config_integrals

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_golden(name):
    with open(os.path.join(GOLDEN, name + ".json")) as f:
        meta = json.load(f)
    npz = os.path.join(GOLDEN, name + ".npz")
    return meta, (np.load(npz) if os.path.exists(npz) else None)


def beh2_integrals():
    meta, a = load_golden("beh2_sto3g")
    return Integrals(meta["L"], meta["nup"], meta["ndown"], meta["econst"], a["h"], a["eri"]), meta, a


def crs_sha256(row, col, val) -> str:
    """SHA-256 of a CRS in the reference layout (uint32 row, uint32 col, float64 val)."""
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(row, dtype=np.uint32).tobytes())
    h.update(np.ascontiguousarray(col, dtype=np.uint32).tobytes())
    h.update(np.ascontiguousarray(val, dtype=np.float64).tobytes())
    return h.hexdigest()


def integrals(name):
    return config_integrals(name)


def dets_case(tag):
    """A determinant-list golden case (tests/golden/dets.*): (Integrals, up, down, words, meta)."""
    import json
    import numpy as np
    from ciflow_gb300.synthetic import Integrals
    with open(os.path.join(GOLDEN, "dets.json")) as f:
        meta = json.load(f)[tag]
    g = np.load(os.path.join(GOLDEN, "dets.npz"))
    L = meta["L"]
    h = np.zeros((L, L))
    hi, hv = g[f"{tag}_h_idx"].astype(int), g[f"{tag}_h_val"]
    h[hi[:, 0], hi[:, 1]] = hv
    h[hi[:, 1], hi[:, 0]] = hv
    eri = np.zeros((L,) * 4)
    ei, ev = g[f"{tag}_eri_idx"].astype(int), g[f"{tag}_eri_val"]
    for p, q, r, s in ((0, 1, 2, 3), (1, 0, 2, 3), (0, 1, 3, 2), (1, 0, 3, 2),
                       (2, 3, 0, 1), (3, 2, 0, 1), (2, 3, 1, 0), (3, 2, 1, 0)):
        eri[ei[:, p], ei[:, q], ei[:, r], ei[:, s]] = ev
    ints = Integrals(L, meta["nup"], meta["ndown"], meta["econst"], h, eri)
    return ints, g[f"{tag}_up"], g[f"{tag}_down"], meta["words"], meta

