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
