"""The C++ façade (include/ciflow_gb300/ciflow.hpp) drives the GPU path with
CIFlow's class and method names: a driver written like the reference's
TestDOCI.cpp / TestDensity.cpp is compiled with g++ against it and run."""
import json
import os
import subprocess

import numpy as np
import pytest

import oracle as O
from tests.helpers import beh2_integrals

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
pytestmark = pytest.mark.gpu


def test_cpp_facade_driver(tmp_path):
    ints, meta, _ = beh2_integrals()
    data = tmp_path / "beh2.bin"
    with open(data, "wb") as f:
        f.write(np.array([ints.L, ints.nup, ints.ndown], np.int32).tobytes())
        f.write(np.array([ints.econst], np.float64).tobytes())
        f.write(np.ascontiguousarray(ints.h).tobytes())
        f.write(np.ascontiguousarray(ints.eri).tobytes())
    exe = tmp_path / "test_facade"
    lib = os.path.join(ROOT, "ciflow_gb300", "_lib")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "test_facade.cpp"), "-o", str(exe), "-L", lib, "-lcigpu",
                    f"-Wl,-rpath,{lib}"], check=True)
    out = subprocess.run([str(exe), str(data), str(tmp_path)], check=True, capture_output=True, text=True).stdout
    r = json.loads(out.strip().splitlines()[-1])
    # reference tests/src/TestDOCI.cpp:31
    assert abs(r["e_doci"] - (-15.225362047972723)) < 1e-10
    assert abs(r["e_fci"] - meta["fci"]["e0"]) < 1e-9
    assert abs(r["e_dens"] - r["e_fci"]) < 1e-9  # TestDensity.cpp:57
    assert abs(r["e_fci_mixed"] - meta["fci"]["e0"]) < 1e-6
    assert r["dim_fci"] == meta["fci"]["dim"] and r["nnz_upper"] == meta["fci"]["nnz"]
    ref = O.build_upper(O.FCI, ints)
    assert r["h00"] == ref.val[0]
    ysum = float(np.sum(O.sym_mvprod(ref, np.ones(ref.n))))
    assert abs(r["ysum"] - ysum) < 1e-9 * max(1.0, abs(ysum))
    # psi4 dump round trip, FCI_File / CI_Big over the full list, text dumps, optimisers
    assert r["psi4_round_trip"] == 1
    assert r["dim_file"] == meta["fci"]["dim"]
    assert abs(r["e_file"] - r["e_fci"]) < 1e-9 and abs(r["e_big"] - r["e_fci"]) < 1e-9
    assert abs(r["e_file_dens"] - r["e_fci"]) < 1e-9  # DensFILE, as TestDensity.cpp
    assert (tmp_path / "fci_vec.txt").read_text().count("\n") > 10
    assert "#THE 2RDM:" in (tmp_path / "fci_rdm.txt").read_text()
    assert r["e_sa_opt"] <= r["e_opt_start"] + 1e-10 and abs(r["e_sa"] - r["e_sa_opt"]) < 1e-8
    assert r["e_lm"] <= r["e_sa"] + 1e-8 and abs(r["e_lm_cim"] - r["e_lm"]) < 1e-8

