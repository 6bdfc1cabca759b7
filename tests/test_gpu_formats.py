"""Text dumps of device results through the Python mirror: the CI vector and the RDMs
of a BeH2 STO-3G solve on the device, in the reference's output format, against the
text the reference wrote for its own eigenvector (tests/golden/formats.json): the same
determinants and elements, values within 1e-9 (the eigenvector up to its sign)."""
import json
import os

import numpy as np
import pytest

from ciflow_gb300.ciflow import DOCI, FCI, FCI_File, Hamiltonian

from .helpers import GOLDEN, beh2_integrals, dets_case

pytestmark = pytest.mark.gpu


def entries(text):
    """{index-tuple: value} of the data lines of a dump."""
    out = {}
    for line in text.splitlines():
        if not line or line.startswith("#"):
            continue
        f = line.split()
        out[tuple(f[:-1])] = float(f[-1])
    return out


@pytest.fixture(scope="module")
def formats():
    with open(os.path.join(GOLDEN, "formats.json")) as f:
        return json.load(f)


def compare(ours, ref, signed):
    """Values within 1e-9 over the entries of both dumps; an entry printed by one side
    only is rounding noise below 1e-10."""
    a, b = entries(ours), entries(ref)
    s = 1.0
    if not signed:
        k = max(b, key=lambda t: abs(b[t]))
        s = np.sign(a[k]) * np.sign(b[k])
    for k in a.keys() | b.keys():
        assert a.get(k, 0.0) * s == pytest.approx(b.get(k, 0.0), abs=1e-9), k
    # elements zero by symmetry are printed when their rounding noise reaches 1e-12
    for k in a.keys() ^ b.keys():
        assert abs(a.get(k, 0.0)) < 1e-10 and abs(b.get(k, 0.0)) < 1e-10, k


@pytest.mark.parametrize("tag", ["fci", "doci"])
def test_device_dumps(tmp_path, formats, tag):
    ints = beh2_integrals()[0]
    cim = (FCI if tag == "fci" else DOCI)(Hamiltonian.from_integrals(ints))
    cim.solve(tol=1e-11)
    v, r = str(tmp_path / "v.txt"), str(tmp_path / "r.txt")
    cim.print_ci_vec(v, formats[f"nauw_{tag}"])
    text = open(v).read()
    compare(text[text.index("#CIMETHOD"):], formats[f"civec_{tag}"], signed=False)
    cim.print_rdm(r)
    compare(open(r).read(), formats[f"rdm_{tag}"], signed=True)


def test_device_dump_of_a_list(tmp_path, formats):
    ints, up, down, words, meta = dets_case("beh2")
    cim = FCI_File(Hamiltonian.from_integrals(ints), up=up, down=down, words=words)
    cim.list_name = "fcibeh2sto3gdeterminants"
    cim.solve(tol=1e-11)
    v = str(tmp_path / "v.txt")
    cim.print_ci_vec(v, formats["nauw_dets"])
    text = open(v).read()
    assert text[text.index("#CIMETHOD"):].splitlines()[0] == formats["civec_dets"].splitlines()[0]
    compare(text[text.index("#CIMETHOD"):], formats["civec_dets"], signed=False)
