"""The oracle reproduces the committed golden fixtures (no GPU).

The fixtures in ``tests/golden/`` were written by ``tests/golden/make_golden.py``; a mismatch
means the oracle (or the synthetic-system generator it runs on) changed.
"""
import json
from pathlib import Path

import numpy as np
import pytest

import golden.make_golden as G

GOLD = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("name", ["cyclic", "helical"])
def test_operators_golden(name):
    ref = np.load(GOLD / f"operators_{name}.npz")
    out = G.operator_case(name)
    assert sorted(out) == sorted(ref.files)
    for k in ref.files:
        assert np.max(np.abs(out[k] - ref[k])) <= 1e-12 * np.max(np.abs(ref[k])), k


@pytest.mark.parametrize("name", ["cyclic", "helical"])
def test_eig_golden(name):
    ref = json.loads((GOLD / f"eig_{name}.json").read_text())
    out = G.eig_case(name)
    for rb, ob in zip(ref["blocks"], out["blocks"]):
        for rs, os_ in zip(rb["steps"], ob["steps"]):
            assert np.max(np.abs(np.array(rs) - np.array(os_))) < 1e-10
        assert np.max(np.abs(np.array(rb["dense_lowest"]) - np.array(ob["dense_lowest"]))) < 1e-10


def test_poisson_golden():
    ref = np.load(GOLD / "poisson_cyclic.npz")
    out = G.poisson_case()
    assert float(out["relres"]) <= 1e-10
    assert np.max(np.abs(out["phi"] - ref["phi"])) <= 1e-9 * np.max(np.abs(ref["phi"]))


@pytest.mark.slow
@pytest.mark.parametrize("name,fixture", [("scf-small-24x12x20-12at-2k-ns40", "scf_small.json"),
                                          ("scf-small-helical-24x12x16-8at-2k-ns28", "scf_small_helical.json"),
                                          ("scf-small-24x12x20-12at-2k-ns40", "scf_small_fd.json")])
def test_scf_golden(name, fixture):
    ref = json.loads((GOLD / fixture).read_text())
    out = G.scf_small(name, fermi_dirac=ref.get("smearing") == "fermi-dirac")
    assert out["n_scf"] == ref["n_scf"]
    assert abs(out["E_per_atom"] - ref["E_per_atom"]) < 1e-10
    for a, b in zip(out["EigVal"], ref["EigVal"]):
        assert np.max(np.abs(np.array(a) - np.array(b))) < 1e-8
