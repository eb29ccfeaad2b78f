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


@pytest.mark.parametrize("name,fixture", [("scf-small-24x12x20-12at-2k-ns40", "xc_cyclic.npz"),
                                          ("scf-small-helical-24x12x16-8at-2k-ns28", "xc_helical.npz")],
                         ids=["cyclic", "helical"])
def test_xc_golden(name, fixture):
    ref = np.load(GOLD / fixture)
    out = G.xc_case(name)
    assert sorted(out) == sorted(ref.files)
    for k in ref.files:
        assert np.max(np.abs(out[k] - ref[k])) <= 1e-13 * np.max(np.abs(ref[k])), k


def test_gga_deck_oracle_record():
    """The oracle's tight SCF of the GGA_wrong_SG15 set-up: converged to its tolerance, for the
    deck's functional, with the printed energy of the saved set-up."""
    from golden.make_deck_fixtures import load
    rec = json.loads((GOLD / "deck_GGA_wrong_SG15_oracle.json").read_text())
    S, _, _, e_ref = load("GGA_wrong_SG15")
    assert rec["xc"] == S.extra["xc"] == "GGA_PBE"
    assert rec["history"][-1][2] <= rec["scf_tol"]
    assert rec["printed_free_energy_per_atom"] == e_ref
    assert abs(rec["history"][-1][1] - rec["free_energy_per_atom"]) < 1e-12
    assert abs(rec["free_energy_per_atom"] - e_ref) < 3e-6


@pytest.mark.slow
@pytest.mark.parametrize("name,fixture", [("scf-small-24x12x20-12at-2k-ns40", "scf_small.json"),
                                          ("scf-small-helical-24x12x16-8at-2k-ns28", "scf_small_helical.json"),
                                          ("scf-small-24x12x20-12at-2k-ns40", "scf_small_fd.json"),
                                          ("scf-small-24x12x20-12at-2k-ns40", "scf_small_gga.json"),
                                          ("scf-small-helical-24x12x16-8at-2k-ns28", "scf_small_helical_gga.json"),
                                          ("scf-small-24x12x20-12at-2k-ns40", "scf_small_pz.json")])
def test_scf_golden(name, fixture):
    ref = json.loads((GOLD / fixture).read_text())
    out = G.scf_small(name, fermi_dirac=ref.get("smearing") == "fermi-dirac", xc=ref.get("xc", "LDA_PW"))
    assert out["n_scf"] == ref["n_scf"]
    assert abs(out["E_per_atom"] - ref["E_per_atom"]) < 1e-10
    for a, b in zip(out["EigVal"], ref["EigVal"]):
        assert np.max(np.abs(np.array(a) - np.array(b))) < 1e-8
