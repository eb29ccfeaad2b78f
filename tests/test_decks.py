"""The deck loader against the reference's own decks and outputs (no GPU).

``cyclix_msparc_gb300.deck`` reads a reference deck (.inpt, .ion, .psp8) and builds the
pseudocharges, the self and correction energy, the pseudocharge radii and the psp8 projectors.
Where the deck's .out was written by the committed reference code from the same input (the
parameters it prints match the .inpt), the numbers it printed must come out again:

* ``Self and correction energy`` (E_corr - Eself, src/electronicGroundState.m:95) within 1e-8 Ha
  (the .out prints 11 significant digits);
* ``Pseudocharge radii`` to the two decimals printed;
* the Chebyshev degree, the number of states and the number of symmetry-reduced Bloch points.

Several .out files were written from parameters other than those in today's .inpt; they print
the parameters they ran with, and the deck is loaded with those (tests/Cyclix/CNT_chiral/C.out,
for example, ran on FD_GRID 120 61 8 against 140 70 15 in its .inpt).  Pseudocharge radii are
compared only where the .out was written by the committed radius rule (rb_y = acos(1 - rb_z^2 /
(2 r^2)) + tau rb_z / 2); the energies do not depend on the radii once b has converged.
Decks whose .out does not describe a run of today's deck files are not listed: the relaxation
deck tests/Cyclix/CNT_relax (its first step ran on another cell length), and H2O_tube and the GGA
MoS2 tubes (not traced).

The full SCF of six decks (cyclic and helical; LDA_PW, LDA_PZ and GGA_PBE; Gaussian and
Fermi-Dirac) and their forces are pinned by tests/golden/pin_decks.py, which writes
tests/golden/deck_pins.json (checked below).  The reference tree is read from the directory named by the
CYCLIX_REFERENCE environment variable; the tests that need it skip when it is unset.
"""
import json
import os
import re

import numpy as np
import pytest

# root of the reference project (the directory holding src/ and tests/), from the environment
REF = os.environ.get("CYCLIX_REFERENCE", "")
HERE = os.path.dirname(os.path.abspath(__file__))

# (deck, compare radii): cyclic and helical (CNT_chiral, phonon/Si_1), one and two species
DECKS = [("LDA_CNT/C.inpt", True), ("GGA_CNT_sg15/C.inpt", True), ("tests/MoS2/MoS2.inpt", True),
         ("tests/Cyclix/CNT_ABINITmatch/C.inpt", False), ("tests/Cyclix/CNT_chiral/C.inpt", False),
         ("tests/phonon/Si_1/Si.inpt", False), ("tests/phonon/Si_2/Si.inpt", False)]
# free energy per atom, oracle SCF vs the .out, by how far each reference run converged:
# LDA_CNT and GGA_CNT_sg15 stopped at SCF error ~6e-5 (TOL_SCF 1e-4), phonon/Si_2 below 1e-5,
# CNT_chiral, phonon/Si_1 (helical) and CNT_ABINITmatch at ~1e-6
PIN_TOL = {"LDA_CNT/C.inpt": 1e-5, "GGA_CNT_sg15/C.inpt": 1e-5, "GGA_wrong_SG15/C.inpt": 1e-5,
           "tests/Cyclix/CNT_chiral/C.inpt": 1e-6,
           "tests/phonon/Si_1/Si.inpt": 1e-6, "tests/phonon/Si_2/Si.inpt": 2e-6,
           "tests/Cyclix/CNT_ABINITmatch/C.inpt": 1e-6}


def _out(inpt):
    return open(os.path.splitext(os.path.join(REF, inpt))[0] + ".out").read()


def _need(inpt):
    if not REF:
        pytest.skip("CYCLIX_REFERENCE (the reference project root) is not set")
    if not os.path.exists(os.path.join(REF, inpt)):
        pytest.skip("reference decks are not present under CYCLIX_REFERENCE")


def _ran_with(inpt):
    from golden.pin_decks import ran_with
    return ran_with(os.path.join(REF, inpt))


@pytest.fixture(scope="module")
def loaded():
    from cyclix_msparc_gb300.deck import load_deck
    cache = {}

    def get(inpt):
        if inpt not in cache:
            cache[inpt] = load_deck(os.path.join(REF, inpt), for_scf=False, overrides=_ran_with(inpt))
        return cache[inpt]
    return get


@pytest.mark.parametrize("inpt,radii_rule", DECKS)
def test_self_and_correction_energy_and_radii(inpt, radii_rule, loaded):
    _need(inpt)
    d = loaded(inpt)
    txt = _out(inpt)
    ref = float(re.search(r"Self and correction energy\s*:\s*([-+0-9.Ee]+)", txt).group(1))
    assert abs((d.S.E_corr - d.S.Eself) - ref) <= 1e-8, (d.S.E_corr - d.S.Eself, ref)
    radii = re.findall(r"Pseudocharge radii of atom type (\d+)\s*:\s*([0-9.]+)\s+([0-9.]+)\s+([0-9.]+)", txt)
    assert len(radii) == len(d.rb)
    if radii_rule:
        for (t, *r), rb in zip(radii, d.rb):
            assert ["%.2f" % v for v in rb] == r, (t, rb, r)
    # the pseudocharge integrates to minus the valence charge
    assert abs(float(d.S.W @ d.S.b) + d.Nelectron) < 1e-4 * d.Nelectron


@pytest.mark.parametrize("inpt,radii_rule", DECKS)
def test_defaults_and_bloch_points(inpt, radii_rule, loaded):
    _need(inpt)
    d = loaded(inpt)
    txt = _out(inpt)
    assert int(re.search(r"CHEB_DEGREE:\s*(\d+)", txt).group(1)) == d.S.npl
    assert int(re.search(r"NSTATES:\s*(\d+)", txt).group(1)) == d.S.Nev
    m = re.search(r"Number of symmetry adapted k-points:\s*(\d+)", txt)
    if m:
        assert int(m.group(1)) == d.S.tnkpt
        assert abs(d.S.wkpt.sum() - 1.0) < 1e-14


def test_psp8_reader_against_the_file_text():
    inpt = "LDA_CNT/C.inpt"
    _need(inpt)
    from cyclix_msparc_gb300.deck import read_psp8
    path = os.path.join(REF, "LDA_CNT", "C.psp8")
    p = read_psp8(path)
    lines = open(path).read().splitlines()
    assert p.Z == float(lines[1].split()[1]) and p.lmax == int(lines[2].split()[2]) and p.lloc == 4
    assert p.r.shape == (int(lines[2].split()[4]),) and p.r[0] == 0.0
    # KB energies: the numbers after the l on each projector block header
    heads = [ln.split() for ln in lines if re.match(r"^\s{3}[0-9]\s{3,}", ln) and len(ln.split()) == 1 + p.nproj[0]]
    assert np.allclose(p.gamma[0], [float(v) for v in heads[0][1:]])
    assert np.allclose(p.gamma[1], [float(v) for v in heads[1][1:]])
    # projectors divided by r, the r = 0 row copied from the next one
    assert np.array_equal(p.proj[1][0], p.proj[1][1])
    # the valence-density column over 4 pi (src/readPseudopot.m:68-72; only its shape matters, since
    # the density guess is rescaled to the electron count)
    assert p.rho_iso.max() > 0 and p.rho_iso.shape == p.r.shape


def test_projector_layout(loaded):
    inpt = "LDA_CNT/C.inpt"
    _need(inpt)
    d = loaded(inpt)
    S = d.S
    p = d.psps[0]
    angnum = sum(int(p.nproj[l]) * (2 * l + 1) for l in range(p.lmax + 1))
    for A in S.Atom:
        assert A.angnum == angnum and A.gamma_Jl.shape == (angnum,)
        for img in A.rcImage:
            assert img.Chi_mat.shape == (img.rc_n_nodes, angnum)
            assert np.all(np.isfinite(img.Chi_mat))
            assert img.rc_pos.min() >= 1 and img.rc_pos.max() <= S.N
    # gamma_Jl ordered (l, projector, m): l = 0 projectors once each, l = 1 three times each
    g = S.Atom[0].gamma_Jl
    assert np.allclose(g[:2], p.gamma[0]) and np.allclose(g[2:5], p.gamma[1][0]) and np.allclose(g[5:8], p.gamma[1][1])


@pytest.mark.parametrize("deck,tol", PIN_TOL.items())
def test_scf_pin_record(deck, tol):
    """The oracle SCF on a reference deck reproduces the free energy the reference printed (the
    record written by tests/golden/pin_decks.py; the reference numbers it holds are re-read from
    the .out here where the reference tree exists)."""
    path = os.path.join(HERE, "golden", "deck_pins.json")
    recs = json.load(open(path)) if os.path.exists(path) else {}
    if deck not in recs:
        pytest.skip("no SCF pin record for this deck")
    rec = recs[deck]
    if REF and os.path.exists(os.path.join(REF, deck)):
        txt = _out(deck)
        ref = float(re.search(r"Free energy per atom\s*:\s*([-+0-9.Ee]+)", txt).group(1))
        assert rec["reference"]["free_energy_per_atom"] == ref
    assert rec["oracle"]["n_scf"] < 60
    assert abs(rec["diff_free_energy_per_atom"]) <= tol, rec["diff_free_energy_per_atom"]


def test_split_projector_columns_is_the_same_operator(loaded):
    """psp8 atoms with 8 projector columns go to the GPU library as two 4-column atoms at the same
    position (the kernels hold 4); the KB term is a sum over columns, so H is unchanged (checked
    with the oracle H at a Bloch point with phases, nu = 2)."""
    inpt = "LDA_CNT/C.inpt"
    _need(inpt)
    import copy
    from cyclix_msparc_gb300.cychel import split_projector_columns
    from oracle import cychel_ops as O
    d = loaded(inpt)
    S = d.S
    atoms, origin = split_projector_columns(S.Atom, 4)
    assert len(atoms) == 2 * len(S.Atom) and all(A.angnum == 4 for A in atoms)
    assert origin == [J for J in range(len(S.Atom)) for _ in range(2)]
    S2 = copy.copy(S)
    S2.Atom, S2.Atoms = atoms, S.Atoms[origin]
    rng = np.random.default_rng(3)
    X = rng.standard_normal((S.N, 3)) + 1j * rng.standard_normal((S.N, 3))
    V = S.rho_at
    for k in (S.kptgrid[0], S.kptgrid[1]):
        Y1 = O.Hamiltonian(S, k, V)(X)
        Y2 = O.Hamiltonian(S2, k, V)(X)
        assert np.max(np.abs(Y1 - Y2)) <= 1e-13 * np.max(np.abs(Y1))
    # atoms that fit are passed through unchanged
    same, org = split_projector_columns(atoms, 4)
    assert same == atoms and org == list(range(len(atoms)))


# forces, oracle vs the .static file: the helical decks' reference runs converged to ~1e-6, the
# LDA_CNT and GGA_CNT_sg15 runs stopped at SCF error ~6e-5 (forces are first order in the density
# error)
# GGA_wrong_SG15 and GGA_CNT_sg15 are the same deck run twice; the committed GGA potential
# (src/exchangeCorrelationPotential.m:362, scalar gradient operators in the divergence) matches the
# first, while the second's forces follow the commented-out vector divergence of :361
FORCE_TOL = {"tests/Cyclix/CNT_chiral/C.inpt": 2e-5, "tests/phonon/Si_1/Si.inpt": 2e-5, "tests/phonon/Si_2/Si.inpt": 2e-5,
             "tests/Cyclix/CNT_ABINITmatch/C.inpt": 2e-5,
             "LDA_CNT/C.inpt": 2e-4, "GGA_wrong_SG15/C.inpt": 2e-4}


@pytest.mark.parametrize("deck,tol", FORCE_TOL.items())
def test_force_pin_record(deck, tol):
    """Drift-free atomic forces of the oracle (oracle/forces.py, src/atomicForce.m) at the converged
    SCF of a deck against the forces the reference printed in the deck's .static file."""
    path = os.path.join(HERE, "golden", "deck_pins.json")
    recs = json.load(open(path)) if os.path.exists(path) else {}
    rec = recs.get(deck)
    if not rec or rec.get("forces") is None:
        pytest.skip("no force record for this deck")
    F = np.array(rec["forces"])
    Fr = np.array(rec["reference"]["forces"])
    assert F.shape == Fr.shape
    assert np.max(np.abs(F - Fr)) <= tol, np.max(np.abs(F - Fr))


def test_deck_fixtures_rebuild_the_setup():
    """tests/golden/deck_<name>.npz rebuilds a consistent CyclixS: the atomic density guess holds
    the valence charge, and (where the reference tree is set) the fixture equals a fresh set-up."""
    from golden.make_deck_fixtures import DECKS, load
    for name, rel in DECKS.items():
        S, scf_tol, poisson_tol, e_ref = load(name)
        assert S.W.shape == (S.N,) and S.b.shape == (S.N,)
        assert abs(float(S.W @ S.rho_at) + S.NegCharge) < 1e-6 * abs(S.NegCharge)
        assert e_ref < 0 and 0 < scf_tol <= 1e-4
        if REF and os.path.exists(os.path.join(REF, rel)):
            from cyclix_msparc_gb300.deck import load_deck
            d = load_deck(os.path.join(REF, rel), overrides=_ran_with(rel))
            assert np.array_equal(d.S.b, S.b) and np.array_equal(d.S.rho_at, S.rho_at)
            assert sum(img.rc_pos.size for A in d.S.Atom for img in A.rcImage) == sum(
                img.rc_pos.size for A in S.Atom for img in A.rcImage)
