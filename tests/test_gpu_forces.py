"""GPU atomic-force pieces against the oracle (oracle/forces.py, src/atomicForce.m):
  * the nonlocal term (cx_nonlocal_force, src/atomicForce.m:254-300) on seeded psi and occupations
    of the small helical (twist 0.05 rad/bohr) and cyclic cells, both Bloch blocks, in FP64 and
    with complex64 blocks (the oracle then takes the same complex64-rounded psi), and on the
    CNT_chiral deck's psp8 projectors (8 columns per atom, passed as two 4-column atoms and summed
    back by the host);
  * the Cartesian gradient of a real field at k = 0 (cx_gradient, the S.grad_1..3 products).
Tolerances: forces 1e-10 relative to the largest component (FP64 products in another order);
gradient 1e-12 relative to the largest value."""
import numpy as np
import pytest

from cyclix_msparc_gb300.workloads import WORKLOADS, block_layout, initial_psi, make_system

pytestmark = pytest.mark.gpu
CELLS = ["scf-small-helical-24x12x16-8at-2k-ns28", "scf-small-24x12x20-12at-2k-ns40"]


def _inputs(S, blocks, prec):
    rng = np.random.default_rng(5)
    psis, occs = [], []
    for b, (_, _, n) in enumerate(blocks):
        psi = initial_psi(S.N, n, 11 + b)
        if prec == "mixed":
            psi = psi.astype(np.complex64).astype(np.complex128)
        psis.append(psi)
        occs.append(rng.uniform(0, 1, n))
    return psis, occs


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("name", CELLS, ids=["helical", "cyclic"])
def test_nonlocal_force_matches_oracle(name, prec):
    from oracle.forces import nonlocal_forces
    from cyclix_msparc_gb300.msparc import CyclixGPU
    wl = WORKLOADS[name]
    S = make_system(wl)
    blocks = block_layout(wl, S)
    psis, occs = _inputs(S, blocks, prec)
    wk = [0.5 + 0.25 * b for b in range(len(blocks))]
    g = CyclixGPU(S, blocks, prec)
    try:
        for b, psi in enumerate(psis):
            g.set_psi(b, psi)
        F = g.nonlocal_force(np.concatenate(occs), wk, 2.0)
    finally:
        g.close()
    ref = nonlocal_forces(S, [np.asarray(k, float) for (k, _, _) in blocks], wk, psis, occs, 2.0)
    assert np.max(np.abs(F - ref)) <= 1e-10 * np.max(np.abs(ref)), (F, ref)


def test_nonlocal_force_on_deck_projectors():
    """CNT_chiral (helical, twist 0.1636 rad/bohr, Gamma point): psp8 atoms of 8 projector columns."""
    from golden.make_deck_fixtures import load
    from oracle.forces import nonlocal_forces
    from cyclix_msparc_gb300.msparc import CyclixGPU
    S, _, _, _ = load("CNT_chiral")
    blocks = [(S.kptgrid[k].copy(), 0, S.Nev) for k in range(S.tnkpt)]
    psis, occs = _inputs(S, blocks, "fp64")
    g = CyclixGPU(S, blocks, "fp64")
    try:
        assert g.nl_origin.size > S.Atoms.shape[0]          # the atoms are split into 4-column parts
        for b, psi in enumerate(psis):
            g.set_psi(b, psi)
        F = g.nonlocal_force(np.concatenate(occs), S.wkpt, S.occfac)
    finally:
        g.close()
    ref = nonlocal_forces(S, [np.asarray(k, float) for (k, _, _) in blocks], S.wkpt, psis, occs, S.occfac)
    assert np.max(np.abs(F - ref)) <= 1e-10 * np.max(np.abs(ref)), (F, ref)


@pytest.mark.parametrize("name", CELLS, ids=["helical", "cyclic"])
def test_gradient_matches_oracle(name):
    from oracle.forces import bloch_gradients
    from cyclix_msparc_gb300.msparc import CyclixGPU
    wl = WORKLOADS[name]
    S = make_system(wl)
    u = np.random.default_rng(3).standard_normal(S.N)
    g = CyclixGPU(S, block_layout(wl, S), "fp64")
    try:
        D = g.gradient(u)
    finally:
        g.close()
    for d, G in enumerate(bloch_gradients(S, (0.0, 0.0, 0.0))):
        ref = (G @ u).real
        assert np.max(np.abs(D[:, d] - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_deck_forces_match_oracle_and_printed():
    """Whole drift-free forces of CNT_chiral (helical, Gamma point, psp8) after a GPU SCF in FP64
    (SCF error 1e-7, Poisson 1e-10): the local and correction terms through cx_field_projections
    with the host set-up, the nonlocal term through cx_nonlocal_force.  Against the oracle's
    atomic_forces on the same psi, phi and occupations within 1e-9 Ha/bohr, and against the forces
    the reference printed (tests/Cyclix/CNT_chiral/C.static, recorded in
    tests/golden/deck_pins.json) within 3e-6 Ha/bohr: the oracle's own SCF at the same tolerances is
    1.3e-6 Ha/bohr from them, and the GPU's converged density 6e-8 (relative) from the oracle's.
    phi is the SCF's own (Veff - Vxc[rho] of the converged last step): a cold cx_poisson solve of
    this cell to 1e-10 stops near a relative residual of 1e-6 after 2000 AAR iterations, which
    moves the local forces by 1.5e-4 Ha/bohr."""
    import json
    from pathlib import Path
    from golden.make_deck_fixtures import load_force_deck
    from oracle.forces import atomic_forces as oracle_forces
    from cyclix_msparc_gb300 import forces as PF
    from cyclix_msparc_gb300.msparc import CyclixGPU
    d, _, _, _ = load_force_deck("CNT_chiral")
    S = d.S
    pins = json.loads((Path(__file__).resolve().parent / "golden" / "deck_pins.json").read_text())
    printed = np.array(pins["tests/Cyclix/CNT_chiral/C.inpt"]["reference"]["forces"])
    setup = PF.local_force_setup(d)
    blocks = [(S.kptgrid[k].copy(), 0, S.Nev) for k in range(S.tnkpt)]
    g = CyclixGPU(S, blocks, "fp64")
    try:
        for b in range(len(blocks)):
            g.set_psi(b, initial_psi(S.N, S.Nev, 700 + b))
        res, EV, rho, V, hist = g.scf(S, scf_tol=1e-7, poisson_tol=1e-10, max_scf=80)
        assert res.converged == 1
        # the SCF's own phi: a converged cx_scf returns Veff = phi + Vxc[rho] of its last step
        phi = V - g.xc(rho, S.extra["xc"])[0]
        occ = PF.occupations(EV, res.lambda_f, S.bet, S.elec_T_type)
        F = PF.atomic_forces(g, setup, phi, occ, S.wkpt, S.occfac)
        psis = [g.get_psi(b) for b in range(len(blocks))]
    finally:
        g.close()
    off = np.concatenate([[0], np.cumsum([n for (_, _, n) in blocks])])
    Fo, _ = oracle_forces(d, psis, [occ[off[b]:off[b + 1]] for b in range(len(blocks))], phi)
    print(f"CNT_chiral forces: n_scf {res.n_scf} err {res.err:.2e}; GPU - oracle {np.max(np.abs(F - Fo)):.2e}, "
          f"GPU - printed {np.max(np.abs(F - printed)):.2e} Ha/bohr")
    assert np.max(np.abs(F - Fo)) < 1e-9, (F, Fo)
    assert np.max(np.abs(F - printed)) < 3e-6, (F, printed)
