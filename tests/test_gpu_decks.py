"""The GPU SCF on three of the reference's own Cyclix decks against the free energy the reference
printed for them (tests/Cyclix/CNT_chiral/C.out: helical, twist 0.1636 rad/bohr, Gamma point;
tests/Cyclix/CNT_ABINITmatch/C.out: cyclic, 9 Bloch points; both LDA_PW with Fermi-Dirac
smearing and psp8 projectors of two projectors per l <= 1, passed to the library as 4-column
atoms; GGA_wrong_SG15/C.out: GGA_PBE, cyclic, 8 Bloch points, Gaussian smearing).  The deck set-up comes from tests/golden/deck_<name>.npz (written by
tests/golden/make_deck_fixtures.py from the reference's deck files with this library's psp8
loader), so the test needs no reference tree.

Tolerance: free energy per atom within 1e-6 Ha/atom of the printed value (the oracle SCF from the
same set-up is within 9.0e-8 and 2.7e-9 of it), in FP64 and in mixed precision.  The SCF runs to
the deck's tolerance (at most 1e-6), except in mixed precision on CNT_ABINITmatch: its filter of
degree 100 in complex64 leaves an SCF error floor near 1e-5 (the error fluctuates between 1e-5
and 2e-4 from step 20 on), so that run stops at 1e-4; its free energy after the FP64 refinement
is still within 1e-8 Ha/atom of the printed value.
"""
import numpy as np
import pytest

from golden.make_deck_fixtures import load

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("name", ["CNT_chiral", "CNT_ABINITmatch"])
def test_deck_free_energy_matches_printed(name, prec):
    from cyclix_msparc_gb300.msparc import CyclixGPU
    from cyclix_msparc_gb300.workloads import initial_psi
    S, scf_tol, poisson_tol, e_ref = load(name)
    blocks = [(S.kptgrid[k].copy(), 0, S.Nev) for k in range(S.tnkpt)]
    g = CyclixGPU(S, blocks, prec)
    try:
        for b in range(len(blocks)):
            g.set_psi(b, initial_psi(S.N, S.Nev, 700 + b))
        tol = 1e-4 if (prec == "mixed" and S.npl >= 100) else min(scf_tol, 1e-6)
        res, EV, rho, V, hist = g.scf(S, scf_tol=tol, poisson_tol=poisson_tol, max_scf=60)
    finally:
        g.close()
    assert res.converged == 1
    e = res.Etotal / S.n_atm
    assert abs(e - e_ref) < 1e-6, (name, prec, e, e_ref)
    # the electron count is conserved: to rounding in FP64; in mixed precision the density is
    # summed from complex64 states, whose W-norms carry FP32 rounding (measured 1.0e-8 relative)
    ctol = 1e-8 if prec == "fp64" else 1e-6
    assert abs(float(np.sum(rho * S.W)) + S.NegCharge) < ctol * abs(S.NegCharge)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gga_deck_matches_oracle_and_printed(prec):
    """GGA_PBE on the GPU for a reference deck: GGA_wrong_SG15/C.inpt (cyclic 121 x 40 x 23, 8 Bloch
    points, SG15 psp8 projectors, Gaussian smearing), converged tightly (SCF error 1e-8, Poisson
    relative residual 1e-10; the mixed run finishes in FP64) so that the fixed point does not depend
    on where either Poisson solver stops: at the deck's own Poisson tolerance of 1e-6 the Jacobi- and
    ILU-preconditioned solves leave different errors in phi, which moved the free energy by up to
    9e-7 Ha/atom.  Against the oracle SCF of the same set-up at the same tolerances
    (tests/golden/deck_GGA_wrong_SG15_oracle.json) within 1e-7 Ha/atom (measured 1.6e-11 in FP64 and
    3.8e-10 in mixed precision), and against the free energy the reference printed within 3e-6
    Ha/atom (measured 1.68e-6, as the oracle): the printed run stopped at its TOL_SCF of 1e-4."""
    import json
    from pathlib import Path
    from cyclix_msparc_gb300.msparc import CyclixGPU
    from cyclix_msparc_gb300.workloads import initial_psi
    S, scf_tol, poisson_tol, e_ref = load("GGA_wrong_SG15")
    ref = json.loads((Path(__file__).resolve().parent / "golden" / "deck_GGA_wrong_SG15_oracle.json").read_text())
    e_oracle = ref["free_energy_per_atom"]
    assert S.extra["xc"] == "GGA_PBE"
    blocks = [(S.kptgrid[k].copy(), 0, S.Nev) for k in range(S.tnkpt)]
    g = CyclixGPU(S, blocks, prec)
    try:
        for b in range(len(blocks)):
            g.set_psi(b, initial_psi(S.N, S.Nev, 700 + b))
        if prec == "fp64":
            res, EV, rho, V, hist = g.scf(S, scf_tol=ref["scf_tol"], poisson_tol=ref["poisson_tol"], max_scf=80)
        else:
            res, EV, rho, V, hist = g.scf(S, scf_tol=1e-6, poisson_tol=ref["poisson_tol"], max_scf=80,
                                          fp64_tol=ref["scf_tol"])
    finally:
        g.close()
    e = res.Etotal / S.n_atm
    print(f"GGA_wrong_SG15 {prec}: n_scf {res.n_scf} err {res.err:.3e} E {e:.12f} - oracle {e - e_oracle:.3e} "
          f"- printed {e - e_ref:.3e}")
    assert res.converged == 1, hist[-5:]
    assert abs(e - e_oracle) < 1e-7, (prec, e, e_oracle)
    assert abs(e - e_ref) < 3e-6, (prec, e, e_ref)
